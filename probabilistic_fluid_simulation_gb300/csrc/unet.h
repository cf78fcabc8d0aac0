// The warm-start network: a 4-level U-Net mapping the normalised divergence
// b / rms(b) to the normalised pressure p / rms(b) (the pressure equation is
// linear in b). Private to the library; the C ABI is in include/pfs.h.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace pfs {
namespace unet {

// An NHWC bf16 tensor view: element (pixel, c) at p[pixel * stride + off + c].
struct Tensor {
    __nv_bfloat16 *p;
    int stride;
    int off;
};

// kernel launchers (unet_kernels.cu); epi: 0 = bias + ReLU -> bf16, 1 = fp32 store, 2 = fp32 add
cudaError_t conv3x3(Tensor in, int cin, const __nv_bfloat16 *w, const float *bias, Tensor out, int cout, float *outf,
                    int fs, int fo, int epi, int n, int H, int W, cudaStream_t st);
cudaError_t wgrad3x3(Tensor x, int cin, int cinp, const __nv_bfloat16 *dy, int cout, float *dw, float *db, int n, int H,
                     int W, cudaStream_t st);
cudaError_t pool2(Tensor in, Tensor out, int c, int n, int H, int W, cudaStream_t st);
cudaError_t pool2_bwd(const float *dout, int ds, int doff, float *din, int is, int ioff, int c, int n, int H, int W,
                      cudaStream_t st);
cudaError_t up2(Tensor in, Tensor out, int c, int n, int H, int W, cudaStream_t st);
cudaError_t up2_bwd(const float *dout, int ds, int doff, float *din, int is, int ioff, int c, int n, int H, int W,
                    cudaStream_t st);
cudaError_t relu_bwd(const float *dout, int ds, int doff, Tensor y, __nv_bfloat16 *dpre, int c, size_t npix,
                     cudaStream_t st);
cudaError_t head(Tensor x, const float *w, const float *b, float *out, int c, size_t npix, cudaStream_t st);
cudaError_t head_bwd(Tensor x, const float *w, const float *dout, float *dx, float *dw, float *db, int c, size_t npix,
                     cudaStream_t st);
cudaError_t mse(const float *pred, const float *target, float *dpred, size_t n, float *loss, cudaStream_t st);
cudaError_t adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps,
                 float c1, float c2, cudaStream_t st);
cudaError_t weights_to_bf16(const float *wf, __nv_bfloat16 *wb, __nv_bfloat16 *wt, int cout, int cin, int cinp,
                            int coutp, cudaStream_t st);
cudaError_t to_input(const float *b, int ld, const float *scale, __nv_bfloat16 *xin, int H, int W, int img,
                     cudaStream_t st);
cudaError_t from_output(const float *y, const float *scale, float *p, int ld, int H, int W, cudaStream_t st);
cudaError_t rms(const float *b, int ld, int H, int W, float *out, cudaStream_t st);
// k x k block means into a dense (H/k) x (W/k) plane; periodic bilinear
// interpolation of such a plane back to (H, W) times `scale`
cudaError_t restrict_mean(const float *b, int ld, int H, int W, int k, float *bc, cudaStream_t st);
cudaError_t prolong(const float *pc, int k, float scale, float *p, int ld, int H, int W, cudaStream_t st);

struct Net;
int create(Net **out, int max_pixels);
void destroy(Net *n);
size_t num_params(const Net *n);
int set_params(Net *n, const float *host);
int get_params(const Net *n, float *host);
int get_grads(const Net *n, float *host);
// loss and gradients for a batch of pre-normalised (b, p) pairs (dense fp32, device)
int forward_backward(Net *n, const float *b, const float *p, int nimg, int H, int W, float *loss, cudaStream_t st);
int adam_step(Net *n, float lr, cudaStream_t st);
// prediction for one plane: p_out = rms(b) * net(b / rms(b)); planes with row pitch ld
int predict(Net *n, const float *b, int ldb, float *p_out, int ldp, int H, int W, cudaStream_t st);
// the same on a grid coarsened k times: b averaged over k x k blocks, the
// network run at (H/k, W/k), its pressure interpolated back and scaled by k^2
// (the 5-point operator in cell units scales with the cell size squared);
// k = 1 is predict()
int predict_coarse(Net *n, const float *b, int ldb, float *p_out, int ldp, int H, int W, int k, cudaStream_t st);

}  // namespace unet
}  // namespace pfs
