// Host side of the warm-start U-Net: layer table, buffers, forward pass,
// backward pass and Adam. Four levels, 3x3 convolutions with circular padding
// (the domain is periodic), 16/32/64/64 channels, 2x2 average pooling,
// nearest upsampling, skip connections by concatenation, a 1x1 output head.
// Weights are bf16 copies of fp32 master weights; activations bf16; all
// accumulation fp32.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "kernels.h"
#include "pfs.h"
#include "unet.h"

namespace pfs {
namespace unet {

namespace {

struct ConvDef {
    int cin, cout, level;
};
// enc1a enc1b enc2a enc2b enc3a enc3b bota botb dec3a dec3b dec2a dec2b dec1a dec1b
const ConvDef kConv[14] = {{1, 16, 0},  {16, 16, 0}, {16, 32, 1}, {32, 32, 1}, {32, 64, 2},
                           {64, 64, 2}, {64, 64, 3}, {64, 64, 3}, {128, 64, 2}, {64, 64, 2},
                           {96, 32, 1}, {32, 32, 1}, {48, 16, 0}, {16, 16, 0}};
constexpr int kHeadC = 16;

inline int cinp_of(int cin) { return cin < 16 ? 16 : cin; }

#define UCK(x)                                                                       \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess) {                                                     \
            cudaGetLastError();                                                      \
            return record_error(PFS_ERR_CUDA, cudaGetErrorString(e_));               \
        }                                                                            \
    } while (0)

}  // namespace

struct Net {
    size_t max_pix = 0;
    // parameters: fp32 master, grads, Adam moments; offsets per layer
    size_t np = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    size_t w_off[14], b_off[14], hw_off, hb_off;
    __nv_bfloat16 *wb[14], *wt[14];
    __nv_bfloat16 *wmem = nullptr;
    long long t = 0;  // Adam step
    // activations (bf16); per level sizes scale by 1/4
    __nv_bfloat16 *amem = nullptr;
    __nv_bfloat16 *x0, *a0, *cat1, *t0, *d1;  // level 0
    __nv_bfloat16 *x1, *a1, *cat2, *t1, *d2;  // level 1
    __nv_bfloat16 *x2, *a2, *cat3, *t2, *d3;  // level 2
    __nv_bfloat16 *x3, *a3, *e4;              // level 3
    __nv_bfloat16 *dpre = nullptr;
    float *fmem = nullptr;
    float *out, *dout, *target_tmp;
    float *dD1, *dT0, *dCat1, *dA0;
    float *dD2, *dT1, *dCat2, *dA1, *dX1;
    float *dD3, *dT2, *dCat3, *dA2, *dX2;
    float *dE4, *dA3, *dX3;
    float *scal = nullptr;  // [0] loss, [1] rms, [2] 1.0
    float *coarse = nullptr;  // coarse-grid prediction: restricted b, then the coarse pressure (2 x max_pix)
};

int create(Net **out, int max_pixels)
{
    *out = nullptr;
    Net *n = new (std::nothrow) Net();
    if (!n) return record_error(PFS_ERR_CUDA, "out of host memory");
    n->max_pix = (size_t)max_pixels;
    // parameter layout
    size_t off = 0, woff = 0;
    for (int k = 0; k < 14; ++k) {
        const int cp = cinp_of(kConv[k].cin);
        n->w_off[k] = off;
        off += (size_t)kConv[k].cout * 9 * cp;
        n->b_off[k] = off;
        off += kConv[k].cout;
        woff += (size_t)kConv[k].cout * 9 * cp + (size_t)kConv[k].cin * 9 * kConv[k].cout;
    }
    n->hw_off = off;
    off += kHeadC;
    n->hb_off = off;
    off += 1;
    n->np = off;
    auto fail = [&](const char *msg) {
        destroy(n);
        return record_error(PFS_ERR_CUDA, msg);
    };
    if (cudaMalloc(&n->params, 4 * n->np * sizeof(float)) != cudaSuccess) return fail("unet parameter allocation");
    cudaMemset(n->params, 0, 4 * n->np * sizeof(float));
    n->grads = n->params + n->np;
    n->m = n->grads + n->np;
    n->v = n->m + n->np;
    if (cudaMalloc(&n->wmem, woff * sizeof(__nv_bfloat16)) != cudaSuccess) return fail("unet weight allocation");
    cudaMemset(n->wmem, 0, woff * sizeof(__nv_bfloat16));
    __nv_bfloat16 *q = n->wmem;
    for (int k = 0; k < 14; ++k) {
        const int cp = cinp_of(kConv[k].cin);
        n->wb[k] = q;
        q += (size_t)kConv[k].cout * 9 * cp;
        n->wt[k] = q;
        q += (size_t)kConv[k].cin * 9 * kConv[k].cout;
    }
    // activations: channels per level (bf16)
    const size_t P0 = n->max_pix, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
    const size_t abf = P0 * (1 + 16 + 48 + 16 + 16) + P1 * (16 + 32 + 96 + 32 + 32) + P2 * (32 + 64 + 128 + 64 + 64) +
                       P3 * (64 + 64 + 64) + P0 * 16 /* dpre */;
    if (cudaMalloc(&n->amem, abf * sizeof(__nv_bfloat16)) != cudaSuccess) return fail("unet activation allocation");
    cudaMemset(n->amem, 0, abf * sizeof(__nv_bfloat16));
    __nv_bfloat16 *a = n->amem;
    auto takeb = [&](size_t cnt) {
        __nv_bfloat16 *r = a;
        a += cnt;
        return r;
    };
    n->x0 = takeb(P0);
    n->a0 = takeb(P0 * 16);
    n->cat1 = takeb(P0 * 48);
    n->t0 = takeb(P0 * 16);
    n->d1 = takeb(P0 * 16);
    n->x1 = takeb(P1 * 16);
    n->a1 = takeb(P1 * 32);
    n->cat2 = takeb(P1 * 96);
    n->t1 = takeb(P1 * 32);
    n->d2 = takeb(P1 * 32);
    n->x2 = takeb(P2 * 32);
    n->a2 = takeb(P2 * 64);
    n->cat3 = takeb(P2 * 128);
    n->t2 = takeb(P2 * 64);
    n->d3 = takeb(P2 * 64);
    n->x3 = takeb(P3 * 64);
    n->a3 = takeb(P3 * 64);
    n->e4 = takeb(P3 * 64);
    n->dpre = takeb(P0 * 16);
    const size_t af = P0 * (3 + 16 + 16 + 48 + 16) + P1 * (32 + 32 + 96 + 32 + 16) + P2 * (64 + 64 + 128 + 64 + 32) +
                      P3 * (64 + 64 + 64) + 8;
    if (cudaMalloc(&n->fmem, af * sizeof(float)) != cudaSuccess) return fail("unet gradient allocation");
    cudaMemset(n->fmem, 0, af * sizeof(float));
    float *f = n->fmem;
    auto takef = [&](size_t cnt) {
        float *r = f;
        f += cnt;
        return r;
    };
    n->out = takef(P0);
    n->dout = takef(P0);
    n->target_tmp = takef(P0);
    n->dD1 = takef(P0 * 16);
    n->dT0 = takef(P0 * 16);
    n->dCat1 = takef(P0 * 48);
    n->dA0 = takef(P0 * 16);
    n->dD2 = takef(P1 * 32);
    n->dT1 = takef(P1 * 32);
    n->dCat2 = takef(P1 * 96);
    n->dA1 = takef(P1 * 32);
    n->dX1 = takef(P1 * 16);
    n->dD3 = takef(P2 * 64);
    n->dT2 = takef(P2 * 64);
    n->dCat3 = takef(P2 * 128);
    n->dA2 = takef(P2 * 64);
    n->dX2 = takef(P2 * 32);
    n->dE4 = takef(P3 * 64);
    n->dA3 = takef(P3 * 64);
    n->dX3 = takef(P3 * 64);
    n->scal = takef(8);
    const float one = 1.0f;
    cudaMemcpy(n->scal + 2, &one, sizeof one, cudaMemcpyHostToDevice);
    *out = n;
    return PFS_OK;
}

void destroy(Net *n)
{
    if (!n) return;
    cudaFree(n->params);
    cudaFree(n->wmem);
    cudaFree(n->amem);
    cudaFree(n->fmem);
    if (n->coarse) cudaFree(n->coarse);
    delete n;
}

size_t num_params(const Net *n) { return n->np; }

static int refresh_bf16(Net *n, cudaStream_t st)
{
    for (int k = 0; k < 14; ++k)
        UCK(weights_to_bf16(n->params + n->w_off[k], n->wb[k], k == 0 ? nullptr : n->wt[k], kConv[k].cout,
                            kConv[k].cin, cinp_of(kConv[k].cin), kConv[k].cout, st));
    return PFS_OK;
}

int set_params(Net *n, const float *host)
{
    UCK(cudaMemcpy(n->params, host, n->np * sizeof(float), cudaMemcpyHostToDevice));
    UCK(cudaMemset(n->m, 0, 2 * n->np * sizeof(float)));
    n->t = 0;
    int rc = refresh_bf16(n, 0);
    if (rc == PFS_OK) UCK(cudaDeviceSynchronize());
    return rc;
}

int get_params(const Net *n, float *host)
{
    UCK(cudaMemcpy(host, n->params, n->np * sizeof(float), cudaMemcpyDeviceToHost));
    return PFS_OK;
}

int get_grads(const Net *n, float *host)
{
    UCK(cudaMemcpy(host, n->grads, n->np * sizeof(float), cudaMemcpyDeviceToHost));
    return PFS_OK;
}

namespace {

Tensor T(__nv_bfloat16 *p, int stride, int off = 0) { return Tensor{p, stride, off}; }

int conv_fwd(Net *n, int k, Tensor in, Tensor out, int nimg, int H, int W, cudaStream_t st)
{
    UCK(conv3x3(in, kConv[k].cin, n->wb[k], n->params + n->b_off[k], out, kConv[k].cout, nullptr, 0, 0, 0, nimg, H, W,
                st));
    return PFS_OK;
}

// forward pass from x0 (bf16 input, nimg images of H x W) to n->out (fp32)
int forward(Net *n, int nimg, int H, int W, cudaStream_t st)
{
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
    int rc;
#define F(x) \
    if ((rc = (x)) != PFS_OK) return rc
    F(conv_fwd(n, 0, T(n->x0, 1), T(n->a0, 16), nimg, H, W, st));
    F(conv_fwd(n, 1, T(n->a0, 16), T(n->cat1, 48, 32), nimg, H, W, st));
    UCK(pool2(T(n->cat1, 48, 32), T(n->x1, 16), 16, nimg, H, W, st));
    F(conv_fwd(n, 2, T(n->x1, 16), T(n->a1, 32), nimg, H1, W1, st));
    F(conv_fwd(n, 3, T(n->a1, 32), T(n->cat2, 96, 64), nimg, H1, W1, st));
    UCK(pool2(T(n->cat2, 96, 64), T(n->x2, 32), 32, nimg, H1, W1, st));
    F(conv_fwd(n, 4, T(n->x2, 32), T(n->a2, 64), nimg, H2, W2, st));
    F(conv_fwd(n, 5, T(n->a2, 64), T(n->cat3, 128, 64), nimg, H2, W2, st));
    UCK(pool2(T(n->cat3, 128, 64), T(n->x3, 64), 64, nimg, H2, W2, st));
    F(conv_fwd(n, 6, T(n->x3, 64), T(n->a3, 64), nimg, H3, W3, st));
    F(conv_fwd(n, 7, T(n->a3, 64), T(n->e4, 64), nimg, H3, W3, st));
    UCK(up2(T(n->e4, 64), T(n->cat3, 128, 0), 64, nimg, H2, W2, st));
    F(conv_fwd(n, 8, T(n->cat3, 128), T(n->t2, 64), nimg, H2, W2, st));
    F(conv_fwd(n, 9, T(n->t2, 64), T(n->d3, 64), nimg, H2, W2, st));
    UCK(up2(T(n->d3, 64), T(n->cat2, 96, 0), 64, nimg, H1, W1, st));
    F(conv_fwd(n, 10, T(n->cat2, 96), T(n->t1, 32), nimg, H1, W1, st));
    F(conv_fwd(n, 11, T(n->t1, 32), T(n->d2, 32), nimg, H1, W1, st));
    UCK(up2(T(n->d2, 32), T(n->cat1, 48, 0), 32, nimg, H, W, st));
    F(conv_fwd(n, 12, T(n->cat1, 48), T(n->t0, 16), nimg, H, W, st));
    F(conv_fwd(n, 13, T(n->t0, 16), T(n->d1, 16), nimg, H, W, st));
    UCK(head(T(n->d1, 16), n->params + n->hw_off, n->params + n->hb_off, n->out, kHeadC, (size_t)nimg * H * W, st));
#undef F
    return PFS_OK;
}

// backward of conv k: dy (fp32, stride ds / offset doff) is the gradient of its
// ReLU output y; x its input. Weight/bias grads accumulate; the input gradient
// (if dx) is stored fp32 with stride xs.
int conv_bwd(Net *n, int k, const float *dy, int ds, int doff, Tensor y, Tensor x, float *dx, int xs, int nimg, int H,
             int W, cudaStream_t st)
{
    const int cin = kConv[k].cin, cout = kConv[k].cout;
    const size_t npix = (size_t)nimg * H * W;
    UCK(relu_bwd(dy, ds, doff, y, n->dpre, cout, npix, st));
    UCK(wgrad3x3(x, cin, cinp_of(cin), n->dpre, cout, n->grads + n->w_off[k], n->grads + n->b_off[k], nimg, H, W, st));
    if (dx) UCK(conv3x3(T(n->dpre, cout), cout, n->wt[k], nullptr, T(nullptr, 0), cin, dx, xs, 0, 1, nimg, H, W, st));
    return PFS_OK;
}

}  // namespace

int forward_backward(Net *n, const float *b, const float *p, int nimg, int H, int W, float *loss, cudaStream_t st)
{
    if (H % 128 || W % 128 || (size_t)nimg * H * W > n->max_pix)
        return record_error(PFS_ERR_INVALID_ARGUMENT, "unet batch: H, W multiples of 128 within the allocated pixels");
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
    const size_t P0 = (size_t)nimg * H * W;
    for (int i = 0; i < nimg; ++i) UCK(to_input(b + (size_t)i * H * W, W, n->scal + 2, n->x0, H, W, i, st));
    int rc = forward(n, nimg, H, W, st);
    if (rc != PFS_OK) return rc;
    UCK(cudaMemsetAsync(n->grads, 0, n->np * sizeof(float), st));
    UCK(cudaMemsetAsync(n->scal, 0, sizeof(float), st));
    UCK(mse(n->out, p, n->dout, P0, n->scal, st));
    UCK(head_bwd(T(n->d1, 16), n->params + n->hw_off, n->dout, n->dD1, n->grads + n->hw_off, n->grads + n->hb_off,
                 kHeadC, P0, st));
#define F(x) \
    if ((rc = (x)) != PFS_OK) return rc
    F(conv_bwd(n, 13, n->dD1, 16, 0, T(n->d1, 16), T(n->t0, 16), n->dT0, 16, nimg, H, W, st));
    F(conv_bwd(n, 12, n->dT0, 16, 0, T(n->t0, 16), T(n->cat1, 48), n->dCat1, 48, nimg, H, W, st));
    UCK(up2_bwd(n->dCat1, 48, 0, n->dD2, 32, 0, 32, nimg, H1, W1, st));
    F(conv_bwd(n, 11, n->dD2, 32, 0, T(n->d2, 32), T(n->t1, 32), n->dT1, 32, nimg, H1, W1, st));
    F(conv_bwd(n, 10, n->dT1, 32, 0, T(n->t1, 32), T(n->cat2, 96), n->dCat2, 96, nimg, H1, W1, st));
    UCK(up2_bwd(n->dCat2, 96, 0, n->dD3, 64, 0, 64, nimg, H2, W2, st));
    F(conv_bwd(n, 9, n->dD3, 64, 0, T(n->d3, 64), T(n->t2, 64), n->dT2, 64, nimg, H2, W2, st));
    F(conv_bwd(n, 8, n->dT2, 64, 0, T(n->t2, 64), T(n->cat3, 128), n->dCat3, 128, nimg, H2, W2, st));
    UCK(up2_bwd(n->dCat3, 128, 0, n->dE4, 64, 0, 64, nimg, H3, W3, st));
    F(conv_bwd(n, 7, n->dE4, 64, 0, T(n->e4, 64), T(n->a3, 64), n->dA3, 64, nimg, H3, W3, st));
    F(conv_bwd(n, 6, n->dA3, 64, 0, T(n->a3, 64), T(n->x3, 64), n->dX3, 64, nimg, H3, W3, st));
    UCK(pool2_bwd(n->dX3, 64, 0, n->dCat3, 128, 64, 64, nimg, H2, W2, st));
    F(conv_bwd(n, 5, n->dCat3, 128, 64, T(n->cat3, 128, 64), T(n->a2, 64), n->dA2, 64, nimg, H2, W2, st));
    F(conv_bwd(n, 4, n->dA2, 64, 0, T(n->a2, 64), T(n->x2, 32), n->dX2, 32, nimg, H2, W2, st));
    UCK(pool2_bwd(n->dX2, 32, 0, n->dCat2, 96, 64, 32, nimg, H1, W1, st));
    F(conv_bwd(n, 3, n->dCat2, 96, 64, T(n->cat2, 96, 64), T(n->a1, 32), n->dA1, 32, nimg, H1, W1, st));
    F(conv_bwd(n, 2, n->dA1, 32, 0, T(n->a1, 32), T(n->x1, 16), n->dX1, 16, nimg, H1, W1, st));
    UCK(pool2_bwd(n->dX1, 16, 0, n->dCat1, 48, 32, 16, nimg, H, W, st));
    F(conv_bwd(n, 1, n->dCat1, 48, 32, T(n->cat1, 48, 32), T(n->a0, 16), n->dA0, 16, nimg, H, W, st));
    F(conv_bwd(n, 0, n->dA0, 16, 0, T(n->a0, 16), T(n->x0, 1), nullptr, 0, nimg, H, W, st));
#undef F
    if (loss) {
        UCK(cudaMemcpyAsync(loss, n->scal, sizeof(float), cudaMemcpyDeviceToHost, st));
        UCK(cudaStreamSynchronize(st));
    }
    return PFS_OK;
}

int adam_step(Net *n, float lr, cudaStream_t st)
{
    n->t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)n->t), c2 = 1.0f - std::pow(b2, (float)n->t);
    UCK(adam(n->params, n->grads, n->m, n->v, n->np, lr, b1, b2, 1e-8f, c1, c2, st));
    return refresh_bf16(n, st);
}

int predict(Net *n, const float *b, int ldb, float *p_out, int ldp, int H, int W, cudaStream_t st)
{
    if (H % 128 || W % 128 || (size_t)H * W > n->max_pix)
        return record_error(PFS_ERR_UNSUPPORTED, "warm start needs H, W multiples of 128 within the network's size");
    UCK(rms(b, ldb, H, W, n->scal + 1, st));
    UCK(to_input(b, ldb, n->scal + 1, n->x0, H, W, 0, st));
    const int rc = forward(n, 1, H, W, st);
    if (rc != PFS_OK) return rc;
    UCK(from_output(n->out, n->scal + 1, p_out, ldp, H, W, st));
    return PFS_OK;
}

int predict_coarse(Net *n, const float *b, int ldb, float *p_out, int ldp, int H, int W, int k, cudaStream_t st)
{
    if (k == 1) return predict(n, b, ldb, p_out, ldp, H, W, st);
    if (k < 1 || H % k || W % k)
        return record_error(PFS_ERR_INVALID_ARGUMENT, "the coarsening factor must divide the grid sides");
    const int Hc = H / k, Wc = W / k;
    if (Hc % 128 || Wc % 128 || (size_t)Hc * Wc > n->max_pix)
        return record_error(PFS_ERR_UNSUPPORTED,
                            "warm start needs coarse sides that are multiples of 128 within the network's size");
    if (!n->coarse) UCK(cudaMalloc(&n->coarse, 2 * n->max_pix * sizeof(float)));
    float *bc = n->coarse, *pc = n->coarse + n->max_pix;
    UCK(restrict_mean(b, ldb, H, W, k, bc, st));
    const int rc = predict(n, bc, Wc, pc, Wc, Hc, Wc, st);
    if (rc != PFS_OK) return rc;
    UCK(prolong(pc, k, (float)(k * k), p_out, ldp, H, W, st));
    return PFS_OK;
}

}  // namespace unet
}  // namespace pfs
