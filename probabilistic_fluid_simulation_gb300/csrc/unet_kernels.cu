// Kernels of the warm-start network (a 4-level U-Net, unet.cu): 3x3
// convolutions with circular padding as implicit GEMMs on the tensor cores
// (mma.sync m16n8k16, bf16 operands, fp32 accumulation), their weight
// gradients, 2x2 average pooling, nearest upsampling, the 1x1 output head,
// ReLU backward, the loss and Adam.
//
// Activations are NHWC bf16; a tensor is (ptr, channel stride, channel
// offset) so concatenations of the decoder are channel ranges of one buffer.
// Spatial dims are multiples of 16 at every level.
#include <cuda_bf16.h>

#include "kernels.h"
#include "unet.h"

namespace pfs {
namespace unet {
namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ unsigned ld32(const bf16 *p) { return *reinterpret_cast<const unsigned *>(p); }

__device__ __forceinline__ void mma16816(float (&c)[4], const unsigned (&a)[4], const unsigned (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ int wrapi(int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

// 3x3 convolution, circular padding. One warp computes 16 consecutive pixels
// of a row x all COUT output channels: A = im2col rows (pixels) x K
// (tap-major, CINP channels per tap), B = weights [COUT][9][CINP].
// Epilogue: EPI_RELU_BF16 (bias, ReLU, bf16 store) or EPI_F32 (fp32 store or
// add, no bias: input gradients).
enum { EPI_RELU_BF16 = 0, EPI_F32_STORE = 1, EPI_F32_ADD = 2 };

template <int CIN, int CINP, int COUT, int EPI>
__global__ void __launch_bounds__(128) k_conv3x3(Tensor in, const bf16 *__restrict__ w, const float *__restrict__ bias,
                                                Tensor out, float *__restrict__ outf, int outf_stride,
                                                int outf_off, int n_img, int H, int W)
{
    constexpr int NT = COUT / 8;
    const int lane = threadIdx.x & 31;
    const int seg = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int segs_per_row = W / 16;
    const int nseg = n_img * H * segs_per_row;
    if (seg >= nseg) return;
    const int img = seg / (H * segs_per_row);
    const int rem = seg - img * H * segs_per_row;
    const int y = rem / segs_per_row, x0 = (rem % segs_per_row) * 16;
    const int r0 = lane >> 2, kq = (lane & 3) * 2;

    float acc[NT][4];
#pragma unroll
    for (int t = 0; t < NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;

    const bf16 *base = in.p + (size_t)img * H * W * in.stride + in.off;
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap) {
        const int yy = wrapi(y + tap / 3 - 1, H);
        const int xa = wrapi(x0 + r0 + tap % 3 - 1, W), xb = wrapi(x0 + r0 + 8 + tap % 3 - 1, W);
        const bf16 *pa = base + ((size_t)yy * W + xa) * in.stride;
        const bf16 *pb = base + ((size_t)yy * W + xb) * in.stride;
#pragma unroll
        for (int c0 = 0; c0 < CINP; c0 += 16) {
            unsigned a[4];
            if (CIN == CINP) {
                a[0] = ld32(pa + c0 + kq);
                a[1] = ld32(pb + c0 + kq);
                a[2] = ld32(pa + c0 + kq + 8);
                a[3] = ld32(pb + c0 + kq + 8);
            } else {  // CIN == 1: only channel 0 is real
                const unsigned short va = (kq == 0) ? *reinterpret_cast<const unsigned short *>(pa) : 0;
                const unsigned short vb = (kq == 0) ? *reinterpret_cast<const unsigned short *>(pb) : 0;
                a[0] = va;
                a[1] = vb;
                a[2] = 0u;
                a[3] = 0u;
            }
            const bf16 *wk = w + (size_t)tap * CINP + c0 + kq;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const bf16 *wt = wk + (size_t)(t * 8 + r0) * 9 * CINP;
                const unsigned b[2] = {ld32(wt), ld32(wt + 8)};
                mma16816(acc[t], a, b);
            }
        }
    }
    // epilogue: acc[t][0..1] -> pixel x0 + r0, channels t*8 + kq + {0,1}; [2..3] -> pixel x0 + r0 + 8
    const size_t pix_a = ((size_t)img * H + y) * W + x0 + r0, pix_b = pix_a + 8;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int co = t * 8 + kq;
        if (EPI == EPI_RELU_BF16) {
            const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
            const __nv_bfloat162 va = __floats2bfloat162_rn(fmaxf(acc[t][0] + b0, 0.f), fmaxf(acc[t][1] + b1, 0.f));
            const __nv_bfloat162 vb = __floats2bfloat162_rn(fmaxf(acc[t][2] + b0, 0.f), fmaxf(acc[t][3] + b1, 0.f));
            *reinterpret_cast<__nv_bfloat162 *>(out.p + pix_a * out.stride + out.off + co) = va;
            *reinterpret_cast<__nv_bfloat162 *>(out.p + pix_b * out.stride + out.off + co) = vb;
        } else {
            float *fa = outf + pix_a * outf_stride + outf_off + co;
            float *fb = outf + pix_b * outf_stride + outf_off + co;
            if (EPI == EPI_F32_ADD) {
                fa[0] += acc[t][0];
                fa[1] += acc[t][1];
                fb[0] += acc[t][2];
                fb[1] += acc[t][3];
            } else {
                fa[0] = acc[t][0];
                fa[1] = acc[t][1];
                fb[0] = acc[t][2];
                fb[1] = acc[t][3];
            }
        }
    }
}

// Weight gradient of a 3x3 conv on the tensor cores. Per tap t,
// dW_t[co][ci] += sum_p dY[p][co] X[shift_t(p)][ci]: a GEMM with M = cout,
// N = cin and K = pixels. A block owns a 32 (co) x 32 (ci) tile for all nine
// taps and a run of row segments of up to 128 pixels; per segment dY
// (pixels x 32 co) and the three input rows the taps read (pixels + 2 x 32
// ci, circular halo) are staged in shared memory as [pixel][channel] tiles,
// from which ldmatrix.trans yields both operands (the pixel dimension is
// strided in memory for both). Four warps, each a 16 x 16 (co, ci) quarter
// of the tile, 9 taps x 2 n-tiles of fp32 accumulators; the block adds its
// partial sums to dW with atomics. Rows of 40 bf16 (80 bytes) keep the
// ldmatrix row reads free of bank conflicts.
constexpr int kWgSeg = 128;  // pixels per row segment (at most)
constexpr int kWgLd = 40;    // shared-memory row pitch, bf16

__device__ __forceinline__ void ldsm_x4_trans(unsigned (&r)[4], const bf16 *p)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// Eight channels of one pixel (channels c..c+7 below `lim` are real, the rest zero).
__device__ __forceinline__ uint4 load8(const bf16 *p, int c, int lim, bool vec)
{
    if (vec && c + 8 <= lim) return *reinterpret_cast<const uint4 *>(p + c);
    __align__(16) bf16 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = (c + k < lim) ? p[c + k] : __float2bfloat16_rn(0.f);
    return *reinterpret_cast<const uint4 *>(v);
}

__global__ void __launch_bounds__(128) k_wgrad_tc(Tensor x, const bf16 *__restrict__ dy, int cout, int cin, int cinp,
                                                 float *__restrict__ dw, float *__restrict__ db, int n_img, int H,
                                                 int W, int seg_len, int segs_per_block)
{
    __shared__ __align__(16) bf16 sD[kWgSeg][kWgLd];
    __shared__ __align__(16) bf16 sX[3][kWgSeg + 2][kWgLd];
    const int co0 = blockIdx.y * 32, ci0 = blockIdx.z * 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wm = (warp & 1) * 16, wn = (warp >> 1) * 16;  // warp's co / ci offsets in the tile
    const bool xvec = (x.stride % 8 == 0) && (x.off % 8 == 0);
    const int segs_per_row = W / seg_len, total = n_img * H * segs_per_row;
    float acc[9][2][4];
#pragma unroll
    for (int t = 0; t < 9; ++t)
#pragma unroll
        for (int n = 0; n < 2; ++n) acc[t][n][0] = acc[t][n][1] = acc[t][n][2] = acc[t][n][3] = 0.f;

    // bias gradient (blocks of the first ci tile): column sums of the staged dY tiles, thread t takes
    // channel co0 + t % 32 and every fourth pixel from t / 32
    const bool bias = db && blockIdx.z == 0;
    float bsum = 0.f;
    const int s_beg = blockIdx.x * segs_per_block, s_end = min(total, s_beg + segs_per_block);
    for (int sg = s_beg; sg < s_end; ++sg) {
        const int img = sg / (H * segs_per_row), rem = sg - img * H * segs_per_row;
        const int y = rem / segs_per_row, x0 = (rem % segs_per_row) * seg_len;
        __syncthreads();  // the previous segment's tiles are consumed
        for (int e = threadIdx.x; e < seg_len * 4; e += blockDim.x) {  // dY: seg_len px x 4 chunks of 8 co
            const int px = e >> 2, part = e & 3;
            const bf16 *src = dy + (((size_t)img * H + y) * W + x0 + px) * cout;
            *reinterpret_cast<uint4 *>(&sD[px][part * 8]) = load8(src, co0 + part * 8, cout, true);
        }
        for (int e = threadIdx.x; e < 3 * (seg_len + 2) * 4; e += blockDim.x) {  // X: 3 rows x (seg_len + 2) px
            const int r = e / ((seg_len + 2) * 4), q = e - r * (seg_len + 2) * 4;
            const int px = q >> 2, part = q & 3;
            const int yy = wrapi(y + r - 1, H), xx = wrapi(x0 + px - 1, W);
            const bf16 *src = x.p + (((size_t)img * H + yy) * W + xx) * x.stride + x.off;
            *reinterpret_cast<uint4 *>(&sX[r][px][part * 8]) = load8(src, ci0 + part * 8, cin, xvec);
        }
        __syncthreads();
        if (bias)
            for (int px = threadIdx.x >> 5; px < seg_len; px += 4) bsum += __bfloat162float(sD[px][threadIdx.x & 31]);
        for (int k0 = 0; k0 < seg_len; k0 += 16) {
            unsigned a[4];
            ldsm_x4_trans(a, &sD[k0 + (lane >> 4) * 8 + (lane & 7)][wm + ((lane >> 3) & 1) * 8]);
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                unsigned b[4];
                ldsm_x4_trans(b, &sX[t / 3][k0 + t % 3 + ((lane >> 3) & 1) * 8 + (lane & 7)][wn + (lane >> 4) * 8]);
                const unsigned b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
                mma16816(acc[t][0], a, b0);
                mma16816(acc[t][1], a, b1);
            }
        }
    }
    // accumulator (m16n8): [0..1] -> co = lane / 4, ci = 2 (lane % 4) + {0, 1}; [2..3] -> co + 8
    const int cr = lane >> 2, cc = (lane & 3) * 2;
#pragma unroll
    for (int t = 0; t < 9; ++t)
#pragma unroll
        for (int n = 0; n < 2; ++n)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int co = co0 + wm + cr + h * 8;
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const int ci = ci0 + wn + n * 8 + cc + j;
                    if (co < cout && ci < cin) atomicAdd(dw + ((size_t)co * 9 + t) * cinp + ci, acc[t][n][h * 2 + j]);
                }
            }
    if (bias && co0 + (threadIdx.x & 31) < cout) atomicAdd(db + co0 + (threadIdx.x & 31), bsum);
}

// 2x2 average pooling (bf16 -> bf16) and its backward (fp32, added).
__global__ void k_pool(Tensor in, Tensor out, int c, int n_img, int H, int W)
{
    const size_t n = (size_t)n_img * (H / 2) * (W / 2) * c;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int ch = e % c;
        const size_t pix = e / c;
        const int x = pix % (W / 2), y = (pix / (W / 2)) % (H / 2), img = pix / ((size_t)(W / 2) * (H / 2));
        auto at = [&](int yy, int xx) {
            return __bfloat162float(in.p[(((size_t)img * H + yy) * W + xx) * in.stride + in.off + ch]);
        };
        const float v = 0.25f * ((at(2 * y, 2 * x) + at(2 * y, 2 * x + 1)) + (at(2 * y + 1, 2 * x) + at(2 * y + 1, 2 * x + 1)));
        out.p[pix * out.stride + out.off + ch] = __float2bfloat16_rn(v);
    }
}

__global__ void k_pool_bwd(const float *__restrict__ dout, int dout_stride, int dout_off, float *__restrict__ din,
                           int din_stride, int din_off, int c, int n_img, int H, int W)
{
    const size_t n = (size_t)n_img * H * W * c;  // input-resolution elements
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int ch = e % c;
        const size_t pix = e / c;
        const int x = pix % W, y = (pix / W) % H, img = pix / ((size_t)W * H);
        const size_t op = ((size_t)img * (H / 2) + y / 2) * (W / 2) + x / 2;
        din[pix * din_stride + din_off + ch] += 0.25f * dout[op * dout_stride + dout_off + ch];
    }
}

// Nearest 2x upsampling (bf16 -> bf16) and its backward (fp32 sum of 4, stored).
__global__ void k_up(Tensor in, Tensor out, int c, int n_img, int H, int W)  // H, W: output dims
{
    const size_t n = (size_t)n_img * H * W * c;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int ch = e % c;
        const size_t pix = e / c;
        const int x = pix % W, y = (pix / W) % H, img = pix / ((size_t)W * H);
        const size_t ip = ((size_t)img * (H / 2) + y / 2) * (W / 2) + x / 2;
        out.p[pix * out.stride + out.off + ch] = in.p[ip * in.stride + in.off + ch];
    }
}

__global__ void k_up_bwd(const float *__restrict__ dout, int dout_stride, int dout_off, float *__restrict__ din,
                         int din_stride, int din_off, int c, int n_img, int H, int W)  // H, W: input (low) dims
{
    const size_t n = (size_t)n_img * H * W * c;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int ch = e % c;
        const size_t pix = e / c;
        const int x = pix % W, y = (pix / W) % H, img = pix / ((size_t)W * H);
        const int W2 = 2 * W, H2 = 2 * H;
        auto at = [&](int yy, int xx) { return dout[(((size_t)img * H2 + yy) * W2 + xx) * dout_stride + dout_off + ch]; };
        din[pix * din_stride + din_off + ch] = (at(2 * y, 2 * x) + at(2 * y, 2 * x + 1)) + (at(2 * y + 1, 2 * x) + at(2 * y + 1, 2 * x + 1));
    }
}

// ReLU backward: dpre (bf16) = dout * (y > 0), y the saved post-activation.
__global__ void k_relu_bwd(const float *__restrict__ dout, int dout_stride, int dout_off, Tensor y,
                           bf16 *__restrict__ dpre, int c, size_t npix)
{
    const size_t n = npix * c;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int ch = e % c;
        const size_t pix = e / c;
        const float g = dout[pix * dout_stride + dout_off + ch];
        dpre[e] = __float2bfloat16_rn(__bfloat162float(y.p[pix * y.stride + y.off + ch]) > 0.f ? g : 0.f);
    }
}

// 1x1 head (16 -> 1): out = sum_c x[c] w[c] + b (fp32).
__global__ void k_head(Tensor x, const float *__restrict__ w, const float *__restrict__ b, float *__restrict__ out,
                       int c, size_t npix)
{
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
        float s = b[0];
        for (int k = 0; k < c; ++k) s = fmaf(__bfloat162float(x.p[p * x.stride + x.off + k]), w[k], s);
        out[p] = s;
    }
}

// Head backward: dx[p][c] = dout[p] w[c] (stored fp32); dw[c] += sum dout x; db += sum dout.
__global__ void __launch_bounds__(256) k_head_bwd(Tensor x, const float *__restrict__ w,
                                                  const float *__restrict__ dout, float *__restrict__ dx,
                                                  float *__restrict__ dw, float *__restrict__ db, int c, size_t npix)
{
    __shared__ float red[17][8];
    float aw[16], ab = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) aw[k] = 0.f;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
        const float g = dout[p];
        ab += g;
        for (int k = 0; k < c; ++k) {
            dx[p * c + k] = g * w[k];
            aw[k] = fmaf(g, __bfloat162float(x.p[p * x.stride + x.off + k]), aw[k]);
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 17; ++k) {
        float v = k < 16 ? aw[k] : ab;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 17) {
        float s = 0.f;
        for (int k = 0; k < 8; ++k) s += red[threadIdx.x][k];
        if (threadIdx.x < c) atomicAdd(dw + threadIdx.x, s);
        else if (threadIdx.x == 16) atomicAdd(db, s);
    }
}

// Mean squared error and its gradient dpred = 2 (pred - target) / n; loss summed into *loss.
__global__ void __launch_bounds__(256) k_mse(const float *__restrict__ pred, const float *__restrict__ target,
                                             float *__restrict__ dpred, size_t n, float *loss)
{
    float s = 0.f;
    const float inv = 2.0f / (float)n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float d = pred[e] - target[e];
        dpred[e] = inv * d;
        s = fmaf(d, d, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (float)n);
}

// Adam on fp32 master parameters.
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        p[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}

// Master fp32 conv weights [cout][9][cinp] -> bf16 for the forward pass, and
// the flipped / transposed bf16 copy [cin][9][coutp] for input gradients.
__global__ void k_weights_to_bf16(const float *__restrict__ wf, bf16 *__restrict__ wb, bf16 *__restrict__ wt, int cout,
                                  int cin, int cinp, int coutp)
{
    const int n = cout * 9 * cinp;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int ci = e % cinp, tap = (e / cinp) % 9, co = e / (9 * cinp);
        const bf16 v = __float2bfloat16_rn(wf[e]);
        wb[e] = v;
        if (wt && ci < cin) wt[((size_t)ci * 9 + (8 - tap)) * coutp + co] = v;
    }
}

// Normalised input: xin (bf16, 1 channel) = b / scale, planes with row pitch ld.
__global__ void k_to_input(const float *__restrict__ b, int ld, const float *__restrict__ scale, bf16 *__restrict__ xin,
                           int H, int W, int img)
{
    const float s = 1.0f / *scale;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < H * W; e += gridDim.x * blockDim.x)
        xin[(size_t)img * H * W + e] = __float2bfloat16_rn(b[(size_t)(e / W) * ld + e % W] * s);
}

__global__ void k_from_output(const float *__restrict__ y, const float *__restrict__ scale, float *__restrict__ p, int ld,
                              int H, int W)
{
    const float s = *scale;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < H * W; e += gridDim.x * blockDim.x)
        p[(size_t)(e / W) * ld + e % W] = y[e] * s;
}

// rms of a plane (ld pitch) into *out (one block).
__global__ void __launch_bounds__(1024) k_rms(const float *__restrict__ b, int ld, int H, int W, float *out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int e = threadIdx.x; e < H * W; e += blockDim.x) {
        const double v = b[(size_t)(e / W) * ld + e % W];
        s += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        const double r = sqrt(t / ((double)H * W));
        *out = r > 0.0 ? (float)r : 1.0f;
    }
}

// Coarse-grid prediction. restrict: block means over k x k cells of a plane
// (pitch ld) into a dense (H/k) x (W/k) plane.
__global__ void k_restrict(const float *__restrict__ b, int ld, int H, int W, int k, float *__restrict__ bc)
{
    const int Wc = W / k, Hc = H / k;
    const float inv = 1.0f / (float)(k * k);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Hc * Wc; e += gridDim.x * blockDim.x) {
        const int I = e % Wc, J = e / Wc;
        float s = 0.0f;
        for (int dj = 0; dj < k; ++dj) {
            const float *row = b + (size_t)(J * k + dj) * ld + I * k;
            for (int di = 0; di < k; ++di) s += row[di];
        }
        bc[e] = s * inv;
    }
}

// prolong: periodic bilinear interpolation of a dense (H/k) x (W/k) plane at
// the fine cell centres, times `scale`, into a plane of pitch ld. Fine cell i
// sits at coarse coordinate (i + 1/2) / k - 1/2 (coarse cell I's centre is at
// fine coordinate k I + (k - 1) / 2).
__global__ void k_prolong(const float *__restrict__ pc, int k, float scale, float *__restrict__ p, int ld, int H, int W)
{
    const int Wc = W / k, Hc = H / k;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < H * W; e += gridDim.x * blockDim.x) {
        const int i = e % W, j = e / W;
        const float x = ((float)i + 0.5f) / (float)k - 0.5f, y = ((float)j + 0.5f) / (float)k - 0.5f;
        const float fx = floorf(x), fy = floorf(y);
        const float sx = x - fx, sy = y - fy;
        const int i0 = ((int)fx + Wc) % Wc, j0 = ((int)fy + Hc) % Hc;
        const int i1 = (i0 + 1) % Wc, j1 = (j0 + 1) % Hc;
        const float v00 = pc[(size_t)j0 * Wc + i0], v10 = pc[(size_t)j0 * Wc + i1];
        const float v01 = pc[(size_t)j1 * Wc + i0], v11 = pc[(size_t)j1 * Wc + i1];
        const float v = (1.0f - sy) * ((1.0f - sx) * v00 + sx * v10) + sy * ((1.0f - sx) * v01 + sx * v11);
        p[(size_t)j * ld + i] = v * scale;
    }
}

inline int nblk(size_t n, int t = 256) { return (int)std::min<size_t>((n + t - 1) / t, 152 * 16); }

}  // namespace

// ---- launchers -------------------------------------------------------------------------------

template <int CIN, int CINP, int COUT, int EPI>
static cudaError_t conv_t(Tensor in, const bf16 *w, const float *bias, Tensor out, float *outf, int fs, int fo, int n,
                          int H, int W, cudaStream_t st)
{
    const int nseg = n * H * (W / 16);
    k_conv3x3<CIN, CINP, COUT, EPI><<<(nseg + 3) / 4, 128, 0, st>>>(in, w, bias, out, outf, fs, fo, n, H, W);
    return launched();
}

#define PFS_CONV_CASE(CI, CIP, CO)                                                                         \
    if (cin == CI && cout == CO) {                                                                         \
        if (epi == 0) return conv_t<CI, CIP, CO, EPI_RELU_BF16>(in, w, bias, out, outf, fs, fo, n, H, W, st); \
        if (epi == 1) return conv_t<CI, CIP, CO, EPI_F32_STORE>(in, w, bias, out, outf, fs, fo, n, H, W, st); \
        return conv_t<CI, CIP, CO, EPI_F32_ADD>(in, w, bias, out, outf, fs, fo, n, H, W, st);                \
    }

cudaError_t conv3x3(Tensor in, int cin, const bf16 *w, const float *bias, Tensor out, int cout, float *outf, int fs,
                    int fo, int epi, int n, int H, int W, cudaStream_t st)
{
    // forward layers
    PFS_CONV_CASE(1, 16, 16)
    PFS_CONV_CASE(16, 16, 16)
    PFS_CONV_CASE(16, 16, 32)
    PFS_CONV_CASE(32, 32, 32)
    PFS_CONV_CASE(32, 32, 64)
    PFS_CONV_CASE(64, 64, 64)
    PFS_CONV_CASE(128, 128, 64)
    PFS_CONV_CASE(96, 96, 32)
    PFS_CONV_CASE(48, 48, 16)
    // input gradients (transposed layers)
    PFS_CONV_CASE(32, 32, 16)
    PFS_CONV_CASE(64, 64, 32)
    PFS_CONV_CASE(64, 64, 128)
    PFS_CONV_CASE(32, 32, 96)
    PFS_CONV_CASE(16, 16, 48)
    return cudaErrorInvalidValue;
}
#undef PFS_CONV_CASE

cudaError_t wgrad3x3(Tensor x, int cin, int cinp, const bf16 *dy, int cout, float *dw, float *db, int n, int H, int W,
                     cudaStream_t st)
{
    if (W % 16 || cout % 8) return cudaErrorInvalidValue;
    const int seg_len = W < kWgSeg ? W : kWgSeg;
    if (W % seg_len) return cudaErrorInvalidValue;
    const int total = n * H * (W / seg_len);
    // about one block per SM per (co, ci) tile: each block's atomics are amortised over many segments
    const int tiles = ((cout + 31) / 32) * ((cin + 31) / 32);
    const int want = (2 * 152 + tiles - 1) / tiles;
    const int per = (total + want - 1) / want;
    dim3 grid((total + per - 1) / per, (cout + 31) / 32, (cin + 31) / 32);
    k_wgrad_tc<<<grid, 128, 0, st>>>(x, dy, cout, cin, cinp, dw, db, n, H, W, seg_len, per);
    return launched();
}

cudaError_t pool2(Tensor in, Tensor out, int c, int n, int H, int W, cudaStream_t st)
{
    k_pool<<<nblk((size_t)n * H * W * c / 4), 256, 0, st>>>(in, out, c, n, H, W);
    return launched();
}
cudaError_t pool2_bwd(const float *dout, int ds, int doff, float *din, int is, int ioff, int c, int n, int H, int W,
                      cudaStream_t st)
{
    k_pool_bwd<<<nblk((size_t)n * H * W * c), 256, 0, st>>>(dout, ds, doff, din, is, ioff, c, n, H, W);
    return launched();
}
cudaError_t up2(Tensor in, Tensor out, int c, int n, int H, int W, cudaStream_t st)
{
    k_up<<<nblk((size_t)n * H * W * c), 256, 0, st>>>(in, out, c, n, H, W);
    return launched();
}
cudaError_t up2_bwd(const float *dout, int ds, int doff, float *din, int is, int ioff, int c, int n, int H, int W,
                    cudaStream_t st)
{
    k_up_bwd<<<nblk((size_t)n * H * W * c), 256, 0, st>>>(dout, ds, doff, din, is, ioff, c, n, H, W);
    return launched();
}
cudaError_t relu_bwd(const float *dout, int ds, int doff, Tensor y, bf16 *dpre, int c, size_t npix, cudaStream_t st)
{
    k_relu_bwd<<<nblk(npix * c), 256, 0, st>>>(dout, ds, doff, y, dpre, c, npix);
    return launched();
}
cudaError_t head(Tensor x, const float *w, const float *b, float *out, int c, size_t npix, cudaStream_t st)
{
    k_head<<<nblk(npix), 256, 0, st>>>(x, w, b, out, c, npix);
    return launched();
}
cudaError_t head_bwd(Tensor x, const float *w, const float *dout, float *dx, float *dw, float *db, int c, size_t npix,
                     cudaStream_t st)
{
    k_head_bwd<<<nblk(npix), 256, 0, st>>>(x, w, dout, dx, dw, db, c, npix);
    return launched();
}
cudaError_t mse(const float *pred, const float *target, float *dpred, size_t n, float *loss, cudaStream_t st)
{
    k_mse<<<nblk(n), 256, 0, st>>>(pred, target, dpred, n, loss);
    return launched();
}
cudaError_t adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps,
                 float c1, float c2, cudaStream_t st)
{
    k_adam<<<nblk(n), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return launched();
}
cudaError_t weights_to_bf16(const float *wf, bf16 *wb, bf16 *wt, int cout, int cin, int cinp, int coutp,
                            cudaStream_t st)
{
    k_weights_to_bf16<<<nblk((size_t)cout * 9 * cinp), 256, 0, st>>>(wf, wb, wt, cout, cin, cinp, coutp);
    return launched();
}
cudaError_t to_input(const float *b, int ld, const float *scale, bf16 *xin, int H, int W, int img, cudaStream_t st)
{
    k_to_input<<<nblk((size_t)H * W), 256, 0, st>>>(b, ld, scale, xin, H, W, img);
    return launched();
}
cudaError_t from_output(const float *y, const float *scale, float *p, int ld, int H, int W, cudaStream_t st)
{
    k_from_output<<<nblk((size_t)H * W), 256, 0, st>>>(y, scale, p, ld, H, W);
    return launched();
}
cudaError_t restrict_mean(const float *b, int ld, int H, int W, int k, float *bc, cudaStream_t st)
{
    k_restrict<<<nblk((size_t)(H / k) * (W / k)), 256, 0, st>>>(b, ld, H, W, k, bc);
    return launched();
}
cudaError_t prolong(const float *pc, int k, float scale, float *p, int ld, int H, int W, cudaStream_t st)
{
    k_prolong<<<nblk((size_t)H * W), 256, 0, st>>>(pc, k, scale, p, ld, H, W);
    return launched();
}
cudaError_t rms(const float *b, int ld, int H, int W, float *out, cudaStream_t st)
{
    k_rms<<<1, 1024, 0, st>>>(b, ld, H, W, out);
    return launched();
}

}  // namespace unet
}  // namespace pfs
