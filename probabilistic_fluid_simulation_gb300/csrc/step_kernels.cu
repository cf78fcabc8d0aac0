// Velocity advection, diffusion, divergence, projection, image advection,
// layout conversion and the residual reduction, on planar float32 fields.
// Each kernel follows one routine of the reference's src/fluid.cpp (cited
// per kernel) with the same per-cell arithmetic, so results are bit-equal.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace pfs {
namespace {

constexpr int kBX = 32, kBY = 8;

inline dim3 grid2d(int w, int h) { return dim3((w + kBX - 1) / kBX, (h + kBY - 1) / kBY); }

__device__ __forceinline__ int wm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wp(int i, int n) { return i + 1 == n ? 0 : i + 1; }

// Backtrace, wrap and corner cells of one sample (src/fluid.cpp:39-58 and
// :97-114): x' = i - (k*u)/n wrapped to [0, n).
struct Corners {
    int i0, i1, j0, j1;
    float sx, sy;
};

__device__ __forceinline__ Corners backtrace(int i, int j, float kx, float ky, float u, float v, float fw, float fh,
                                            int w, int h)
{
    float xp = fsub((float)i, fdiv(fmul(kx, u), fw));
    float yp = fsub((float)j, fdiv(fmul(ky, v), fh));
    xp = wrap_coord(xp, fw);
    yp = wrap_coord(yp, fh);
    Corners c;
    c.i0 = cell_of(xp, w);
    c.j0 = cell_of(yp, h);
    c.i1 = (c.i0 + 1) % w;
    c.j1 = (c.j0 + 1) % h;
    c.sx = fsub(xp, (float)c.i0);
    c.sy = fsub(yp, (float)c.j0);
    return c;
}

// src/fluid.cpp:24-70
__global__ void k_advect(const float *__restrict__ u, const float *__restrict__ v, float *__restrict__ uo,
                         float *__restrict__ vo, int ld, int w, int h, float dt)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t o = (size_t)j * ld + i;
    const Corners c = backtrace(i, j, dt, dt, u[o], v[o], (float)w, (float)h, w, h);
    const size_t r0 = (size_t)c.j0 * ld, r1 = (size_t)c.j1 * ld;
    uo[o] = bilerp(c.sx, c.sy, u[r0 + c.i0], u[r0 + c.i1], u[r1 + c.i0], u[r1 + c.i1]);
    vo[o] = bilerp(c.sx, c.sy, v[r0 + c.i0], v[r0 + c.i1], v[r1 + c.i0], v[r1 + c.i1]);
}

// One diffusion sweep, src/fluid.cpp:151-186
__global__ void k_diffuse(const float *__restrict__ u, const float *__restrict__ v, float *__restrict__ uo,
                          float *__restrict__ vo, int ld, int w, int h, float alpha, float beta)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t r = (size_t)j * ld, rm = (size_t)wm(j, h) * ld, rp = (size_t)wp(j, h) * ld;
    const int im = wm(i, w), ip = wp(i, w);
    uo[r + i] = jacobi_d(u[r + im], u[r + ip], u[rm + i], u[rp + i], u[r + i], alpha, beta);
    vo[r + i] = jacobi_d(v[r + im], v[r + ip], v[rm + i], v[rp + i], v[r + i], alpha, beta);
}

// Divergence, src/fluid.cpp:218-237 (gamma = (float)(-1.0/dt) from the host);
// also sums b^2 (double) for the residual's denominator.
__global__ void __launch_bounds__(256) k_divergence(const float *__restrict__ u, const float *__restrict__ v,
                                                    float *__restrict__ b, int ld, int w, int h, float gamma,
                                                    Reduce red)
{
    FFAcc acc;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        const size_t r = (size_t)j * ld, rm = (size_t)wm(j, h) * ld, rp = (size_t)wp(j, h) * ld;
        for (int i = threadIdx.x; i < w; i += blockDim.x) {
            const float du = fsub(u[r + wp(i, w)], u[r + wm(i, w)]);
            const float dv = fsub(v[rp + i], v[rm + i]);
            const float bv = fmul(gamma, fadd(du, dv));
            b[r + i] = bv;
            acc_square(acc, bv);
        }
    }
    reduce_blocks(acc.value(), red, 1);
}

// Residual of the pressure system (src/fluid.cpp:239-257 solves 4p - sum nb = b),
// r = b + pL + pR + pT + pB - 4p. The five additions are error-free (TwoSum),
// so hi + lo carries r with a relative error near 2^-48 (the error terms are
// summed in float). r^2 = hi^2 + (fma error of hi^2) + 2 hi lo is added to
// the float-float accumulator.
__device__ __forceinline__ void residual_sq(FFAcc &acc, float b, float l, float r, float t, float bo, float c)
{
    FF s = two_sum(b, l);
    float e = s.lo;
    s = two_sum(s.hi, r);
    e = __fadd_rn(e, s.lo);
    s = two_sum(s.hi, t);
    e = __fadd_rn(e, s.lo);
    s = two_sum(s.hi, bo);
    e = __fadd_rn(e, s.lo);
    s = two_sum(s.hi, __fmul_rn(-4.0f, c));  // -4p is exact
    e = __fadd_rn(e, s.lo);
    const FF q = two_sum(s.hi, e);
    const float sq = __fmul_rn(q.hi, q.hi);
    const float sq_err = __fmaf_rn(q.hi, q.hi, -sq);
    const float cross = __fmul_rn(__fmul_rn(2.0f, q.hi), q.lo);
    acc.add(sq, __fadd_rn(sq_err, cross));
}

__global__ void __launch_bounds__(256) k_residual(const float *__restrict__ p, const float *__restrict__ b, int ld,
                                                  int w, int h, Reduce red, SolveState *state, int sweeps_here,
                                                  double tol)
{
    if (state && *(volatile int *)&state->done) return;  // same answer for every block
    FFAcc acc;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        const size_t r = (size_t)j * ld, rm = (size_t)wm(j, h) * ld, rp = (size_t)wp(j, h) * ld;
        for (int i = threadIdx.x; i < w; i += blockDim.x)
            residual_sq(acc, b[r + i], p[r + wm(i, w)], p[r + wp(i, w)], p[rm + i], p[rp + i], p[r + i]);
    }
    reduce_blocks(acc.value(), red, 0, state, sweeps_here, tol);
}

__global__ void __launch_bounds__(256) k_norms(const float *__restrict__ p, const float *__restrict__ b, int ld, int w,
                                               int h, Reduce red)
{
    FFAcc acc, accb;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        const size_t r = (size_t)j * ld, rm = (size_t)wm(j, h) * ld, rp = (size_t)wp(j, h) * ld;
        for (int i = threadIdx.x; i < w; i += blockDim.x) {
            const float bv = b[r + i];
            residual_sq(acc, bv, p[r + wm(i, w)], p[r + wp(i, w)], p[rm + i], p[rp + i], p[r + i]);
            acc_square(accb, bv);
        }
    }
    reduce_blocks(acc.value(), red, 0);
    __syncthreads();
    reduce_blocks(accb.value(), red, 1);
}

// Residual on warp strips (w % 4 == 0): each warp covers 128 columns (four
// per lane, float4 rows) and a chunk of rows, keeping rows r-1, r, r+1 of p in
// registers; left/right neighbours come from the adjacent lanes by shuffle,
// and the lanes at the strip edges read their outside neighbour directly.
// Same per-cell arithmetic as residual_sq, so the same sums.
constexpr int kResChunk = 8;    // rows per warp
constexpr int kResWarps = 8;    // warps per block

__global__ void __launch_bounds__(kResWarps * 32) k_residual_strip(const float *__restrict__ p,
                                                                   const float *__restrict__ b, int ld, int w,
                                                                   int h, int nsx, int nwork, Reduce red,
                                                                   SolveState *state, int sweeps_here, double tol,
                                                                   int with_b)
{
    if (state && *(volatile int *)&state->done) return;  // same answer for every block
    const int lane = threadIdx.x & 31;
    FFAcc acc[4], accb;  // one accumulator per lane column: four independent chains
    for (int wid = blockIdx.x * kResWarps + (threadIdx.x >> 5); wid < nwork; wid += gridDim.x * kResWarps) {
        const int sx = wid % nsx, sy = wid / nsx;
        const int x = sx * 128 + 4 * lane;
        const bool active = x < w;
        const int xs = active ? x : w - 4;  // inactive lanes shadow a valid column, results discarded
        const int last_lane = min(31, (w - sx * 128) / 4 - 1);
        const int xl = (sx * 128 == 0) ? w - 1 : sx * 128 - 1;         // left outside neighbour
        const int xr = (sx * 128 + 4 * (last_lane + 1)) % w;           // right outside neighbour
        const int y0 = sy * kResChunk, y1 = min(h, y0 + kResChunk);
        const float *pc = p + xs;
        float4 up = *reinterpret_cast<const float4 *>(pc + (size_t)wm(y0, h) * ld);
        float4 cu = *reinterpret_cast<const float4 *>(pc + (size_t)y0 * ld);
        for (int y = y0; y < y1; ++y) {
            const float4 dn = *reinterpret_cast<const float4 *>(pc + (size_t)wp(y, h) * ld);
            const float4 bb = *reinterpret_cast<const float4 *>(b + (size_t)y * ld + xs);
            float lft = __shfl_up_sync(0xffffffffu, cu.w, 1);
            float rgt = __shfl_down_sync(0xffffffffu, cu.x, 1);
            if (lane == 0) lft = p[(size_t)y * ld + xl];
            if (lane == last_lane) rgt = p[(size_t)y * ld + xr];
            if (active) {
                residual_sq(acc[0], bb.x, lft, cu.y, up.x, dn.x, cu.x);
                residual_sq(acc[1], bb.y, cu.x, cu.z, up.y, dn.y, cu.y);
                residual_sq(acc[2], bb.z, cu.y, cu.w, up.z, dn.z, cu.z);
                residual_sq(acc[3], bb.w, cu.z, rgt, up.w, dn.w, cu.w);
                if (with_b) {
                    acc_square(accb, bb.x);
                    acc_square(accb, bb.y);
                    acc_square(accb, bb.z);
                    acc_square(accb, bb.w);
                }
            }
            up = cu;
            cu = dn;
        }
    }
    reduce_blocks((acc[0].value() + acc[1].value()) + (acc[2].value() + acc[3].value()), red, 0, state, sweeps_here,
                  tol);
    if (with_b) {
        __syncthreads();
        reduce_blocks(accb.value(), red, 1);
    }
}

// Projection, src/fluid.cpp:269-296: u - ((pR-pL)*dt)/2, v - ((pB-pT)*dt)/2.
__device__ __forceinline__ void project_cell(const float *__restrict__ u, const float *__restrict__ v,
                                             const float *__restrict__ p, int ld, int w, int h, float dt, int i,
                                             int j, float &uo, float &vo)
{
    const size_t r = (size_t)j * ld;
    const float gx = fmul(fmul(fsub(p[r + wp(i, w)], p[r + wm(i, w)]), dt), 0.5f);
    const float gy = fmul(fmul(fsub(p[(size_t)wp(j, h) * ld + i], p[(size_t)wm(j, h) * ld + i]), dt), 0.5f);
    uo = fsub(u[r + i], gx);
    vo = fsub(v[r + i], gy);
}

__global__ void k_project(const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ p,
                          float *__restrict__ uo, float *__restrict__ vo, int ld, int w, int h, float dt)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    float a, c;
    project_cell(u, v, p, ld, w, h, dt, i, j, a, c);
    uo[(size_t)j * ld + i] = a;
    vo[(size_t)j * ld + i] = c;
}

// Projection, then image advection (src/fluid.cpp:72-127) of the pixel at the
// same cell with the just-projected velocity. Valid when the image grid equals
// the velocity grid: then viw = vih = 1 and the nearest velocity cell of pixel
// (i, j) is (i, j) itself.
__global__ void k_project_advect_image(const float *__restrict__ u, const float *__restrict__ v,
                                       const float *__restrict__ p, float *__restrict__ uo, float *__restrict__ vo,
                                       int ld, int w, int h, float dt, const float *__restrict__ img,
                                       float *__restrict__ imgo, size_t plane, int c)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    float un, vn;
    project_cell(u, v, p, ld, w, h, dt, i, j, un, vn);
    const size_t o = (size_t)j * ld + i;
    uo[o] = un;
    vo[o] = vn;
    // dt / viw with viw = 1.0f is dt exactly
    const Corners k = backtrace(i, j, dt, dt, un, vn, (float)w, (float)h, w, h);
    const size_t r0 = (size_t)k.j0 * ld, r1 = (size_t)k.j1 * ld;
    for (int ch = 0; ch < c; ++ch) {
        const float *s = img + ch * plane;
        imgo[ch * plane + o] = bilerp(k.sx, k.sy, s[r0 + k.i0], s[r0 + k.i1], s[r1 + k.i0], s[r1 + k.i1]);
    }
}

// Image advection, src/fluid.cpp:72-127, planar image and velocity.
__global__ void k_advect_image_planar(const float *__restrict__ img, float *__restrict__ imgo, size_t plane,
                                      int ild, int iw, int ih, int c, const float *__restrict__ u,
                                      const float *__restrict__ v, int vld, int vw, int vh, float dt, float viw,
                                      float vih, float kx, float ky)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= iw || j >= ih) return;
    const int vi = min(__float2int_rz(fmul((float)i, viw)), vw - 1);
    const int vj = min(__float2int_rz(fmul((float)j, vih)), vh - 1);
    const size_t vo = (size_t)vj * vld + vi;
    const Corners k = backtrace(i, j, kx, ky, u[vo], v[vo], (float)iw, (float)ih, iw, ih);
    const size_t r0 = (size_t)k.j0 * ild, r1 = (size_t)k.j1 * ild, o = (size_t)j * ild + i;
    for (int ch = 0; ch < c; ++ch) {
        const float *s = img + ch * plane;
        imgo[ch * plane + o] = bilerp(k.sx, k.sy, s[r0 + k.i0], s[r0 + k.i1], s[r1 + k.i0], s[r1 + k.i1]);
    }
}

// Image advection on the reference layout: image (ih, iw, c), velocity (vh, vw, 4).
__global__ void k_advect_image_interleaved(const float *__restrict__ img, float *__restrict__ imgo, int iw, int ih,
                                           int c, const float *__restrict__ vel, int vw, int vh, float dt,
                                           float viw, float vih, float kx, float ky)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= iw || j >= ih) return;
    const int vi = min(__float2int_rz(fmul((float)i, viw)), vw - 1);
    const int vj = min(__float2int_rz(fmul((float)j, vih)), vh - 1);
    const float2 uv = *reinterpret_cast<const float2 *>(vel + ((size_t)vj * vw + vi) * 4);
    const Corners k = backtrace(i, j, kx, ky, uv.x, uv.y, (float)iw, (float)ih, iw, ih);
    const size_t c00 = ((size_t)k.j0 * iw + k.i0) * c, c10 = ((size_t)k.j0 * iw + k.i1) * c;
    const size_t c01 = ((size_t)k.j1 * iw + k.i0) * c, c11 = ((size_t)k.j1 * iw + k.i1) * c;
    const size_t o = ((size_t)j * iw + i) * c;
    for (int ch = 0; ch < c; ++ch)
        imgo[o + ch] = bilerp(k.sx, k.sy, img[c00 + ch], img[c10 + ch], img[c01 + ch], img[c11 + ch]);
}

__global__ void k_split_velocity(const float4 *__restrict__ vp, float *__restrict__ u, float *__restrict__ v, int ld,
                                 int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const float4 q = vp[(size_t)j * w + i];
    u[(size_t)j * ld + i] = q.x;
    v[(size_t)j * ld + i] = q.y;
}

__global__ void k_split_channel(const float *__restrict__ buf, int ch, int nch, float *__restrict__ plane, int ld,
                                int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    plane[(size_t)j * ld + i] = buf[((size_t)j * w + i) * nch + ch];
}

__global__ void k_merge_velocity(float4 *__restrict__ out, const float *__restrict__ u, const float *__restrict__ v,
                                 const float *__restrict__ p, const float *__restrict__ b, int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t o = (size_t)j * ld + i;
    out[(size_t)j * w + i] = make_float4(u[o], v[o], p[o], b[o]);
}

__global__ void k_split_image(const float *__restrict__ img, float *__restrict__ planes, size_t plane, int ld, int w,
                              int h, int c)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    for (int ch = 0; ch < c; ++ch) planes[ch * plane + (size_t)j * ld + i] = img[((size_t)j * w + i) * c + ch];
}

__global__ void k_merge_image(float *__restrict__ img, const float *__restrict__ planes, size_t plane, int ld, int w,
                              int h, int c)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    for (int ch = 0; ch < c; ++ch) img[((size_t)j * w + i) * c + ch] = planes[ch * plane + (size_t)j * ld + i];
}

}  // namespace

__global__ void k_widen(const float *__restrict__ in, double *__restrict__ out, size_t n)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = (double)in[k];
}

cudaError_t launch_widen(const float *in, double *out, size_t n, cudaStream_t st)
{
    if (!out || !n) return cudaSuccess;
    k_widen<<<kReduceBlocks, 256, 0, st>>>(in, out, n);
    return launched();
}

cudaError_t launch_advect(const float *u, const float *v, float *uo, float *vo, int ld, int w, int h, float dt,
                          cudaStream_t st)
{
    k_advect<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(u, v, uo, vo, ld, w, h, dt);
    return launched();
}

cudaError_t launch_diffuse_sweep(const float *u, const float *v, float *uo, float *vo, int ld, int w, int h,
                                 float alpha, float beta, cudaStream_t st)
{
    k_diffuse<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(u, v, uo, vo, ld, w, h, alpha, beta);
    return launched();
}

cudaError_t launch_divergence(const float *u, const float *v, float *b, int ld, int w, int h, float gamma,
                              const Reduce &red, cudaStream_t st)
{
    k_divergence<<<red.nblocks, 256, 0, st>>>(u, v, b, ld, w, h, gamma, red);
    return launched();
}

static bool strip_ok(int w, int ld) { return w % 4 == 0 && ld % 4 == 0; }

static void strip_grid(int w, int h, int nblocks_max, int &nsx, int &nwork, int &blocks)
{
    nsx = (w + 127) / 128;
    nwork = nsx * ((h + kResChunk - 1) / kResChunk);
    blocks = std::min((nwork + kResWarps - 1) / kResWarps, nblocks_max);
}

cudaError_t launch_residual(const float *p, const float *b, int ld, int w, int h, const Reduce &red,
                            SolveState *state, int sweeps_here, double tol, cudaStream_t st)
{
    if (strip_ok(w, ld)) {
        int nsx, nwork, blocks;
        strip_grid(w, h, red.nblocks, nsx, nwork, blocks);
        k_residual_strip<<<blocks, kResWarps * 32, 0, st>>>(p, b, ld, w, h, nsx, nwork, red, state, sweeps_here, tol, 0);
        return launched();
    }
    k_residual<<<red.nblocks, 256, 0, st>>>(p, b, ld, w, h, red, state, sweeps_here, tol);
    return launched();
}

cudaError_t launch_norms(const float *p, const float *b, int ld, int w, int h, const Reduce &red, cudaStream_t st)
{
    if (strip_ok(w, ld)) {
        int nsx, nwork, blocks;
        strip_grid(w, h, red.nblocks, nsx, nwork, blocks);
        k_residual_strip<<<blocks, kResWarps * 32, 0, st>>>(p, b, ld, w, h, nsx, nwork, red, nullptr, 0, 0.0, 1);
        return launched();
    }
    k_norms<<<red.nblocks, 256, 0, st>>>(p, b, ld, w, h, red);
    return launched();
}

cudaError_t launch_project(const float *u, const float *v, const float *p, float *uo, float *vo, int ld, int w,
                           int h, float dt, cudaStream_t st)
{
    k_project<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(u, v, p, uo, vo, ld, w, h, dt);
    return launched();
}

cudaError_t launch_project_advect_image(const float *u, const float *v, const float *p, float *uo, float *vo,
                                        int ld, int w, int h, float dt, const float *img, float *imgo,
                                        size_t img_plane, int c, cudaStream_t st)
{
    k_project_advect_image<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(u, v, p, uo, vo, ld, w, h, dt, img, imgo,
                                                                     img_plane, c);
    return launched();
}

// viw = fvw/fiw, kx = dt/viw exactly as src/fluid.cpp:82-83,97 compute them.
static void image_scales(int iw, int ih, int vw, int vh, float dt, float &viw, float &vih, float &kx, float &ky)
{
    viw = (float)vw / (float)iw;
    vih = (float)vh / (float)ih;
    kx = dt / viw;
    ky = dt / vih;
}

cudaError_t launch_advect_image_planar(const float *img, float *imgo, size_t img_plane, int ild, int iw, int ih,
                                       int c, const float *u, const float *v, int vld, int vw, int vh, float dt,
                                       cudaStream_t st)
{
    float viw, vih, kx, ky;
    image_scales(iw, ih, vw, vh, dt, viw, vih, kx, ky);
    k_advect_image_planar<<<grid2d(iw, ih), dim3(kBX, kBY), 0, st>>>(img, imgo, img_plane, ild, iw, ih, c, u, v, vld,
                                                                     vw, vh, dt, viw, vih, kx, ky);
    return launched();
}

cudaError_t launch_advect_image_interleaved(const float *img, float *imgo, int iw, int ih, int c,
                                            const float *vel, int vw, int vh, float dt, cudaStream_t st)
{
    float viw, vih, kx, ky;
    image_scales(iw, ih, vw, vh, dt, viw, vih, kx, ky);
    k_advect_image_interleaved<<<grid2d(iw, ih), dim3(kBX, kBY), 0, st>>>(img, imgo, iw, ih, c, vel, vw, vh, dt,
                                                                           viw, vih, kx, ky);
    return launched();
}

cudaError_t launch_split_velocity(const float *vp, float *u, float *v, int ld, int w, int h, cudaStream_t st)
{
    k_split_velocity<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(reinterpret_cast<const float4 *>(vp), u, v, ld, w, h);
    return launched();
}

cudaError_t launch_split_channel(const float *buf, int ch, int nch, float *plane, int ld, int w, int h,
                                 cudaStream_t st)
{
    k_split_channel<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(buf, ch, nch, plane, ld, w, h);
    return launched();
}

cudaError_t launch_merge_velocity(float *out, const float *u, const float *v, const float *p, const float *b,
                                  int ld, int w, int h, cudaStream_t st)
{
    k_merge_velocity<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(reinterpret_cast<float4 *>(out), u, v, p, b, ld, w, h);
    return launched();
}

cudaError_t launch_split_image(const float *img, float *planes, size_t plane, int ld, int w, int h, int c,
                               cudaStream_t st)
{
    k_split_image<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(img, planes, plane, ld, w, h, c);
    return launched();
}

cudaError_t launch_merge_image(float *img, const float *planes, size_t plane, int ld, int w, int h, int c,
                               cudaStream_t st)
{
    k_merge_image<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(img, planes, plane, ld, w, h, c);
    return launched();
}

}  // namespace pfs
