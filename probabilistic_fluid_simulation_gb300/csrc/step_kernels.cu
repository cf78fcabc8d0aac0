// Velocity advection, diffusion, divergence, projection, image advection,
// layout conversion and the residual reduction, on planar float32 fields.
// Each kernel follows one routine of the reference's src/fluid.cpp (cited
// per kernel) with the same per-cell arithmetic, so results are bit-equal.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "reduce.cuh"
#include "cells.cuh"

namespace pfs {
namespace {

constexpr int kBX = 32, kBY = 8;

inline dim3 grid2d(int w, int h) { return dim3((w + kBX - 1) / kBX, (h + kBY - 1) / kBY); }

// src/fluid.cpp:24-70 (BC: boundary mode, cells.cuh)
template <int BC>
__global__ void k_advect(const float *__restrict__ u, const float *__restrict__ v, float *__restrict__ uo,
                         float *__restrict__ vo, int ld, int w, int h, float dt)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    advect_cell<BC>(u, v, uo, vo, ld, w, h, dt, i, j);
}

// One diffusion sweep, src/fluid.cpp:151-186
__global__ void k_diffuse(const float *__restrict__ u, const float *__restrict__ v, float *__restrict__ uo,
                          float *__restrict__ vo, int ld, int w, int h, float alpha, float beta)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t r = (size_t)j * ld, rm = (size_t)wm(j, h) * ld, rp = (size_t)wp(j, h) * ld;
    const int im = wm(i, w), ip = wp(i, w);
    const long long n = (long long)ld * h;
    (void)n;
    PFS_ST(uo, r + i, n,
           jacobi_d(PFS_LD(u, r + im, n, kBsDiffuse), PFS_LD(u, r + ip, n, kBsDiffuse), PFS_LD(u, rm + i, n, kBsDiffuse),
                    PFS_LD(u, rp + i, n, kBsDiffuse), PFS_LD(u, r + i, n, kBsDiffuse), alpha, beta),
           kBsDiffuse);
    PFS_ST(vo, r + i, n,
           jacobi_d(PFS_LD(v, r + im, n, kBsDiffuse), PFS_LD(v, r + ip, n, kBsDiffuse), PFS_LD(v, rm + i, n, kBsDiffuse),
                    PFS_LD(v, rp + i, n, kBsDiffuse), PFS_LD(v, r + i, n, kBsDiffuse), alpha, beta),
           kBsDiffuse);
}

// Divergence, src/fluid.cpp:218-237 (gamma = (float)(-1.0/dt) from the host);
// also sums b^2 (double) for the residual's denominator.
__global__ void __launch_bounds__(256) k_divergence(const float *__restrict__ u, const float *__restrict__ v,
                                                    float *__restrict__ b, int ld, int w, int h, float gamma,
                                                    Reduce red)
{
    FFAcc acc;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        for (int i = threadIdx.x; i < w; i += blockDim.x) acc_square(acc, divergence_cell(u, v, b, ld, w, h, gamma, i, j));
    }
    reduce_blocks(acc.value(), red, 1);
}

__global__ void __launch_bounds__(256) k_residual(const float *__restrict__ p, const float *__restrict__ b, int ld,
                                                  int w, int h, Reduce red, SolveState *state, int sweeps_here,
                                                  double tol, int stall_window)
{
    if (state && *(volatile int *)&state->done) return;  // same answer for every block
    FFAcc acc;
    const long long n = (long long)ld * h;
    (void)n;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        const size_t r = (size_t)j * ld, rm = (size_t)wm(j, h) * ld, rp = (size_t)wp(j, h) * ld;
        for (int i = threadIdx.x; i < w; i += blockDim.x)
            residual_sq(acc, PFS_LD(b, r + i, n, kBsResidual), PFS_LD(p, r + wm(i, w), n, kBsResidual),
                        PFS_LD(p, r + wp(i, w), n, kBsResidual), PFS_LD(p, rm + i, n, kBsResidual),
                        PFS_LD(p, rp + i, n, kBsResidual), PFS_LD(p, r + i, n, kBsResidual));
    }
    reduce_blocks(acc.value(), red, 0, state, sweeps_here, tol, stall_window);
}

__global__ void __launch_bounds__(256) k_norms(const float *__restrict__ p, const float *__restrict__ b, int ld, int w,
                                               int h, Reduce red)
{
    FFAcc acc, accb;
    const long long n = (long long)ld * h;
    (void)n;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        const size_t r = (size_t)j * ld, rm = (size_t)wm(j, h) * ld, rp = (size_t)wp(j, h) * ld;
        for (int i = threadIdx.x; i < w; i += blockDim.x) {
            const float bv = PFS_LD(b, r + i, n, kBsResidual);
            residual_sq(acc, bv, PFS_LD(p, r + wm(i, w), n, kBsResidual), PFS_LD(p, r + wp(i, w), n, kBsResidual),
                        PFS_LD(p, rm + i, n, kBsResidual), PFS_LD(p, rp + i, n, kBsResidual),
                        PFS_LD(p, r + i, n, kBsResidual));
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
                                                                   int with_b, int stall_window)
{
    if (state && *(volatile int *)&state->done) return;  // same answer for every block
    const int lane = threadIdx.x & 31;
    FFAcc2 acc[2];  // one chain per lane column, two columns per packed accumulator
    FFAcc accb;
    for (int wid = blockIdx.x * kResWarps + (threadIdx.x >> 5); wid < nwork; wid += gridDim.x * kResWarps) {
        const int sx = wid % nsx, sy = wid / nsx;
        const int y0 = sy * kResChunk, y1 = min(h, y0 + kResChunk);
        residual_strip_task(p, b, ld, w, h, sx, y0, y1, lane, acc, with_b ? &accb : nullptr);
    }
    reduce_blocks(acc[0].value() + acc[1].value(), red, 0, state, sweeps_here, tol, stall_window);
    if (with_b) {
        __syncthreads();
        reduce_blocks(accb.value(), red, 1);
    }
}

template <int BC>
__global__ void k_project(const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ p,
                          float *__restrict__ uo, float *__restrict__ vo, int ld, int w, int h, float dt)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    float a, c;
    project_cell<BC>(u, v, p, ld, w, h, dt, i, j, a, c);
    PFS_ST(uo, (size_t)j * ld + i, (long long)ld * h, a, kBsProject);
    PFS_ST(vo, (size_t)j * ld + i, (long long)ld * h, c, kBsProject);
}

// Projection, then image advection (src/fluid.cpp:72-127) of the pixel at the
// same cell with the just-projected velocity. Valid when the image grid equals
// the velocity grid: then viw = vih = 1 and the nearest velocity cell of pixel
// (i, j) is (i, j) itself.
template <int BC>
__global__ void k_project_advect_image(const float *__restrict__ u, const float *__restrict__ v,
                                       const float *__restrict__ p, float *__restrict__ uo, float *__restrict__ vo,
                                       int ld, int w, int h, float dt, const float *__restrict__ img,
                                       float *__restrict__ imgo, size_t plane, int c)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    project_image_cell<BC>(u, v, p, uo, vo, ld, w, h, dt, img, imgo, plane, c, i, j);
}

// Image advection, src/fluid.cpp:72-127, planar image and velocity.
template <int BC>
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
    const long long nv = (long long)vld * vh, ni = (long long)plane * c;
    (void)nv;
    (void)ni;
    const Corners k = backtrace<BC>(i, j, kx, ky, PFS_LD(u, vo, nv, kBsImage), PFS_LD(v, vo, nv, kBsImage), (float)iw,
                                    (float)ih, iw, ih);
    const size_t r0 = (size_t)k.j0 * ild, r1 = (size_t)k.j1 * ild, o = (size_t)j * ild + i;
    for (int ch = 0; ch < c; ++ch) {
        const size_t s = ch * plane;
        PFS_ST(imgo, s + o, ni,
               bilerp(k.sx, k.sy, PFS_LD(img, s + r0 + k.i0, ni, kBsImage), PFS_LD(img, s + r0 + k.i1, ni, kBsImage),
                      PFS_LD(img, s + r1 + k.i0, ni, kBsImage), PFS_LD(img, s + r1 + k.i1, ni, kBsImage)),
               kBsImage);
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
    const size_t vk = ((size_t)vj * vw + vi) * 4;
    const long long ni = (long long)iw * ih * c;
    (void)ni;
    const float2 uv = PFS_SPAN(vk, 2, (long long)vw * vh * 4, kBsImage)
                          ? *reinterpret_cast<const float2 *>(vel + vk)
                          : make_float2(0.0f, 0.0f);
    const Corners k = backtrace(i, j, kx, ky, uv.x, uv.y, (float)iw, (float)ih, iw, ih);
    const size_t c00 = ((size_t)k.j0 * iw + k.i0) * c, c10 = ((size_t)k.j0 * iw + k.i1) * c;
    const size_t c01 = ((size_t)k.j1 * iw + k.i0) * c, c11 = ((size_t)k.j1 * iw + k.i1) * c;
    const size_t o = ((size_t)j * iw + i) * c;
    for (int ch = 0; ch < c; ++ch)
        PFS_ST(imgo, o + ch, ni,
               bilerp(k.sx, k.sy, PFS_LD(img, c00 + ch, ni, kBsImage), PFS_LD(img, c10 + ch, ni, kBsImage),
                      PFS_LD(img, c01 + ch, ni, kBsImage), PFS_LD(img, c11 + ch, ni, kBsImage)),
               kBsImage);
}

__global__ void k_split_velocity(const float4 *__restrict__ vp, float *__restrict__ u, float *__restrict__ v, int ld,
                                 int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const long long n = (long long)ld * h;
    (void)n;
    const float4 q = PFS_LD(vp, (size_t)j * w + i, (long long)w * h, kBsLayout);
    PFS_ST(u, (size_t)j * ld + i, n, q.x, kBsLayout);
    PFS_ST(v, (size_t)j * ld + i, n, q.y, kBsLayout);
}

__global__ void k_split_channel(const float *__restrict__ buf, int ch, int nch, float *__restrict__ plane, int ld,
                                int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    PFS_ST(plane, (size_t)j * ld + i, (long long)ld * h,
           PFS_LD(buf, ((size_t)j * w + i) * nch + ch, (long long)w * h * nch, kBsLayout), kBsLayout);
}

// One interleaved (u, v, p, b) buffer into its planes, each cell read once
// (b may be null). The source may be host memory mapped into the device's
// address space: each 16-byte cell crosses the link once.
__global__ void k_split_vp(const float4 *__restrict__ vp, float *__restrict__ u, float *__restrict__ v,
                           float *__restrict__ p, float *__restrict__ b, int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const float4 q = PFS_LD(vp, (size_t)j * w + i, (long long)w * h, kBsLayout);
    const size_t o = (size_t)j * ld + i;
    const long long n = (long long)ld * h;
    (void)n;
    PFS_ST(u, o, n, q.x, kBsLayout);
    PFS_ST(v, o, n, q.y, kBsLayout);
    PFS_ST(p, o, n, q.z, kBsLayout);
    if (b) PFS_ST(b, o, n, q.w, kBsLayout);
}

__global__ void k_merge_velocity(float4 *__restrict__ out, const float *__restrict__ u, const float *__restrict__ v,
                                 const float *__restrict__ p, const float *__restrict__ b, int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t o = (size_t)j * ld + i;
    const long long n = (long long)ld * h;
    (void)n;
    PFS_ST(out, (size_t)j * w + i, (long long)w * h,
           make_float4(PFS_LD(u, o, n, kBsLayout), PFS_LD(v, o, n, kBsLayout), PFS_LD(p, o, n, kBsLayout),
                       PFS_LD(b, o, n, kBsLayout)),
           kBsLayout);
}

__global__ void k_split_image(const float *__restrict__ img, float *__restrict__ planes, size_t plane, int ld, int w,
                              int h, int c)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    for (int ch = 0; ch < c; ++ch)
        PFS_ST(planes, ch * plane + (size_t)j * ld + i, (long long)plane * c,
               PFS_LD(img, ((size_t)j * w + i) * c + ch, (long long)w * h * c, kBsLayout), kBsLayout);
}

__global__ void k_merge_image(float *__restrict__ img, const float *__restrict__ planes, size_t plane, int ld, int w,
                              int h, int c)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    for (int ch = 0; ch < c; ++ch)
        PFS_ST(img, ((size_t)j * w + i) * c + ch, (long long)w * h * c,
               PFS_LD(planes, ch * plane + (size_t)j * ld + i, (long long)plane * c, kBsLayout), kBsLayout);
}

}  // namespace

__global__ void k_widen(const float *__restrict__ in, double *__restrict__ out, size_t n)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        PFS_ST(out, k, n, (double)PFS_LD(in, k, n, kBsAux), kBsAux);
}

cudaError_t launch_widen(const float *in, double *out, size_t n, cudaStream_t st)
{
    if (!out || !n) return cudaSuccess;
    k_widen<<<reduce_grid(), 256, 0, st>>>(in, out, n);
    return launched();
}

// Damped Jacobi pass on a predicted start: pout = p + (b - A p) / 8, the
// Jacobi update with weight 1/2 (gain (1 + l) / 2 on an error mode of Jacobi
// eigenvalue l: zero on the checkerboard mode that undamped sweeps keep).
__global__ void k_damp(const float *__restrict__ pin, const float *__restrict__ b, float *__restrict__ pout, int ld,
                       int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t r = (size_t)j * ld;
    const int im = i == 0 ? w - 1 : i - 1, ip = i + 1 == w ? 0 : i + 1;
    const int jm = j == 0 ? h - 1 : j - 1, jp = j + 1 == h ? 0 : j + 1;
    const long long n = (long long)ld * h;
    (void)n;
    const float c = PFS_LD(pin, r + i, n, kBsAux);
    const float q = fsub(fadd(fadd(fadd(fadd(PFS_LD(b, r + i, n, kBsAux), PFS_LD(pin, r + im, n, kBsAux)),
                                        PFS_LD(pin, r + ip, n, kBsAux)),
                                   PFS_LD(pin, (size_t)jm * ld + i, n, kBsAux)),
                              PFS_LD(pin, (size_t)jp * ld + i, n, kBsAux)),
                         fmul(4.0f, c));
    PFS_ST(pout, r + i, n, fadd(c, fmul(q, 0.125f)), kBsAux);
}

cudaError_t launch_damp(const float *pin, const float *b, float *pout, int ld, int w, int h, cudaStream_t st)
{
    k_damp<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(pin, b, pout, ld, w, h);
    return launched();
}

// r = b - A p per cell (the sum order of the Jacobi update), float.
__global__ void k_residual_field(const float *__restrict__ p, const float *__restrict__ b, float *__restrict__ r, int ld,
                                 int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t o = (size_t)j * ld;
    const int im = i == 0 ? w - 1 : i - 1, ip = i + 1 == w ? 0 : i + 1;
    const int jm = j == 0 ? h - 1 : j - 1, jp = j + 1 == h ? 0 : j + 1;
    const long long n = (long long)ld * h;
    (void)n;
    PFS_ST(r, o + i, n,
           fsub(fadd(fadd(fadd(fadd(PFS_LD(b, o + i, n, kBsAux), PFS_LD(p, o + im, n, kBsAux)),
                               PFS_LD(p, o + ip, n, kBsAux)),
                          PFS_LD(p, (size_t)jm * ld + i, n, kBsAux)),
                     PFS_LD(p, (size_t)jp * ld + i, n, kBsAux)),
                fmul(4.0f, PFS_LD(p, o + i, n, kBsAux))),
           kBsAux);
}

cudaError_t launch_residual_field(const float *p, const float *b, float *r, int ld, int w, int h, cudaStream_t st)
{
    k_residual_field<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(p, b, r, ld, w, h);
    return launched();
}

__global__ void k_add(float *__restrict__ p, const float *__restrict__ d, size_t n)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        PFS_ST(p, k, n, fadd(PFS_LD(p, k, n, kBsAux), PFS_LD(d, k, n, kBsAux)), kBsAux);
}

cudaError_t launch_add(float *p, const float *d, size_t n, cudaStream_t st)
{
    k_add<<<reduce_grid(), 256, 0, st>>>(p, d, n);
    return launched();
}

// A few words copied (src non-null) or zeroed by one warp. Stores to mapped
// host memory are visible to the host once it has seen the kernel complete
// (a stream or event synchronisation).
__global__ void k_small_words(const unsigned *__restrict__ src, unsigned *__restrict__ dst, int words)
{
    for (int k = threadIdx.x; k < words; k += 32) PFS_ST(dst, k, words, src ? PFS_LD(src, k, words, kBsAux) : 0u, kBsAux);
}

cudaError_t launch_copy_small(const void *src, void *dst, size_t bytes, cudaStream_t st)
{
    if (bytes % 4 != 0 || bytes > (1u << 20)) return cudaErrorInvalidValue;
    k_small_words<<<1, 32, 0, st>>>(static_cast<const unsigned *>(src), static_cast<unsigned *>(dst),
                                    (int)(bytes / 4));
    return launched();
}

cudaError_t launch_zero_small(void *dst, size_t bytes, cudaStream_t st)
{
    return launch_copy_small(nullptr, dst, bytes, st);
}

#define PFS_BC_DISPATCH(bc, KERNEL, GRID, ...)                                     \
    do {                                                                           \
        switch (bc) {                                                              \
        case 0: KERNEL<0><<<GRID, dim3(kBX, kBY), 0, st>>>(__VA_ARGS__); break;    \
        case 1: KERNEL<1><<<GRID, dim3(kBX, kBY), 0, st>>>(__VA_ARGS__); break;    \
        case 2: KERNEL<2><<<GRID, dim3(kBX, kBY), 0, st>>>(__VA_ARGS__); break;    \
        default: return cudaErrorInvalidValue;                                     \
        }                                                                          \
    } while (0)

cudaError_t launch_advect(const float *u, const float *v, float *uo, float *vo, int ld, int w, int h, float dt,
                          cudaStream_t st, int bc)
{
    PFS_BC_DISPATCH(bc, k_advect, grid2d(w, h), u, v, uo, vo, ld, w, h, dt);
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

int device_sms()
{
    static std::atomic<int> cached[64];  // per device ordinal, 0 = not yet read
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    int n = cached[dev].load(std::memory_order_relaxed);
    if (n == 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 0;
        cached[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

int reduce_grid()
{
    const int sms = device_sms();
    return sms > 0 ? std::min(kReduceBlocks, 4 * sms) : kReduceBlocks;
}

// The strip kernel loads four cells of p and b at once (16-byte vector loads),
// so it needs w and ld multiples of 4 and both planes 16-byte aligned; any
// other layout (an offset view of a caller's plane, for one) takes the scalar
// kernel, which gives the same sums.
static bool strip_ok(const float *p, const float *b, int w, int ld)
{
    return w % 4 == 0 && ld % 4 == 0 && (((uintptr_t)p | (uintptr_t)b) & 15u) == 0;
}

static void strip_grid(int w, int h, int nblocks_max, int &nsx, int &nwork, int &blocks)
{
    nsx = (w + 127) / 128;
    nwork = nsx * ((h + kResChunk - 1) / kResChunk);
    blocks = std::min((nwork + kResWarps - 1) / kResWarps, nblocks_max);
}

cudaError_t launch_residual(const float *p, const float *b, int ld, int w, int h, const Reduce &red,
                            SolveState *state, int sweeps_here, double tol, cudaStream_t st, int stall_window)
{
    if (strip_ok(p, b, w, ld)) {
        int nsx, nwork, blocks;
        strip_grid(w, h, red.nblocks, nsx, nwork, blocks);
        k_residual_strip<<<blocks, kResWarps * 32, 0, st>>>(p, b, ld, w, h, nsx, nwork, red, state, sweeps_here, tol, 0,
                                                             stall_window);
        return launched();
    }
    k_residual<<<red.nblocks, 256, 0, st>>>(p, b, ld, w, h, red, state, sweeps_here, tol, stall_window);
    return launched();
}

cudaError_t launch_norms(const float *p, const float *b, int ld, int w, int h, const Reduce &red, cudaStream_t st)
{
    if (strip_ok(p, b, w, ld)) {
        int nsx, nwork, blocks;
        strip_grid(w, h, red.nblocks, nsx, nwork, blocks);
        k_residual_strip<<<blocks, kResWarps * 32, 0, st>>>(p, b, ld, w, h, nsx, nwork, red, nullptr, 0, 0.0, 1, 0);
        return launched();
    }
    k_norms<<<red.nblocks, 256, 0, st>>>(p, b, ld, w, h, red);
    return launched();
}

cudaError_t launch_project(const float *u, const float *v, const float *p, float *uo, float *vo, int ld, int w,
                           int h, float dt, cudaStream_t st, int bc)
{
    PFS_BC_DISPATCH(bc, k_project, grid2d(w, h), u, v, p, uo, vo, ld, w, h, dt);
    return launched();
}

cudaError_t launch_project_advect_image(const float *u, const float *v, const float *p, float *uo, float *vo,
                                        int ld, int w, int h, float dt, const float *img, float *imgo,
                                        size_t img_plane, int c, cudaStream_t st, int bc)
{
    PFS_BC_DISPATCH(bc, k_project_advect_image, grid2d(w, h), u, v, p, uo, vo, ld, w, h, dt, img, imgo, img_plane,
                    c);
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
                                       cudaStream_t st, int bc)
{
    float viw, vih, kx, ky;
    image_scales(iw, ih, vw, vh, dt, viw, vih, kx, ky);
    PFS_BC_DISPATCH(bc, k_advect_image_planar, grid2d(iw, ih), img, imgo, img_plane, ild, iw, ih, c, u, v, vld, vw, vh,
                    dt, viw, vih, kx, ky);
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

cudaError_t launch_split_vp(const float *vp, float *u, float *v, float *p, float *b, int ld, int w, int h,
                            cudaStream_t st)
{
    k_split_vp<<<grid2d(w, h), dim3(kBX, kBY), 0, st>>>(reinterpret_cast<const float4 *>(vp), u, v, p, b, ld, w, h);
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
