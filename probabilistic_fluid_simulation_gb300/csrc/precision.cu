// Precision forms of the timestep: velocity, image and the pressure
// correction stored in bf16 / fp16 / float32 and computed in FP32, with the
// pressure itself and its residual kept in FP64 (mixed-precision iterative
// refinement); and an all-FP64 form, the FP64 run of the same method used to
// measure every form's error.
//
// The method is the reference's (src/fluid.cpp:298-320) in the configuration
// viscosity 0 with an even diffusion count, where its buffer roles reduce to:
// advect the velocity; divergence of the advected velocity; Jacobi on the
// pressure from the previous step's final pressure; projection with the final
// pressure; image advection with the projected velocity.
//
// Iterative refinement keeps the method: with x the FP64 pressure and
// r = b - A x, m Jacobi sweeps on A e = r started from e = 0 give
// x + e = m Jacobi sweeps on A x = b started from x, because a Jacobi sweep is
// affine (x' = M x + D^-1 b). Only the rounding differs: x, r and the update
// x += e are FP64; the sweeps on e store e and r in 16 or 32 bits (r scaled
// by 1 / max|r| so it fills the 16-bit range) and compute in FP32.
//
// Start of each step's iteration: the previous final pressure (the
// reference), zero, or the warm-start network's prediction followed by
// damped passes x += (b - A x) / 8 and checked against the previous pressure.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "precision.h"
#include "reduce.cuh"
#include "storage.cuh"
#include "unet.h"

namespace pfs {
namespace {

// ---- arithmetic in the compute type: one rounding per operation ----
template <typename C>
struct Ar;
template <>
struct Ar<float> {
    __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ static float sub(float a, float b) { return __fsub_rn(a, b); }
    __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
    __device__ static float div(float a, float b) { return __fdiv_rn(a, b); }
    __device__ static float fmod_(float a, float b) { return fmodf(a, b); }
    __device__ static int trunc(float a) { return __float2int_rz(a); }
};
template <>
struct Ar<double> {
    __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
    __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
    __device__ static double div(double a, double b) { return __ddiv_rn(a, b); }
    __device__ static double fmod_(double a, double b) { return fmod(a, b); }
    __device__ static int trunc(double a) { return __double2int_rz(a); }
};

// Storage load/store in the compute type (double storage is only used with
// double compute).
template <typename T, typename C>
__device__ __forceinline__ C ldv(const T *p)
{
    if constexpr (std::is_same<T, double>::value) return (C)*p;
    else return (C)Store<T>::to_f(*p);
}
template <typename T, typename C>
__device__ __forceinline__ void stv(T *p, C v)
{
    if constexpr (std::is_same<T, double>::value) *p = (double)v;
    else *p = Store<T>::from_f((float)v);
}

template <typename C>
__device__ __forceinline__ C fmod_small_t(C x, C n)
{
    if (x >= n) return x == (C)2 * n ? (C)0 : Ar<C>::sub(x, n);
    if (x == -n) return -(C)0;
    return x;
}
// fmod(fmod(x, n) + n, n) (src/fluid.cpp:48-49), exact fast path as wrap_coord.
template <typename C>
__device__ __forceinline__ C wrap_t(C x, C n)
{
    if (x >= -n && x < (C)2 * n) return fmod_small_t(Ar<C>::add(fmod_small_t(x, n), n), n);
    return Ar<C>::fmod_(Ar<C>::add(Ar<C>::fmod_(x, n), n), n);
}

template <typename C>
__device__ __forceinline__ C bilerp_t(C sx, C sy, C f00, C f10, C f01, C f11)
{
    const C ox = Ar<C>::sub((C)1, sx), oy = Ar<C>::sub((C)1, sy);
    const C a = Ar<C>::mul(Ar<C>::mul(ox, oy), f00);
    const C b = Ar<C>::mul(Ar<C>::mul(sx, oy), f10);
    const C c = Ar<C>::mul(Ar<C>::mul(ox, sy), f01);
    const C d = Ar<C>::mul(Ar<C>::mul(sx, sy), f11);
    return Ar<C>::add(Ar<C>::add(Ar<C>::add(a, b), c), d);
}

template <typename C>
struct CornersT {
    int i0, i1, j0, j1;
    C sx, sy;
};

template <typename C>
__device__ __forceinline__ CornersT<C> backtrace_t(int i, int j, C kx, C ky, C u, C v, int w, int h)
{
    const C fw = (C)w, fh = (C)h;
    C xp = Ar<C>::sub((C)i, Ar<C>::div(Ar<C>::mul(kx, u), fw));
    C yp = Ar<C>::sub((C)j, Ar<C>::div(Ar<C>::mul(ky, v), fh));
    xp = wrap_t(xp, fw);
    yp = wrap_t(yp, fh);
    CornersT<C> c;
    c.i0 = min(max(Ar<C>::trunc(xp), 0), w - 1);
    c.j0 = min(max(Ar<C>::trunc(yp), 0), h - 1);
    c.i1 = (c.i0 + 1) % w;
    c.j1 = (c.j0 + 1) % h;
    c.sx = Ar<C>::sub(xp, (C)c.i0);
    c.sy = Ar<C>::sub(yp, (C)c.j0);
    return c;
}

__device__ __forceinline__ int wm_(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wp_(int i, int n) { return i + 1 == n ? 0 : i + 1; }

constexpr int kBX = 32, kBY = 8;
inline dim3 g2(int w, int h) { return dim3((w + kBX - 1) / kBX, (h + kBY - 1) / kBY); }

// src/fluid.cpp:24-70
template <typename T, typename C>
__global__ void k_lp_advect(const T *__restrict__ u, const T *__restrict__ v, T *__restrict__ uo, T *__restrict__ vo,
                            int ld, int w, int h, C dt)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t o = (size_t)j * ld + i;
    const CornersT<C> c = backtrace_t<C>(i, j, dt, dt, ldv<T, C>(u + o), ldv<T, C>(v + o), w, h);
    const size_t r0 = (size_t)c.j0 * ld, r1 = (size_t)c.j1 * ld;
    stv<T, C>(uo + o, bilerp_t<C>(c.sx, c.sy, ldv<T, C>(u + r0 + c.i0), ldv<T, C>(u + r0 + c.i1), ldv<T, C>(u + r1 + c.i0),
                                 ldv<T, C>(u + r1 + c.i1)));
    stv<T, C>(vo + o, bilerp_t<C>(c.sx, c.sy, ldv<T, C>(v + r0 + c.i0), ldv<T, C>(v + r0 + c.i1), ldv<T, C>(v + r1 + c.i0),
                                 ldv<T, C>(v + r1 + c.i1)));
}

// src/fluid.cpp:218-237; also sum b^2 (slot 1).
template <typename T, typename B, typename C>
__global__ void __launch_bounds__(256) k_lp_divergence(const T *__restrict__ u, const T *__restrict__ v,
                                                       B *__restrict__ b, int ld, int w, int h, C gamma, Reduce red)
{
    FFAcc accf;
    double accd = 0.0;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        const size_t r = (size_t)j * ld, rm = (size_t)wm_(j, h) * ld, rp = (size_t)wp_(j, h) * ld;
        for (int i = threadIdx.x; i < w; i += blockDim.x) {
            const C du = Ar<C>::sub(ldv<T, C>(u + r + wp_(i, w)), ldv<T, C>(u + r + wm_(i, w)));
            const C dv = Ar<C>::sub(ldv<T, C>(v + rp + i), ldv<T, C>(v + rm + i));
            const C bv = Ar<C>::mul(gamma, Ar<C>::add(du, dv));
            b[r + i] = (B)bv;
            if constexpr (std::is_same<C, double>::value) accd = __fma_rn(bv, bv, accd);
            else acc_square(accf, bv);
        }
    }
    reduce_blocks(std::is_same<C, double>::value ? accd : accf.value(), red, 1);
}

// The pressure of the refined forms (bf16, fp16, float32 storage) is an
// unevaluated pair of floats hi + lo, about 48 significant bits, kept in the
// 8 bytes per cell an FP64 plane takes (hi in the first half of the plane's
// memory, lo in the second), so the refinement runs on the FP32 pipe with
// error-free transformations instead of on GB300's FP64 pipe (which held the
// FP64 version of this pass at 80% busy and a sixth of the HBM rate). The FP64
// form keeps FP64 planes.
__device__ __forceinline__ FF ff_add(FF x, float a, float a_lo)
{
    const FF s = two_sum(x.hi, a);
    return two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, a_lo)));
}

// r = b + xL + xR + xT + xB - 4 xc for pairs: the hi parts summed with their
// exact rounding errors (TwoSum), the errors and lo parts summed in float.
__device__ __forceinline__ FF ff_residual(float b, FF l, FF r, FF t, FF bo, FF c)
{
    FF s = two_sum(b, l.hi);
    float e = __fadd_rn(s.lo, l.lo);
    s = two_sum(s.hi, r.hi);
    e = __fadd_rn(e, __fadd_rn(s.lo, r.lo));
    s = two_sum(s.hi, t.hi);
    e = __fadd_rn(e, __fadd_rn(s.lo, t.lo));
    s = two_sum(s.hi, bo.hi);
    e = __fadd_rn(e, __fadd_rn(s.lo, bo.lo));
    s = two_sum(s.hi, __fmul_rn(-4.0f, c.hi));  // -4 hi is exact
    e = __fadd_rn(e, __fadd_rn(s.lo, __fmul_rn(-4.0f, c.lo)));
    return two_sum(s.hi, e);
}

// Refinement: x_out = x_in + e / scale (e may be null: no correction yet);
// r = b - A x_out per cell, stored as float; sum r^2 (slot 0) and max |r|
// (as float bits, atomicMax). A block stages x_in + e / scale for a 32 x 32
// tile and its one-cell halo (periodic wrap) in shared memory, so each
// corrected pressure is formed once.
constexpr int kRefTile = 32;
template <typename T>
__global__ void __launch_bounds__(256) k_lp_refine(const float *__restrict__ xh_in, const float *__restrict__ xl_in,
                                                   const T *__restrict__ e, const double *__restrict__ escale,
                                                   const float *__restrict__ b, float *__restrict__ xh_out,
                                                   float *__restrict__ xl_out, float *__restrict__ rout, int ld, int w,
                                                   int h, Reduce red, unsigned *maxabs)
{
    constexpr int TS = kRefTile, SP = kRefTile + 2;
    __shared__ float2 xs[SP][SP];
    // 1 / scale as a float pair (three FP64 operations per thread)
    float ih = 0.0f, il = 0.0f;
    if (e) {
        const double inv = 1.0 / *escale;
        ih = (float)inv;
        il = (float)(inv - (double)ih);
    }
    const int tx = (w + TS - 1) / TS, ntiles = tx * ((h + TS - 1) / TS);
    const int lane = threadIdx.x & 31;
    FFAcc acc;
    unsigned mx = 0u;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int i0 = (t % tx) * TS, j0 = (t / tx) * TS;
        const int iw = min(TS, w - i0), jh = min(TS, h - j0);
        // columns i0-1 .. i0+iw and rows j0-1 .. j0+jh, wrapped: all in [0, w) x [0, h) for any w, h >= 1
        for (int k = threadIdx.x; k < SP * SP; k += blockDim.x) {
            const int a = k % SP, c = k / SP;
            if (a > iw + 1 || c > jh + 1) continue;
            int gi = i0 - 1 + a, gj = j0 - 1 + c;
            gi = gi < 0 ? gi + w : (gi >= w ? gi - w : gi);
            gj = gj < 0 ? gj + h : (gj >= h ? gj - h : gj);
            const size_t o = (size_t)gj * ld + gi;
            FF v{xh_in[o], xl_in[o]};
            if (e) {  // + e * (ih + il): the product and its rounding error (FMA), then added to the pair
                const float ev = Store<T>::to_f(e[o]);
                const float p = __fmul_rn(ev, ih);
                v = ff_add(v, p, __fadd_rn(__fmaf_rn(ev, ih, -p), __fmul_rn(ev, il)));
            }
            xs[c][a] = make_float2(v.hi, v.lo);
        }
        __syncthreads();
        if (lane < iw) {
            for (int c = threadIdx.x >> 5; c < jh; c += blockDim.x >> 5) {
                const size_t o = (size_t)(j0 + c) * ld + i0 + lane;
                const float2 xc = xs[c + 1][lane + 1], xl = xs[c + 1][lane], xr = xs[c + 1][lane + 2];
                const float2 xt = xs[c][lane + 1], xb = xs[c + 2][lane + 1];
                const FF q = ff_residual(b[o], FF{xl.x, xl.y}, FF{xr.x, xr.y}, FF{xt.x, xt.y}, FF{xb.x, xb.y},
                                         FF{xc.x, xc.y});
                xh_out[o] = xc.x;
                xl_out[o] = xc.y;
                rout[o] = q.hi;
                mx = max(mx, __float_as_uint(fabsf(q.hi)));
                const float sq = __fmul_rn(q.hi, q.hi);
                acc.add(sq, __fadd_rn(__fmaf_rn(q.hi, q.hi, -sq), __fmul_rn(__fmul_rn(2.0f, q.hi), q.lo)));
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0 && mx) atomicMax(maxabs, mx);
    reduce_blocks(acc.value(), red, 0);
}

// Damped pass on a predicted start, pairs: x_out = x + (b - A x) / 8 (the
// Jacobi update with weight 1/2; gain (1 + l) / 2 on a mode of Jacobi
// eigenvalue l).
__global__ void k_ff_damp(const float *__restrict__ xh, const float *__restrict__ xl, const float *__restrict__ b,
                          float *__restrict__ xho, float *__restrict__ xlo, int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t r = (size_t)j * ld;
    auto at = [&](size_t o) { return FF{xh[o], xl[o]}; };
    const FF c = at(r + i);
    const FF q = ff_residual(b[r + i], at(r + wm_(i, w)), at(r + wp_(i, w)), at((size_t)wm_(j, h) * ld + i),
                             at((size_t)wp_(j, h) * ld + i), c);
    const FF x = ff_add(c, __fmul_rn(q.hi, 0.125f), __fmul_rn(q.lo, 0.125f));
    xho[r + i] = x.hi;
    xlo[r + i] = x.lo;
}

// x += d (a predicted correction), pairs.
__global__ void k_ff_add(float *__restrict__ xh, float *__restrict__ xl, const float *__restrict__ d, size_t n)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const FF x = ff_add(FF{xh[k], xl[k]}, d[k], 0.0f);
        xh[k] = x.hi;
        xl[k] = x.lo;
    }
}

// r (float) -> 16-bit right-hand side scaled by 1 / max|r|; records the scale.
template <typename T>
__global__ void k_lp_scale(const float *__restrict__ r, T *__restrict__ rt, size_t n, const unsigned *maxabs,
                           double *escale)
{
    const float m = __uint_as_float(*maxabs);
    const float s = m > 0.0f ? 1.0f / m : 1.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0) *escale = (double)s;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        rt[k] = Store<T>::from_f(r[k] * s);
}

// The float32 form's right-hand side: rt = r / max|r| over the grid's cells
// (padding columns get 0) and sum rt^2 into red.result[1], the norm the fused
// residual checks of the correction solve divide by.
__global__ void __launch_bounds__(256) k_lp_scale_f32(const float *__restrict__ r, float *__restrict__ rt, int ld,
                                                      int w, int h, const unsigned *maxabs, double *escale, Reduce red)
{
    const float m = __uint_as_float(*maxabs);
    const float s = m > 0.0f ? 1.0f / m : 1.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0) *escale = (double)s;
    FFAcc acc;
    for (int j = blockIdx.x; j < h; j += gridDim.x)
        for (int i = threadIdx.x; i < ld; i += blockDim.x) {
            const size_t k = (size_t)j * ld + i;
            const float v = i < w ? r[k] * s : 0.0f;
            rt[k] = v;
            acc_square(acc, v);
        }
    reduce_blocks(acc.value(), red, 1);
}

// FP64 form: one Jacobi sweep (src/fluid.cpp:239-257 in double). The
// division by 4 is a multiplication by 0.25: both are the correctly rounded
// value of the same exact quotient (4 is a power of two), so the bits are
// those of the division, without FP64 division's iteration.
__global__ void k_f64_sweep(const double *__restrict__ pin, const double *__restrict__ b, double *__restrict__ pout,
                            int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t r = (size_t)j * ld;
    const double s = __dadd_rn(__dadd_rn(__dadd_rn(pin[r + wm_(i, w)], pin[r + wp_(i, w)]),
                                         pin[(size_t)wm_(j, h) * ld + i]),
                               pin[(size_t)wp_(j, h) * ld + i]);
    pout[r + i] = __dmul_rn(__dadd_rn(s, b[r + i]), 0.25);
}

// FP64 form: residual exactly as the oracle evaluates it, sum r^2 (slot 0).
__global__ void __launch_bounds__(256) k_f64_residual(const double *__restrict__ p, const double *__restrict__ b,
                                                      int ld, int w, int h, Reduce red)
{
    double acc = 0.0;
    for (int j = blockIdx.x; j < h; j += gridDim.x) {
        const size_t r = (size_t)j * ld, rm = (size_t)wm_(j, h) * ld, rp = (size_t)wp_(j, h) * ld;
        for (int i = threadIdx.x; i < w; i += blockDim.x) {
            double q = __dadd_rn(b[r + i], p[r + wm_(i, w)]);
            q = __dadd_rn(q, p[r + wp_(i, w)]);
            q = __dadd_rn(q, p[rm + i]);
            q = __dadd_rn(q, p[rp + i]);
            q = __dsub_rn(q, __dmul_rn(4.0, p[r + i]));
            acc = __fma_rn(q, q, acc);
        }
    }
    reduce_blocks(acc, red, 0);
}

// The pressure as the projection reads it: an FP64 plane (the FP64 form) or
// the refined forms' float pair (hi, lo), 8 bytes per cell either way.
struct XPlane {
    const double *d;   // FP64 plane, or null
    const float *hi;   // pair planes when d is null
    const float *lo;
    // x_a - x_b, rounded once to C
    template <typename C>
    __device__ __forceinline__ C diff(size_t a, size_t b) const
    {
        if (d) return (C)(d[a] - d[b]);
        const FF s = two_sum(hi[a], -hi[b]);  // exact difference of the hi parts
        return (C)__fadd_rn(s.hi, __fadd_rn(s.lo, __fsub_rn(lo[a], lo[b])));
    }
};

// Projection (src/fluid.cpp:269-296) with the refined pressure: the gradient
// is formed in C from the pressure values, ((pR - pL) * dt) / 2.
template <typename C>
__device__ __forceinline__ void lp_grad(const XPlane &x, int ld, int w, int h, C dt, int i, int j, C &gx, C &gy)
{
    const size_t r = (size_t)j * ld;
    const C dx = x.diff<C>(r + wp_(i, w), r + wm_(i, w));
    const C dy = x.diff<C>((size_t)wp_(j, h) * ld + i, (size_t)wm_(j, h) * ld + i);
    gx = Ar<C>::div(Ar<C>::mul(dx, dt), (C)2);
    gy = Ar<C>::div(Ar<C>::mul(dy, dt), (C)2);
}

template <typename T, typename C>
__global__ void k_lp_project(const T *__restrict__ ua, const T *__restrict__ va, XPlane x, T *__restrict__ u,
                             T *__restrict__ v, int ld, int w, int h, C dt)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    C gx, gy;
    lp_grad<C>(x, ld, w, h, dt, i, j, gx, gy);
    const size_t o = (size_t)j * ld + i;
    stv<T, C>(u + o, Ar<C>::sub(ldv<T, C>(ua + o), gx));
    stv<T, C>(v + o, Ar<C>::sub(ldv<T, C>(va + o), gy));
}

// src/fluid.cpp:72-127 on planar T fields.
template <typename T, typename C>
__global__ void k_lp_advect_image(const T *__restrict__ img, T *__restrict__ imgo, size_t plane, int ild, int iw,
                                  int ih, int c, const T *__restrict__ u, const T *__restrict__ v, int vld, int vw,
                                  int vh, C viw, C vih, C kx, C ky)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= iw || j >= ih) return;
    const int vi = min(Ar<C>::trunc(Ar<C>::mul((C)i, viw)), vw - 1);
    const int vj = min(Ar<C>::trunc(Ar<C>::mul((C)j, vih)), vh - 1);
    const size_t vo = (size_t)vj * vld + vi;
    const CornersT<C> k = backtrace_t<C>(i, j, kx, ky, ldv<T, C>(u + vo), ldv<T, C>(v + vo), iw, ih);
    const size_t r0 = (size_t)k.j0 * ild, r1 = (size_t)k.j1 * ild, o = (size_t)j * ild + i;
    for (int ch = 0; ch < c; ++ch) {
        const T *s = img + ch * plane;
        stv<T, C>(imgo + ch * plane + o, bilerp_t<C>(k.sx, k.sy, ldv<T, C>(s + r0 + k.i0), ldv<T, C>(s + r0 + k.i1),
                                                    ldv<T, C>(s + r1 + k.i0), ldv<T, C>(s + r1 + k.i1)));
    }
}

// interleaved float32 (h, w, nch) channel k -> planar T / double
template <typename T>
__global__ void k_lp_split(const float *__restrict__ buf, int k, int nch, T *__restrict__ plane, int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const float x = buf[((size_t)j * w + i) * nch + k];
    if constexpr (std::is_same<T, double>::value) plane[(size_t)j * ld + i] = (double)x;
    else plane[(size_t)j * ld + i] = Store<T>::from_f(x);
}

// planar T / double -> interleaved O (float or double) channel k
template <typename T, typename O>
__global__ void k_lp_merge(O *__restrict__ buf, int k, int nch, const T *__restrict__ plane, int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    double x;
    if constexpr (std::is_same<T, double>::value) x = plane[(size_t)j * ld + i];
    else if constexpr (std::is_same<T, float>::value) x = (double)plane[(size_t)j * ld + i];
    else x = (double)Store<T>::to_f(plane[(size_t)j * ld + i]);
    buf[((size_t)j * w + i) * nch + k] = (O)x;
}

// pair planes -> interleaved O (float or double) channel k: the pair's value rounded once
template <typename O>
__global__ void k_ff_merge(O *__restrict__ buf, int k, int nch, const float *__restrict__ xh, const float *__restrict__ xl,
                           int ld, int w, int h)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    if (i >= w || j >= h) return;
    const size_t o = (size_t)j * ld + i;
    buf[((size_t)j * w + i) * nch + k] = (O)((double)xh[o] + (double)xl[o]);
}

inline int rup(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

// =============================================================================================
// Host side

struct LpState {
    int form = 0;  // PFS_PREC_*
    int w = 0, h = 0, ld = 0, iw = 0, ih = 0, ic = 0, ild = 0;
    size_t plane = 0, iplane = 0;
    size_t tbytes = 0;  // bytes per element of the velocity / image / correction storage
    // velocity (T) current and advected; image (T) x2; pressure x (double) x2;
    // b (float, or double in the FP64 form); r (float) and 16-bit r, e x2
    void *u = nullptr, *v = nullptr, *ua = nullptr, *va = nullptr, *img[2] = {nullptr, nullptr};
    double *x[2] = {nullptr, nullptr};
    double *xback = nullptr;  // the previous pressure, kept while a predicted start is tried
    float *pred = nullptr;    // the network's pressure (or correction) for a predicted start
    void *b = nullptr;
    float *r = nullptr;
    void *rt = nullptr, *e[2] = {nullptr, nullptr};
    int xcur = 0, icur = 0;
    void *mem = nullptr;
    double *rmem = nullptr;
    unsigned *maxabs = nullptr;
    double *escale = nullptr;
    double *hres = nullptr;    // pinned and mapped: written by launch_copy_small
    double *hres_d = nullptr;  // its device alias
    Reduce red{};
    void *stage = nullptr;
    size_t stage_bytes = 0;
    // F32R: the correction solve's fused residual checks (their own partials and
    // result pair: result[1] holds sum rt^2) and its device / mapped solve state
    Reduce red_in{};
    double *in_mem = nullptr;
    SolveState *dstate = nullptr;
    SolveState *hstate = nullptr;  // pinned and mapped
    SolveState *hstate_d = nullptr;
};

namespace {

int lp_fail(int code, const char *msg) { return record_error(code, msg); }

#define LCK(x)                                                     \
    do {                                                           \
        cudaError_t e_ = (x);                                      \
        if (e_ != cudaSuccess) return lp_fail(PFS_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

// The two float planes of a refined form's pressure kept in FP64-plane memory.
inline float *pair_hi(const LpState &s, double *x) { return reinterpret_cast<float *>(x); }
inline float *pair_lo(const LpState &s, double *x) { return reinterpret_cast<float *>(x) + s.plane; }

template <typename T, typename C>
int lp_velocity_and_image(LpState &s, const LpParams &p, cudaStream_t st, double *xfinal)
{
    const int w = s.w, h = s.h, ld = s.ld;
    T *u = (T *)s.u, *v = (T *)s.v, *ua = (T *)s.ua, *va = (T *)s.va;
    XPlane xp;
    if constexpr (std::is_same<T, double>::value) xp = {xfinal, nullptr, nullptr};
    else xp = {nullptr, pair_hi(s, xfinal), pair_lo(s, xfinal)};
    k_lp_project<T, C><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(ua, va, xp, u, v, ld, w, h, (C)p.dt);
    LCK(launched());
    if (s.ic > 0) {
        const C viw = (C)w / (C)s.iw, vih = (C)h / (C)s.ih;
        const C kx = (C)p.dt / viw, ky = (C)p.dt / vih;
        k_lp_advect_image<T, C><<<g2(s.iw, s.ih), dim3(kBX, kBY), 0, st>>>(
            (T *)s.img[s.icur], (T *)s.img[1 - s.icur], s.iplane, s.ild, s.iw, s.ih, s.ic, u, v, ld, w, h, viw, vih, kx,
            ky);
        LCK(launched());
        s.icur = 1 - s.icur;
    }
    return PFS_OK;
}

double rel_of(double rr, double bb) { return bb > 0.0 ? std::sqrt(rr) / std::sqrt(bb) : std::sqrt(rr); }

// r = b - A x for the refined forms (no correction): x copied to xo, r to s.r,
// relative residual returned (blocking).
template <typename T>
int lp_residual(LpState &s, const double *x, double *xo, cudaStream_t st, double &rel)
{
    LCK(launch_zero_small(s.maxabs, sizeof(unsigned), st));
    k_lp_refine<T><<<s.red.nblocks, 256, 0, st>>>(pair_hi(s, const_cast<double *>(x)), pair_lo(s, const_cast<double *>(x)),
                                                   (const T *)nullptr, s.escale, (const float *)s.b, pair_hi(s, xo),
                                                   pair_lo(s, xo), s.r, s.ld, s.w, s.h, s.red, s.maxabs);
    LCK(launched());
    LCK(launch_copy_small(s.red.result, s.hres_d, 2 * sizeof(double), st));
    LCK(cudaStreamSynchronize(st));
    rel = rel_of(s.hres[0], s.hres[1]);
    return PFS_OK;
}

// Predicted start: the network's pressure for b (on the grid coarsened
// p.coarsen times), widened to FP64; then, for each further pass, the
// network's correction for the residual r = b - A x (A is linear, so the
// correction solves A e = r as the pressure solves A p = b) added in FP64.
// Every pass is followed by PFS_START_DAMP_PASSES damped passes. The start is
// kept unless its residual is above PFS_START_SLACK times the previous
// pressure's or not finite; then the previous pressure is (PFS_START_FALLBACK). Afterwards x[xcur] holds the start and
// s.xback the previous pressure.
template <typename T>
int lp_network_start(LpState &s, const LpParams &p, cudaStream_t st, LpOut &o)
{
    if (!s.xback) LCK(cudaMalloc(&s.xback, s.plane * sizeof(double)));
    if (!s.pred) LCK(cudaMalloc(&s.pred, s.plane * sizeof(float)));
    LCK(cudaMemcpyAsync(s.xback, s.x[s.xcur], s.plane * sizeof(double), cudaMemcpyDeviceToDevice, st));
    double rel_net = 0.0, rel_plain = 0.0;
    o.start_passes = 0;
    for (int pass = 0; pass < p.passes; ++pass) {
        const float *rhs = pass == 0 ? (const float *)s.b : s.r;  // s.r: residual of x (last lp_residual)
        const int rc = unet::predict_coarse(p.net, rhs, s.ld, s.pred, s.ld, s.h, s.w, p.coarsen, st);
        if (rc != PFS_OK) return rc;
        if (pass == 0) {
            LCK(cudaMemcpyAsync(pair_hi(s, s.x[s.xcur]), s.pred, s.plane * sizeof(float), cudaMemcpyDeviceToDevice, st));
            LCK(cudaMemsetAsync(pair_lo(s, s.x[s.xcur]), 0, s.plane * sizeof(float), st));
        } else {
            k_ff_add<<<reduce_grid(), 256, 0, st>>>(pair_hi(s, s.x[s.xcur]), pair_lo(s, s.x[s.xcur]), s.pred, s.plane);
            LCK(launched());
        }
        for (int k = 0; k < PFS_START_DAMP_PASSES; ++k) {
            k_ff_damp<<<g2(s.w, s.h), dim3(kBX, kBY), 0, st>>>(pair_hi(s, s.x[s.xcur]), pair_lo(s, s.x[s.xcur]),
                                                                (const float *)s.b, pair_hi(s, s.x[1 - s.xcur]),
                                                                pair_lo(s, s.x[1 - s.xcur]), s.ld, s.w, s.h);
            LCK(launched());
            s.xcur = 1 - s.xcur;
        }
        o.start_passes += PFS_START_DAMP_PASSES;
        const int e = lp_residual<T>(s, s.x[s.xcur], s.x[1 - s.xcur], st, rel_net);
        if (e != PFS_OK) return e;
    }
    const int e = lp_residual<T>(s, s.xback, s.x[1 - s.xcur], st, rel_plain);  // other slot: previous
    if (e != PFS_OK) return e;
    if (rel_net <= PFS_START_SLACK * rel_plain) {
        o.start_kind = PFS_START_NETWORK;
        o.rel_start = rel_net;
    } else {  // a broken prediction (or not finite): keep the plain start
        s.xcur = 1 - s.xcur;
        o.start_kind = PFS_START_FALLBACK;
        o.rel_start = rel_plain;
    }
    return PFS_OK;
}

template <typename T>
cudaError_t lp_sweeps(const T *in, const T *rhs, T *out, int ld, int w, int h, int L, int chunk, cudaStream_t st)
{
    if constexpr (std::is_same<T, __nv_bfloat16>::value)
        return launch_sweep_stream_bf16(in, rhs, out, ld, w, h, L, chunk, st);
    else if constexpr (std::is_same<T, __half>::value)
        return launch_sweep_stream_f16(in, rhs, out, ld, w, h, L, chunk, st);
    else
        return launch_sweep_stream(in, rhs, out, nullptr, ld, w, h, L, 8, chunk, nullptr, st);
}

// Correction solve of the float32 refined form in residual mode: Jacobi
// sweeps on A e = rt from e = 0 with the plain form's fused sweep kernel, the
// last launch of every `every` sweeps evaluating the correction's exact
// residual ||rt - A e|| / ||rt|| on the device (as the plain form's solve
// does), until it is at most tol_in, or (window > 0) it has not fallen 1%
// within `window` sweeps, or `budget` sweeps have run. The host reads the state between batches of check
// intervals (1, 2, 4, ... 64); launches after the deciding check return at
// once. Returns the sweeps done, the plane holding e and the state's done
// code (0: budget spent, 1: converged, 2: stalled).
int lp_correction_f32(LpState &s, const LpParams &p, double tol_in, int budget, int window, cudaStream_t st,
                      int &sweeps, const float *&eout, int &done_code)
{
    const int every = p.check_every > 0 ? p.check_every : 32;
    const int L = std::max(1, std::min(p.levels, 8));
    const int chunk = std::max(p.chunk, 16);
    const float *rt = (const float *)s.rt;
    float *e[2] = {(float *)s.e[0], (float *)s.e[1]};
    LCK(launch_zero_small(s.dstate, sizeof(SolveState), st));
    const int *done = &s.dstate->done;
    struct Mark {
        int sweeps, plane;
    };
    Mark marks[64];
    int nmarks = 0, S = 0, cur = -1, batch = 1, in_batch = 0;
    bool finished = budget <= 0;
    while (!finished) {
        const int stop = std::min(budget, (S / every + 1) * every);
        while (S < stop) {
            int n = std::min(L, stop - S);
            bool last = (S + n == stop);
            if (last && n == 8) {  // the check launch fuses at most 7 levels: 8 = 4 + 4
                n = 4;
                last = false;
            }
            const int out = cur == 0 ? 1 : 0;
            const float *in = cur < 0 ? nullptr : e[cur];  // null: the zero start
            if (last)
                LCK(launch_sweep_stream_check(in, rt, e[out], nullptr, s.ld, s.w, s.h, n, chunk, s.red_in, s.dstate,
                                              S + n, tol_in, done, st, window));
            else
                LCK(launch_sweep_stream(in, rt, e[out], nullptr, s.ld, s.w, s.h, n, 8, chunk, done, st));
            cur = out;
            S += n;
        }
        marks[nmarks++] = {S, cur};
        if (++in_batch == batch || S >= budget || nmarks == 64) {
            LCK(launch_copy_small(s.dstate, s.hstate_d, sizeof(SolveState), st));
            LCK(cudaStreamSynchronize(st));
            if (s.hstate->done || S >= budget) {
                finished = true;
            } else {
                nmarks = 0;  // the deciding check can only be in a later batch
                in_batch = 0;
                batch = std::min(batch * 2, 64);
            }
        }
    }
    const SolveState hs = *s.hstate;
    done_code = hs.done;
    int plane = cur;
    if (hs.done) {
        int k = nmarks - 1;
        while (k > 0 && marks[k].sweeps != hs.sweeps) --k;
        if (nmarks == 0 || marks[k].sweeps != hs.sweeps) return lp_fail(PFS_ERR_CUDA, "lost the deciding check");
        S = hs.sweeps;
        plane = marks[k].plane;
    }
    sweeps = S;
    eout = (S > 0 && plane >= 0) ? e[plane] : nullptr;
    return PFS_OK;
}

// One step of a refined form (bf16, fp16 or float32 storage).
template <typename T>
int lp_step_ir(LpState &s, const LpParams &p, cudaStream_t st, LpOut &o)
{
    const int w = s.w, h = s.h, ld = s.ld;
    k_lp_advect<T, float><<<g2(w, h), dim3(kBX, kBY), 0, st>>>((T *)s.u, (T *)s.v, (T *)s.ua, (T *)s.va, ld, w, h,
                                                                p.dt);
    LCK(launched());
    const float gamma = (float)(-1.0 / (double)p.dt);
    k_lp_divergence<T, float, float><<<s.red.nblocks, 256, 0, st>>>((T *)s.ua, (T *)s.va, (float *)s.b, ld, w, h,
                                                                    gamma, s.red);
    LCK(launched());
    o.start_kind = p.start_mode;
    if (p.start_mode == PFS_START_ZERO) {
        LCK(cudaMemsetAsync(s.x[s.xcur], 0, s.plane * sizeof(double), st));
    } else if (p.start_mode == PFS_START_NETWORK) {
        const int rc = lp_network_start<T>(s, p, st, o);
        if (rc != PFS_OK) return rc;
    }
    const int m = p.check_every > 0 ? p.check_every : 32;  // sweeps between refinements
    const bool resid = p.tol > 0.0;
    // predicted start: if the residual stops falling between refinements, the previous pressure takes over
    const bool watch = resid && o.start_kind == PFS_START_NETWORK;
    double last_rel = o.rel_start;
    int S = 0;
    T *ecur = nullptr;  // correction of the last inner solve (null before the first)
    bool stalled_in = false;  // the last correction solve ran its whole interval without converging
    double best_rel = 0.0;    // lowest residual of the 16-bit forms' refinements so far
    int best_sweeps = 0;
    o.checks = 0;
    // The float32 form in residual mode filters each correction before adding
    // it: the Jacobi iteration multiplies the checkerboard mode of an error by
    // -1 every sweep and the modes near it by almost -1, so the rounding noise
    // a float32 correction picks up in them over its thousands of sweeps would
    // never be damped by later sweeps (in exact arithmetic neither b nor the
    // iterates carry these modes: the central-difference divergence has no
    // checkerboard component). Unfiltered, that noise held the residual near
    // 2.6e-5 at 2048^2. PFS_START_DAMP_PASSES damped passes e += (rt - A e) / 8
    // on the correction remove it (gain (1 + mu) / 2 on a mode of Jacobi
    // eigenvalue mu: 0 on the checkerboard, about 1 on the smooth modes the
    // iteration is working on), in float32 at the rate of a sweep. (The same
    // passes in FP64 on x after the update cost 3 ms per capped 4096^2 step.)
    for (;;) {
        // x_new = x + e/scale; r = b - A x_new (FP64); |r| stats
        LCK(launch_zero_small(s.maxabs, sizeof(unsigned), st));
        k_lp_refine<T><<<s.red.nblocks, 256, 0, st>>>(pair_hi(s, s.x[s.xcur]), pair_lo(s, s.x[s.xcur]), ecur, s.escale,
                                                       (const float *)s.b, pair_hi(s, s.x[1 - s.xcur]),
                                                       pair_lo(s, s.x[1 - s.xcur]), s.r, ld, w, h, s.red, s.maxabs);
        LCK(launched());
        s.xcur = 1 - s.xcur;
        LCK(launch_copy_small(s.red.result, s.hres_d, 2 * sizeof(double), st));
        LCK(cudaStreamSynchronize(st));
        o.checks++;
        o.rel = rel_of(s.hres[0], s.hres[1]);
        o.bnorm = std::sqrt(s.hres[1]);
        if ((resid && o.rel <= p.tol) || S >= p.max_iters) break;
        if (watch && ecur && o.start_kind == PFS_START_NETWORK && !(o.rel < last_rel)) {
            LCK(cudaMemcpyAsync(s.x[s.xcur], s.xback, s.plane * sizeof(double), cudaMemcpyDeviceToDevice, st));
            o.start_kind = PFS_START_FALLBACK;
            ecur = nullptr;  // next pass: residual of the previous pressure, no correction
            continue;
        }
        if constexpr (std::is_same<T, float>::value) {
            if (resid) {
                // a correction solve that ran its whole interval must have bought a 1% fall
                if (stalled_in && !(o.rel < kStallGain * last_rel)) {
                    o.stalled = true;
                    break;
                }
                last_rel = o.rel;
                const double rn = std::sqrt(s.hres[0]), bn = std::sqrt(s.hres[1]);
                // the correction's residual relative to its own right-hand side that
                // makes the pressure's relative residual tol (the scaled float32
                // right-hand side carries r to a relative 2^-24)
                const double tol_in = rn > 0.0 ? 0.999 * p.tol * bn / rn : 0.0;
                k_lp_scale_f32<<<reduce_grid(), 256, 0, st>>>(s.r, (float *)s.rt, ld, w, h, s.maxabs, s.escale,
                                                               s.red_in);
                LCK(launched());
                const int every = p.check_every > 0 ? p.check_every : 32;
                const int interval = f32r_refine_interval(std::max(w, h), every);
                int n = 0, code = 0;
                const float *eo = nullptr;
                const int rc = lp_correction_f32(s, p, tol_in, std::min(interval, p.max_iters - S), 0, st, n, eo, code);
                if (rc != PFS_OK) return rc;
                if (eo) {  // the filter: an even number of passes through the other plane ends back in eo
                    float *ea = const_cast<float *>(eo);
                    float *eb = (ea == (float *)s.e[0]) ? (float *)s.e[1] : (float *)s.e[0];
                    for (int k = 0; k < PFS_START_DAMP_PASSES; ++k)
                        LCK(launch_damp(k % 2 ? eb : ea, (const float *)s.rt, k % 2 ? ea : eb, ld, w, h, st));
                }
                stalled_in = code == 0 && n == interval;
                ecur = (T *)const_cast<float *>(eo);
                S += n;
                continue;
            }
        }
        last_rel = o.rel;
        // the 16-bit forms: stop once the refinements stop lowering the residual (their rounding floor)
        if (resid && p.stall_window > 0) {
            if (best_rel == 0.0 || o.rel < kStallGain * best_rel) {
                best_rel = o.rel;
                best_sweeps = S;
            } else if (S - best_sweeps >= p.stall_window) {
                o.stalled = true;
                break;
            }
        }
        // inner solve: n sweeps on A e = r from e = 0
        const int n = std::min(m, p.max_iters - S);
        k_lp_scale<T><<<s.red.nblocks, 256, 0, st>>>(s.r, (T *)s.rt, s.plane, s.maxabs, s.escale);
        LCK(launched());
        int done = 0, cur = -1;
        while (done < n) {
            const int L = std::min(p.levels, n - done);
            const int out = (cur == 0) ? 1 : 0;
            const T *in = cur < 0 ? nullptr : (const T *)s.e[cur];
            LCK(lp_sweeps<T>(in, (const T *)s.rt, (T *)s.e[out], ld, w, h, L, p.chunk, st));
            cur = out;
            done += L;
        }
        ecur = (T *)s.e[cur];
        S += n;
    }
    o.sweeps = S;
    o.capped = p.tol > 0.0 && !(o.rel <= p.tol) && !o.stalled;
    return lp_velocity_and_image<T, float>(s, p, st, s.x[s.xcur]);
}

// One step of the FP64 form: plain Jacobi on x in FP64, checks every m sweeps.
int lp_step64(LpState &s, const LpParams &p, cudaStream_t st, LpOut &o)
{
    const int w = s.w, h = s.h, ld = s.ld;
    const double dt = (double)p.dt;
    k_lp_advect<double, double><<<g2(w, h), dim3(kBX, kBY), 0, st>>>((double *)s.u, (double *)s.v, (double *)s.ua,
                                                                      (double *)s.va, ld, w, h, dt);
    LCK(launched());
    const double gamma = -1.0 / dt;
    k_lp_divergence<double, double, double><<<s.red.nblocks, 256, 0, st>>>((double *)s.ua, (double *)s.va,
                                                                           (double *)s.b, ld, w, h, gamma, s.red);
    LCK(launched());
    o.start_kind = p.start_mode;
    if (p.start_mode == PFS_START_ZERO) LCK(cudaMemsetAsync(s.x[s.xcur], 0, s.plane * sizeof(double), st));
    const bool resid = p.tol > 0.0;
    int S = 0;
    o.checks = 0;
    while (S < p.max_iters) {
        int stop = p.max_iters;
        if (resid && p.check_every > 0) stop = std::min(p.max_iters, (S / p.check_every + 1) * p.check_every);
        for (; S < stop; ++S) {
            k_f64_sweep<<<g2(w, h), dim3(kBX, kBY), 0, st>>>(s.x[s.xcur], (double *)s.b, s.x[1 - s.xcur], ld, w, h);
            LCK(launched());
            s.xcur = 1 - s.xcur;
        }
        if (!resid) break;
        k_f64_residual<<<s.red.nblocks, 256, 0, st>>>(s.x[s.xcur], (double *)s.b, ld, w, h, s.red);
        LCK(launched());
        LCK(launch_copy_small(s.red.result, s.hres_d, 2 * sizeof(double), st));
        LCK(cudaStreamSynchronize(st));
        o.checks++;
        o.rel = rel_of(s.hres[0], s.hres[1]);
        o.bnorm = std::sqrt(s.hres[1]);
        if (o.rel <= p.tol) break;
    }
    o.sweeps = S;
    o.capped = resid && S == p.max_iters && !(o.rel <= p.tol);
    return lp_velocity_and_image<double, double>(s, p, st, s.x[s.xcur]);
}

template <typename T>
int lp_upload_t(LpState &s, const float *A, const float *B, const float *I, cudaStream_t st)
{
    const int w = s.w, h = s.h, ld = s.ld;
    k_lp_split<T><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(A, 0, 4, (T *)s.u, ld, w, h);
    k_lp_split<T><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(A, 1, 4, (T *)s.v, ld, w, h);
    if constexpr (std::is_same<T, double>::value) {
        k_lp_split<double><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(B, 2, 4, s.x[0], ld, w, h);
    } else {  // the pair (p, 0)
        k_lp_split<float><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(B, 2, 4, pair_hi(s, s.x[0]), ld, w, h);
        LCK(cudaMemsetAsync(pair_lo(s, s.x[0]), 0, s.plane * sizeof(float), st));
    }
    LCK(launched(3));
    s.xcur = 0;
    for (int k = 0; k < s.ic; ++k) {
        k_lp_split<T><<<g2(s.iw, s.ih), dim3(kBX, kBY), 0, st>>>(I, k, s.ic, (T *)s.img[0] + k * s.iplane, s.ild, s.iw,
                                                                 s.ih);
        LCK(launched());
    }
    s.icur = 0;
    return PFS_OK;
}

template <typename T, typename O>
int lp_download_t(LpState &s, O *vp, O *img, cudaStream_t st)
{
    const int w = s.w, h = s.h, ld = s.ld;
    if (vp) {
        k_lp_merge<T, O><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(vp, 0, 4, (T *)s.u, ld, w, h);
        k_lp_merge<T, O><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(vp, 1, 4, (T *)s.v, ld, w, h);
        if constexpr (std::is_same<T, double>::value)
            k_lp_merge<double, O><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(vp, 2, 4, s.x[s.xcur], ld, w, h);
        else
            k_ff_merge<O><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(vp, 2, 4, pair_hi(s, s.x[s.xcur]), pair_lo(s, s.x[s.xcur]),
                                                               ld, w, h);
        if (s.form == PFS_PREC_F64)
            k_lp_merge<double, O><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(vp, 3, 4, (double *)s.b, ld, w, h);
        else
            k_lp_merge<float, O><<<g2(w, h), dim3(kBX, kBY), 0, st>>>(vp, 3, 4, (float *)s.b, ld, w, h);
        LCK(launched(4));
    }
    if (img)
        for (int k = 0; k < s.ic; ++k) {
            k_lp_merge<T, O><<<g2(s.iw, s.ih), dim3(kBX, kBY), 0, st>>>(img, k, s.ic, (T *)s.img[s.icur] + k * s.iplane,
                                                                        s.ild, s.iw, s.ih);
            LCK(launched());
        }
    return PFS_OK;
}

}  // namespace

int lp_create(LpState **out, int form, int w, int h, int iw, int ih, int ic)
{
    *out = nullptr;
    LpState *s = new (std::nothrow) LpState();
    if (!s) return lp_fail(PFS_ERR_CUDA, "out of host memory");
    s->form = form;
    s->w = w;
    s->h = h;
    s->ld = rup(w, 32);
    s->plane = (size_t)s->ld * h;
    s->iw = iw;
    s->ih = ih;
    s->ic = ic;
    s->ild = rup(std::max(iw, 1), 32);
    s->iplane = (size_t)s->ild * ih;
    s->tbytes = form == PFS_PREC_F64 ? 8 : form == PFS_PREC_F32R ? 4 : 2;
    const size_t P = s->plane, TB = s->tbytes;
    const size_t bbytes = (form == PFS_PREC_F64 ? 8 : 4) * P;
    // u v ua va (T) | x x (double) | b | r (float) | rt e e (T) | image x2 (T)
    const size_t total = 4 * TB * P + 2 * 8 * P + bbytes + 4 * P + 3 * TB * P + 2 * TB * s->iplane * ic + 6 * 256;
    cudaError_t e = cudaMalloc(&s->mem, total);
    if (e == cudaSuccess) e = cudaMemset(s->mem, 0, total);
    if (e != cudaSuccess) {
        delete s;
        return lp_fail(PFS_ERR_CUDA, cudaGetErrorString(e));
    }
    unsigned char *q = (unsigned char *)s->mem;
    auto take = [&](size_t n) {
        void *r = q;
        q += (n + 255) / 256 * 256;
        return r;
    };
    s->u = take(TB * P);
    s->v = take(TB * P);
    s->ua = take(TB * P);
    s->va = take(TB * P);
    s->x[0] = (double *)take(8 * P);
    s->x[1] = (double *)take(8 * P);
    s->b = take(bbytes);
    s->r = (float *)take(4 * P);
    s->rt = take(TB * P);
    s->e[0] = take(TB * P);
    s->e[1] = take(TB * P);
    s->img[0] = take(TB * s->iplane * ic);
    s->img[1] = take(TB * s->iplane * ic);
    const int nb = kReduceBlocks;
    // partials (2 nb doubles) | result (2) | escale (1) | tickets 0, 1 and maxabs (3 unsigned, padded to 16 B)
    const size_t rbytes = (2 * nb + 3) * sizeof(double) + 16;
    e = cudaMalloc(&s->rmem, rbytes);
    if (e == cudaSuccess) e = cudaMemset(s->rmem, 0, rbytes);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->hres, 2 * sizeof(double), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->hres_d, s->hres, 0);
    if (e != cudaSuccess) {
        lp_destroy(s);
        return lp_fail(PFS_ERR_CUDA, cudaGetErrorString(e));
    }
    s->red.partials = s->rmem;
    s->red.result = s->rmem + 2 * nb;
    s->escale = s->rmem + 2 * nb + 2;
    s->red.ticket = reinterpret_cast<unsigned *>(s->rmem + 2 * nb + 3);
    s->red.nblocks = reduce_grid();
    s->maxabs = s->red.ticket + 2;
    if (form == PFS_PREC_F32R) {
        // the correction solve's checks: partials for the fused check launches at chunks of 16 rows or
        // more and for the scale kernel's norm | result pair | two tickets
        const int ns = std::max(reduce_grid(), sweep_stream_blocks(w, h, kMinChunkRows));
        const size_t ibytes = (2 * (size_t)ns + 2) * sizeof(double) + 16;
        e = cudaMalloc(&s->in_mem, ibytes);
        if (e == cudaSuccess) e = cudaMemset(s->in_mem, 0, ibytes);
        if (e == cudaSuccess) e = cudaMalloc(&s->dstate, sizeof(SolveState));
        if (e == cudaSuccess) e = cudaMemset(s->dstate, 0, sizeof(SolveState));
        if (e == cudaSuccess) e = cudaHostAlloc(&s->hstate, sizeof(SolveState), cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->hstate_d, s->hstate, 0);
        if (e != cudaSuccess) {
            lp_destroy(s);
            return lp_fail(PFS_ERR_CUDA, cudaGetErrorString(e));
        }
        s->red_in.partials = s->in_mem;
        s->red_in.result = s->in_mem + 2 * (size_t)ns;
        s->red_in.ticket = reinterpret_cast<unsigned *>(s->in_mem + 2 * (size_t)ns + 2);
        s->red_in.nblocks = ns;
    }
    *out = s;
    return PFS_OK;
}

void lp_destroy(LpState *s)
{
    if (!s) return;
    if (s->mem) cudaFree(s->mem);
    if (s->rmem) cudaFree(s->rmem);
    if (s->hres) cudaFreeHost(s->hres);
    if (s->stage) cudaFree(s->stage);
    if (s->xback) cudaFree(s->xback);
    if (s->pred) cudaFree(s->pred);
    if (s->in_mem) cudaFree(s->in_mem);
    if (s->dstate) cudaFree(s->dstate);
    if (s->hstate) cudaFreeHost(s->hstate);
    delete s;
}

int lp_upload(LpState *s, const float *vp_dev, const float *tmp_dev, const float *img_dev, cudaStream_t st)
{
    switch (s->form) {
    case PFS_PREC_BF16: return lp_upload_t<__nv_bfloat16>(*s, vp_dev, tmp_dev, img_dev, st);
    case PFS_PREC_F16: return lp_upload_t<__half>(*s, vp_dev, tmp_dev, img_dev, st);
    case PFS_PREC_F64: return lp_upload_t<double>(*s, vp_dev, tmp_dev, img_dev, st);
    case PFS_PREC_F32R: return lp_upload_t<float>(*s, vp_dev, tmp_dev, img_dev, st);
    default: return lp_fail(PFS_ERR_UNSUPPORTED, "unknown precision form");
    }
}

int lp_step(LpState *s, const LpParams &p, cudaStream_t st, LpOut &o)
{
    switch (s->form) {
    case PFS_PREC_BF16: return lp_step_ir<__nv_bfloat16>(*s, p, st, o);
    case PFS_PREC_F16: return lp_step_ir<__half>(*s, p, st, o);
    case PFS_PREC_F64: return lp_step64(*s, p, st, o);
    case PFS_PREC_F32R: return lp_step_ir<float>(*s, p, st, o);
    default: return lp_fail(PFS_ERR_UNSUPPORTED, "unknown precision form");
    }
}

int lp_download(LpState *s, float *vp_dev, float *img_dev, cudaStream_t st)
{
    switch (s->form) {
    case PFS_PREC_BF16: return lp_download_t<__nv_bfloat16, float>(*s, vp_dev, img_dev, st);
    case PFS_PREC_F16: return lp_download_t<__half, float>(*s, vp_dev, img_dev, st);
    case PFS_PREC_F64: return lp_download_t<double, float>(*s, vp_dev, img_dev, st);
    case PFS_PREC_F32R: return lp_download_t<float, float>(*s, vp_dev, img_dev, st);
    default: return lp_fail(PFS_ERR_UNSUPPORTED, "unknown precision form");
    }
}

int lp_download_f64(LpState *s, double *vp_dev, double *img_dev, cudaStream_t st)
{
    switch (s->form) {
    case PFS_PREC_BF16: return lp_download_t<__nv_bfloat16, double>(*s, vp_dev, img_dev, st);
    case PFS_PREC_F16: return lp_download_t<__half, double>(*s, vp_dev, img_dev, st);
    case PFS_PREC_F64: return lp_download_t<double, double>(*s, vp_dev, img_dev, st);
    case PFS_PREC_F32R: return lp_download_t<float, double>(*s, vp_dev, img_dev, st);
    default: return lp_fail(PFS_ERR_UNSUPPORTED, "unknown precision form");
    }
}

}  // namespace pfs
