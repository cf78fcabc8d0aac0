// Per-cell pieces of the timestep (advection, divergence, projection, image
// advection, exact residual) shared by the step kernels (step_kernels.cu) and
// the persistent ensemble kernel (ensemble.cu). Every formula keeps the
// reference's operation order (src/fluid.cpp, cited per function).
#pragma once

#include "bounds.cuh"
#include "common.cuh"
#include "reduce.cuh"

namespace pfs {
namespace {

__device__ __forceinline__ int wm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wp(int i, int n) { return i + 1 == n ? 0 : i + 1; }

// Boundary modes of the backtrace (pfs_params.boundary): 0 periodic wrap (the
// reference); 1 clamp, the reference's commented-out alternative
// (src/fluid.cpp:43-45,100-102): std::max(0.5f, std::min<float>(n - 1.5, x)),
// after which i0 + 1 stays inside the grid; 2 walls: clamp, and zero velocity
// on the boundary cells after advection and after projection.
template <int BC>
__device__ __forceinline__ float bound_coord(float x, float n)
{
    if constexpr (BC == 0) {
        return wrap_coord(x, n);
    } else {
        const float hi = fsub(n, 1.5f);        // exact: n is an integer below 2^23
        const float m = (x < hi) ? x : hi;     // std::min<float>(hi, x)
        return (0.5f < m) ? m : 0.5f;          // std::max(0.5f, m)
    }
}

__device__ __forceinline__ bool on_edge(int i, int j, int w, int h)
{
    return i == 0 || j == 0 || i == w - 1 || j == h - 1;
}

// Backtrace, wrap (or clamp) and corner cells of one sample (src/fluid.cpp:39-58
// and :97-114): x' = i - (k*u)/n wrapped to [0, n).
struct Corners {
    int i0, i1, j0, j1;
    float sx, sy;
};

template <int BC = 0>
__device__ __forceinline__ Corners backtrace(int i, int j, float kx, float ky, float u, float v, float fw, float fh,
                                            int w, int h)
{
    float xp = fsub((float)i, fdiv(fmul(kx, u), fw));
    float yp = fsub((float)j, fdiv(fmul(ky, v), fh));
    xp = bound_coord<BC>(xp, fw);
    yp = bound_coord<BC>(yp, fh);
    Corners c;
    c.i0 = cell_of(xp, w);
    c.j0 = cell_of(yp, h);
    c.i1 = (c.i0 + 1) % w;
    c.j1 = (c.j0 + 1) % h;
    c.sx = fsub(xp, (float)c.i0);
    c.sy = fsub(yp, (float)c.j0);
    return c;
}

// Velocity advection of cell (i, j), src/fluid.cpp:24-70: the new velocity
// (uo, vo) without storing it.
template <int BC = 0>
__device__ __forceinline__ void advect_value(const float *__restrict__ u, const float *__restrict__ v, int ld, int w,
                                             int h, float dt, int i, int j, float &uo, float &vo)
{
    const size_t o = (size_t)j * ld + i;
    const long long n = (long long)ld * h;  // plane extent (checked build)
    (void)n;
    if (BC == 2 && on_edge(i, j, w, h)) {
        uo = 0.0f;
        vo = 0.0f;
        return;
    }
    const Corners c = backtrace<BC>(i, j, dt, dt, PFS_LD(u, o, n, kBsAdvect), PFS_LD(v, o, n, kBsAdvect), (float)w,
                                    (float)h, w, h);
    const size_t r0 = (size_t)c.j0 * ld, r1 = (size_t)c.j1 * ld;
    uo = bilerp(c.sx, c.sy, PFS_LD(u, r0 + c.i0, n, kBsAdvect), PFS_LD(u, r0 + c.i1, n, kBsAdvect),
                PFS_LD(u, r1 + c.i0, n, kBsAdvect), PFS_LD(u, r1 + c.i1, n, kBsAdvect));
    vo = bilerp(c.sx, c.sy, PFS_LD(v, r0 + c.i0, n, kBsAdvect), PFS_LD(v, r0 + c.i1, n, kBsAdvect),
                PFS_LD(v, r1 + c.i0, n, kBsAdvect), PFS_LD(v, r1 + c.i1, n, kBsAdvect));
}

// Velocity advection of cell (i, j), stored.
template <int BC = 0>
__device__ __forceinline__ void advect_cell(const float *__restrict__ u, const float *__restrict__ v,
                                            float *__restrict__ uo, float *__restrict__ vo, int ld, int w, int h,
                                            float dt, int i, int j)
{
    const size_t o = (size_t)j * ld + i;
    const long long n = (long long)ld * h;
    (void)n;
    float a, b;
    advect_value<BC>(u, v, ld, w, h, dt, i, j, a, b);
    PFS_ST(uo, o, n, a, kBsAdvect);
    PFS_ST(vo, o, n, b, kBsAdvect);
}

// Divergence of cell (i, j), src/fluid.cpp:218-237, without storing it.
__device__ __forceinline__ float divergence_value(const float *__restrict__ u, const float *__restrict__ v, int ld,
                                                  int w, int h, float gamma, int i, int j)
{
    const size_t r = (size_t)j * ld;
    const long long n = (long long)ld * h;
    (void)n;
    const float du = fsub(PFS_LD(u, r + wp(i, w), n, kBsDivergence), PFS_LD(u, r + wm(i, w), n, kBsDivergence));
    const float dv = fsub(PFS_LD(v, (size_t)wp(j, h) * ld + i, n, kBsDivergence),
                          PFS_LD(v, (size_t)wm(j, h) * ld + i, n, kBsDivergence));
    return fmul(gamma, fadd(du, dv));
}

// Divergence of cell (i, j) into b; returns it.
__device__ __forceinline__ float divergence_cell(const float *__restrict__ u, const float *__restrict__ v,
                                                 float *__restrict__ b, int ld, int w, int h, float gamma, int i,
                                                 int j)
{
    const float bv = divergence_value(u, v, ld, w, h, gamma, i, j);
    PFS_ST(b, (size_t)j * ld + i, (long long)ld * h, bv, kBsDivergence);
    return bv;
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

// residual_sq for two cells at once (element x: one cell, element y: another),
// each element with exactly the arithmetic of residual_sq.
__device__ __forceinline__ void residual_sq2(FFAcc2 &acc, float2 b, float2 l, float2 r, float2 t, float2 bo, float2 c)
{
    FF2 s = two_sum2(b, l);
    float2 e = s.lo;
    s = two_sum2(s.hi, r);
    e = __fadd2_rn(e, s.lo);
    s = two_sum2(s.hi, t);
    e = __fadd2_rn(e, s.lo);
    s = two_sum2(s.hi, bo);
    e = __fadd2_rn(e, s.lo);
    s = two_sum2(s.hi, __fmul2_rn(make_float2(-4.0f, -4.0f), c));  // -4p is exact
    e = __fadd2_rn(e, s.lo);
    const FF2 q = two_sum2(s.hi, e);
    const float2 sq = __fmul2_rn(q.hi, q.hi);
    const float2 sq_err = __ffma2_rn(q.hi, q.hi, make_float2(-sq.x, -sq.y));
    const float2 cross = __fmul2_rn(__fmul2_rn(make_float2(2.0f, 2.0f), q.hi), q.lo);
    acc.add(sq, __fadd2_rn(sq_err, cross));
}

// The residual of the four cells a lane holds in row c (float4 x, y, z, w),
// with the row above `up`, the row below `dn`, the outside neighbours lft
// (of x) and rgt (of w): cells x, y into acc[0], z, w into acc[1].
__device__ __forceinline__ void residual_sq4(FFAcc2 (&acc)[2], const float4 &bb, float lft, const float4 &c,
                                             float rgt, const float4 &up, const float4 &dn)
{
    residual_sq2(acc[0], make_float2(bb.x, bb.y), make_float2(lft, c.x), make_float2(c.y, c.z),
                 make_float2(up.x, up.y), make_float2(dn.x, dn.y), make_float2(c.x, c.y));
    residual_sq2(acc[1], make_float2(bb.z, bb.w), make_float2(c.y, c.z), make_float2(c.w, rgt),
                 make_float2(up.z, up.w), make_float2(dn.z, dn.w), make_float2(c.z, c.w));
}

// Projection, src/fluid.cpp:269-296: u - ((pR-pL)*dt)/2, v - ((pB-pT)*dt)/2
// (walls: zero on the boundary cells).
template <int BC = 0>
__device__ __forceinline__ void project_cell(const float *__restrict__ u, const float *__restrict__ v,
                                             const float *__restrict__ p, int ld, int w, int h, float dt, int i,
                                             int j, float &uo, float &vo)
{
    const size_t r = (size_t)j * ld;
    const long long n = (long long)ld * h;
    (void)n;
    const float gx =
        fmul(fmul(fsub(PFS_LD(p, r + wp(i, w), n, kBsProject), PFS_LD(p, r + wm(i, w), n, kBsProject)), dt), 0.5f);
    const float gy = fmul(fmul(fsub(PFS_LD(p, (size_t)wp(j, h) * ld + i, n, kBsProject),
                                    PFS_LD(p, (size_t)wm(j, h) * ld + i, n, kBsProject)),
                               dt),
                          0.5f);
    uo = fsub(PFS_LD(u, r + i, n, kBsProject), gx);
    vo = fsub(PFS_LD(v, r + i, n, kBsProject), gy);
    if (BC == 2 && on_edge(i, j, w, h)) {
        uo = 0.0f;
        vo = 0.0f;
    }
}

// Projection then image advection of cell (i, j) with the just-projected
// velocity (image grid = velocity grid: viw = vih = 1, and dt / viw = dt).
template <int BC = 0>
__device__ __forceinline__ void project_image_cell(const float *__restrict__ u, const float *__restrict__ v,
                                                   const float *__restrict__ p, float *__restrict__ uo,
                                                   float *__restrict__ vo, int ld, int w, int h, float dt,
                                                   const float *__restrict__ img, float *__restrict__ imgo,
                                                   size_t plane, int c, int i, int j)
{
    float un, vn;
    project_cell<BC>(u, v, p, ld, w, h, dt, i, j, un, vn);
    const size_t o = (size_t)j * ld + i;
    const long long n = (long long)ld * h, ni = (long long)plane * c;  // velocity plane, image planes
    (void)n;
    (void)ni;
    PFS_ST(uo, o, n, un, kBsProject);
    PFS_ST(vo, o, n, vn, kBsProject);
    const Corners k = backtrace<BC>(i, j, dt, dt, un, vn, (float)w, (float)h, w, h);
    const size_t r0 = (size_t)k.j0 * ld, r1 = (size_t)k.j1 * ld;
    for (int ch = 0; ch < c; ++ch) {
        const size_t s = ch * plane;
        PFS_ST(imgo, s + o, ni,
               bilerp(k.sx, k.sy, PFS_LD(img, s + r0 + k.i0, ni, kBsImage), PFS_LD(img, s + r0 + k.i1, ni, kBsImage),
                      PFS_LD(img, s + r1 + k.i0, ni, kBsImage), PFS_LD(img, s + r1 + k.i1, ni, kBsImage)),
               kBsImage);
    }
}

// Residual sums of one warp task of the strip residual: strip sx (128
// columns, four per lane), rows [y0, y1). Adds r^2 into acc (one chain per
// lane column: columns x, y in acc[0], z, w in acc[1]) and, with accb, b^2.
__device__ __forceinline__ void residual_strip_task(const float *__restrict__ p, const float *__restrict__ b, int ld,
                                                    int w, int h, int sx, int y0, int y1, int lane, FFAcc2 (&acc)[2],
                                                    FFAcc *accb)
{
    const int x = sx * 128 + 4 * lane;
    const bool active = x < w;
    const int xs = active ? x : w - 4;  // inactive lanes shadow a valid column, results discarded
    const int last_lane = min(31, (w - sx * 128) / 4 - 1);
    const int xl = (sx * 128 == 0) ? w - 1 : sx * 128 - 1;  // left outside neighbour
    const int xr = (sx * 128 + 4 * (last_lane + 1)) % w;    // right outside neighbour
    // loads bypass L1 (ld.global.cg): inside the persistent ensemble kernel the
    // pressure planes are rewritten by other blocks between checks
    const long long n = (long long)ld * h;
    (void)n;
    // four floats of plane q from element k (k checked against the plane in the checked build)
    auto row4 = [&](const float *q, size_t k) {
        return PFS_SPAN(k, 4, n, kBsResidual) ? __ldcg(reinterpret_cast<const float4 *>(q + k))
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    auto one = [&](size_t k) { return PFS_SPAN(k, 1, n, kBsResidual) ? __ldcg(p + k) : 0.0f; };
    float4 up = row4(p, xs + (size_t)wm(y0, h) * ld);
    float4 cu = row4(p, xs + (size_t)y0 * ld);
    for (int y = y0; y < y1; ++y) {
        const float4 dn = row4(p, xs + (size_t)wp(y, h) * ld);
        const float4 bb = row4(b, (size_t)y * ld + xs);
        float lft = __shfl_up_sync(0xffffffffu, cu.w, 1);
        float rgt = __shfl_down_sync(0xffffffffu, cu.x, 1);
        if (lane == 0) lft = one((size_t)y * ld + xl);
        if (lane == last_lane) rgt = one((size_t)y * ld + xr);
        if (active) {
            residual_sq4(acc, bb, lft, cu, rgt, up, dn);
            if (accb) {
                acc_square(*accb, bb.x);
                acc_square(*accb, bb.y);
                acc_square(*accb, bb.z);
                acc_square(*accb, bb.w);
            }
        }
        up = cu;
        cu = dn;
    }
}

}  // namespace
}  // namespace pfs
