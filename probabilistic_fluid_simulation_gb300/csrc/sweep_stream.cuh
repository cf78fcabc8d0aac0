// The fused (temporally blocked) pressure sweep as a warp task, shared by the
// standalone launch (sweep_kernels.cu) and the persistent ensemble kernel
// (ensemble.cu). See sweep_kernels.cu for the design.
#pragma once

#include "bounds.cuh"
#include "cells.cuh"
#include "common.cuh"
#include "kernels.h"
#include "reduce.cuh"
#include "storage.cuh"

namespace pfs {
namespace {

// Level s+1 of the lane's four cells of row r from level s: `c` is row r
// (horizontal neighbours from lanes l-1 / l+1), `up` row r-1, `dn` row r+1,
// `bq` the quarter b/4 of row r. Per cell the reference computes
// RN(RN(s + b) / 4) with s = ((l + r) + t) + bo rounded after each add
// (pfs::jacobi_p); this computes the sum s the same way and then
// RN(s * 0.25 + b/4) in one fused multiply-add. Scaling by a power of two
// commutes with rounding to nearest in the normal range, so the two agree
// bit for bit whenever b/4 is exact and |s + b| >= 2^-124 (or s + b = 0,
// signed zeros included), and when s + b does not overflow: they can differ
// only for pressures within a factor 4 of float32's subnormal range. That
// takes a dependent rounding and a packed multiply off each level. The first
// add pairs values from different lanes and runs as four scalar adds; the
// rest act on the aligned pairs (x, y) and (z, w) with the packed f32x2
// instructions of sm_100+ (__fadd2_rn / __ffma2_rn round each element to
// nearest), which halves their issue slots.
__device__ __forceinline__ float4 jacobi4(const float4 &c, const float4 &up, const float4 &dn, const float4 &bq)
{
    const float lft = __shfl_up_sync(0xffffffffu, c.w, 1);
    const float rgt = __shfl_down_sync(0xffffffffu, c.x, 1);
    float2 a = make_float2(__fadd_rn(lft, c.y), __fadd_rn(c.x, c.z));
    float2 z = make_float2(__fadd_rn(c.y, c.w), __fadd_rn(c.z, rgt));
    a = __fadd2_rn(a, make_float2(up.x, up.y));
    z = __fadd2_rn(z, make_float2(up.z, up.w));
    a = __fadd2_rn(a, make_float2(dn.x, dn.y));
    z = __fadd2_rn(z, make_float2(dn.z, dn.w));
    const float2 q = make_float2(0.25f, 0.25f);
    a = __ffma2_rn(a, q, make_float2(bq.x, bq.y));
    z = __ffma2_rn(z, q, make_float2(bq.z, bq.w));
    return make_float4(a.x, a.y, z.x, z.y);
}

// v * s for a power of two s, on the pairs (x, y) and (z, w).
__device__ __forceinline__ float4 scale4(const float4 &v, float s)
{
    const float2 q = make_float2(s, s);
    const float2 a = __fmul2_rn(make_float2(v.x, v.y), q);
    const float2 z = __fmul2_rn(make_float2(v.z, v.w), q);
    return make_float4(a.x, a.y, z.x, z.y);
}

template <typename T>
struct StreamArgs {
    const T *pin;     // null: the input iterate is all zeros
    const T *b;
    T *pout;
    T *pprev;         // receives level L-1 (the second-to-last iterate) when non-null
    const int *done;  // solve already converged: return at once
    int ld, w, h;
    int nsx, nwork, chunk;
    // launches that also evaluate the residual of their last level (a check point)
    Reduce red;          // partials for one block per 4 warp tasks; result[1] holds sum b^2
    SolveState *state;   // records the check, raises done at or below tol
    int sweeps_here;     // sweep count of the solve after this launch
    double tol;
    int stall_window;    // > 0: stop when the residual stops falling (SolveState)
};

// Warps per block of the standalone sweep kernel. Each of an SM's four
// schedulers holds 16384 registers, so the warps a scheduler can take follow
// from the registers per thread whatever the block size (at 176 registers,
// blocks of two warps measured the same as four); the 7- and 8-level kernels
// are held at two blocks per SM, two warps per scheduler (launch_stream_t).
constexpr int kStreamWarps = 4;

constexpr int gcd_c(int a, int b) { return b == 0 ? a : gcd_c(b, a % b); }
constexpr int lcm_c(int a, int b) { return a / gcd_c(a, b) * b; }
// The smallest divisor of u that is at least 4, else the smallest multiple of u that is.
constexpr int ring_depth(int u, int d = 4) { return d > u ? (4 + u - 1) / u * u : (u % d == 0 ? d : ring_depth(u, d + 1)); }

// Register rings of the pipeline. Level s (0..L-1) keeps rows y-s-2, y-s-1,
// y-s in three register sets whose roles rotate with period 3; the divergence
// rows y-1 .. y-L (as b/4) plus the row being loaded live in a ring of NB = L+1
// registers (L+2 when the launch also evaluates the residual of level L,
// which needs b one row further back). The rows copied from global memory
// land in a shared-memory ring of D rows per plane (D-1 rows in flight).
// Unrolling the row loop by U = lcm(3, NB, D) makes every ring index a
// compile-time name: register rings without moves, shared-memory slots at
// fixed offsets, one shared-memory read of b per row instead of one per level.
template <typename T, int L, bool RES = false>
struct Ring {
    static constexpr int NB = L + 1 + (RES ? 1 : 0);
    static constexpr int UR = lcm_c(3, NB);
    static constexpr int D = ring_depth(UR);
    static constexpr int U = lcm_c(UR, D);
    static constexpr int vecs_per_warp = 2 * D * 32;  // p and b rings, one vector per lane and row
    static constexpr int bytes_per_block = 4 * vecs_per_warp * Store<T>::vec_bytes;
};

template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem);
template <>
__device__ __forceinline__ void cp_async<16>(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
template <>
__device__ __forceinline__ void cp_async<8>(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Offsets count vectors of four cells (16 B in float32), which keeps them in
// 32 bits for planes below 2^33 cells (launch_stream_t checks): each address
// is then one wide multiply-add from the plane's base, and the periodic wrap
// of the copied rows one compare and subtract.
template <typename T>
struct Cursor {
    int off;     // vector offset of the next row to copy (lane column), the same in the p and b planes
    int st_vo;   // vector offset of this step's level-L row from the lane column
    int st_rel;  // that row minus y0 (stored when 0 <= st_rel < rows)
};

// Issue the cp.async of the next row into ring slot `slot` of p and b.
template <typename T>
__device__ __forceinline__ void prefetch_row(Cursor<T> &cu, typename Store<T>::Vec *pr, typename Store<T>::Vec *br,
                                             int slot, const StreamArgs<T> &a)
{
    using V = typename Store<T>::Vec;
    constexpr int VB = Store<T>::vec_bytes;
    const long long n = (long long)a.ld * a.h;  // plane extent (checked build)
    (void)n;
    const int ldv = a.ld >> 2, hv = a.h * ldv;  // row and plane, in vectors
    if (a.pin && PFS_SPAN(4LL * cu.off, 4, n, kBsSweepLoadP))
        cp_async<VB>(pr + slot * 32, reinterpret_cast<const V *>(a.pin) + cu.off);
    if (PFS_SPAN(4LL * cu.off, 4, n, kBsSweepLoadB)) cp_async<VB>(br + slot * 32, reinterpret_cast<const V *>(a.b) + cu.off);
    cu.off += ldv;
    if (cu.off >= hv) cu.off -= hv;
}

// One row step t of the pipeline (load row y = ybeg + t); K = t mod U is a
// compile-time constant, so R[K % 3]..., bq[...] and the shared-memory slots
// (row t in slot K % D) are fixed names. (Deriving the stored row from t
// instead of the running st_off / st_rel measured 4% slower.)
// T0 >= 0: t = T0 + K is known at compile time (the ramp at the start of a
// task), and the levels whose row at this step lies outside the trapezoid the
// stored rows need are not computed. Level s at step t produces level s+1 at
// row ybeg + t - s - 1, and the stored rows need level s+1 from row
// ybeg + s + 1 on (from y0 - (E - s - 1)), so it is useful from t = 2s + 2 on.
// At 8 levels and 32-row chunks that is 72 of the 384 level rows of a task.
// A skipped level leaves its ring slot holding an older row, which feeds only
// rows outside the trapezoid in turn.
// With RES, TR keeps the last three level-L rows (period 3) and the step adds
// the exact squared residual of level L at row y-L-1 (the row stored at the
// previous step) into acc, with the per-cell arithmetic of the residual
// kernels (residual_sq), for the stored lanes only.
template <typename T, int L, bool PREV, bool RES, int K, int T0, bool GUARD>
__device__ __forceinline__ void stream_step(int t, float4 (&R)[3][L], float4 (&bq)[Ring<T, L, RES>::NB],
                                            float4 (&TR)[3], FFAcc2 (&acc)[2], typename Store<T>::Vec *pr,
                                            typename Store<T>::Vec *br, Cursor<T> &cu, const StreamArgs<T> &a,
                                            int nsteps, int rows, T *out, T *outp)
{
    using V = typename Store<T>::Vec;
    constexpr int NB = Ring<T, L, RES>::NB;
    constexpr int D = Ring<T, L, RES>::D;
    float4(&P)[L] = R[K % 3];
    float4(&Cur)[L] = R[(K + 1) % 3];
    float4(&N)[L] = R[(K + 2) % 3];
    // unguarded blocks copy rows past the task's last one as well: they lie in
    // the plane (rows wrap) and land in slots whose rows are consumed
    if (!GUARD || t + D - 1 < nsteps) prefetch_row(cu, pr, br, (K + D - 1) % D, a);
    cp_async_commit();
    cp_async_wait<D - 1>();  // row t has landed
    N[0] = Store<T>::to_f4(pr[(K % D) * 32]);  // zeros when a.pin is null (ring zero-filled)
    bq[K % NB] = scale4(Store<T>::to_f4(br[(K % D) * 32]), 0.25f);  // b/4 of row y, used from the next step
    float4 top = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int s = 0; s < L; ++s) {
        if (T0 >= 0 && T0 + K < 2 * s + 2) continue;        // compile-time: outside the trapezoid
        const float4 &bb = bq[(K + NB * L - s - 1) % NB];  // b/4 of row y-s-1
        const float4 o = jacobi4(Cur[s], P[s], N[s], bb);   // level s+1, row y-s-1
        if (s + 1 < L) N[s + 1] = o;
        else top = o;
    }
    const int ldv = a.ld >> 2;
    if (out && (unsigned)cu.st_rel < (unsigned)rows &&
        PFS_SPAN(out + 4LL * cu.st_vo - a.pout, 4, (long long)a.ld * a.h, kBsSweepStore))
        reinterpret_cast<V *>(out)[cu.st_vo] = Store<T>::from_f4(top);
    if (PREV && outp && (unsigned)(cu.st_rel + 1) < (unsigned)rows &&
        PFS_SPAN(outp + 4LL * (cu.st_vo + ldv) - a.pprev, 4, (long long)a.ld * a.h, kBsSweepStorePrev))
        reinterpret_cast<V *>(outp)[cu.st_vo + ldv] = Store<T>::from_f4(N[L - 1]);
    if constexpr (RES) {
        TR[K % 3] = top;                                  // level L, row y-L
        const float4 &c = TR[(K + 2) % 3];                // row y-L-1
        const float4 &up = TR[(K + 1) % 3];               // row y-L-2
        const float4 bb = scale4(bq[(K + NB * (L + 1) - L - 1) % NB], 4.0f);  // b of row y-L-1
        const float lft = __shfl_up_sync(0xffffffffu, c.w, 1);
        const float rgt = __shfl_down_sync(0xffffffffu, c.x, 1);
        if (out && (unsigned)(cu.st_rel - 1) < (unsigned)rows) {
            residual_sq4(acc, bb, lft, c, rgt, up, top);
        }
    }
    cu.st_vo += ldv;
    cu.st_rel += 1;
}

template <typename T, int L, bool PREV, bool RES, int K, int T0, bool GUARD = true>
__device__ __forceinline__ void stream_steps(int t, float4 (&R)[3][L], float4 (&bq)[Ring<T, L, RES>::NB],
                                             float4 (&TR)[3], FFAcc2 (&acc)[2], typename Store<T>::Vec *pr,
                                             typename Store<T>::Vec *br, Cursor<T> &cu, const StreamArgs<T> &a,
                                             int nsteps, int rows, T *out, T *outp)
{
    if constexpr (K < Ring<T, L, RES>::U) {
        if (!GUARD || t + K < nsteps) {
            stream_step<T, L, PREV, RES, K, T0, GUARD>(t + K, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out,
                                                       outp);
            stream_steps<T, L, PREV, RES, K + 1, T0, GUARD>(t, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out,
                                                            outp);
        }
    }
}

// The ramp: the unrolled iterations I = 0, 1, ... whose first step I * U is
// below 2L, with their step numbers known at compile time.
template <typename T, int L, bool PREV, bool RES, int I, bool GUARD>
__device__ __forceinline__ void stream_ramp(float4 (&R)[3][L], float4 (&bq)[Ring<T, L, RES>::NB], float4 (&TR)[3],
                                            FFAcc2 (&acc)[2], typename Store<T>::Vec *pr,
                                            typename Store<T>::Vec *br, Cursor<T> &cu, const StreamArgs<T> &a,
                                            int nsteps, int rows, T *out, T *outp)
{
    constexpr int U = Ring<T, L, RES>::U;
    if constexpr (I * U < 2 * L) {
        stream_steps<T, L, PREV, RES, 0, I * U, GUARD>(I * U, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out,
                                                       outp);
        stream_ramp<T, L, PREV, RES, I + 1, GUARD>(R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
    }
}
template <int L, int U>
constexpr int ramp_steps() { return (2 * L + U - 1) / U * U; }

// Blocks of 128 threads per SM the register budget aims for: the deepest
// pipelines need more than 65536 / (3 * 128) registers per thread without
// spilling.
template <int L>
constexpr int min_blocks() { return L >= 7 ? 2 : 3; }

// One warp task of the fused sweep: strip wid % nsx, row chunk wid / nsx.
// `ring` is this warp's shared-memory ring (Ring<T, L>::vecs_per_warp vectors).
// With RES the task also adds the squared residual of level L over its stored
// cells into acc: it loads one more halo row at each end (level L is then
// valid one row beyond the chunk), and L < G keeps level L valid one column
// beyond the stored lanes.
template <typename T, int G, int L, bool PREV, bool RES = false>
__device__ __forceinline__ void stream_task(const StreamArgs<T> &a, int wid, int lane, typename Store<T>::Vec *ring,
                                            FFAcc2 (&acc)[2])
{
    static_assert(L >= 1 && L <= G && G % 4 == 0, "fusion depth must fit the halo");
    static_assert(!RES || L < G, "the residual needs level L one column beyond the stored lanes");
    using V = typename Store<T>::Vec;
    const int sx = wid % a.nsx, sy = wid / a.nsx;
    const int xo = sx * (128 - 2 * G);
    const int xl = xo - G + 4 * lane;
    int cx = xl % a.w;
    if (cx < 0) cx += a.w;
    const bool st_lane = lane >= G / 4 && lane < 32 - G / 4 && xl < a.w;
    const int y0 = sy * a.chunk;
    const int rows = min(a.h, y0 + a.chunk) - y0;
    constexpr int E = RES ? L + 1 : L;  // halo rows loaded at each end
    const int ybeg = y0 - E;
    const int nsteps = rows + 2 * E;

    constexpr int D = Ring<T, L, RES>::D;
    V *pr = ring + lane;
    V *br = pr + D * 32;
    if (!a.pin) {  // zero input iterate: no p rows are copied, the ring stays zero
#pragma unroll
        for (int k = 0; k < D; ++k) pr[k * 32] = V{};
    }

    Cursor<T> cu;
    int ld_row = ybeg % a.h;
    if (ld_row < 0) ld_row += a.h;
    cu.off = ld_row * (a.ld >> 2) + (cx >> 2);  // cx and ld are multiples of 4
    cu.st_rel = -E - L;  // level L at step 0 is row ybeg - L = y0 - E - L
    cu.st_vo = (y0 - E - L) * (a.ld >> 2);
    T *out = st_lane ? a.pout + cx : nullptr;
    T *outp = (PREV && st_lane) ? a.pprev + cx : nullptr;
#pragma unroll
    for (int k = 0; k < D - 1; ++k) {
        if (k < nsteps) prefetch_row(cu, pr, br, k, a);
        cp_async_commit();
    }

    constexpr int NB = Ring<T, L, RES>::NB;
    float4 R[3][L], bq[NB], TR[3];
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int s = 0; s < L; ++s) R[0][s] = R[1][s] = R[2][s] = z;
#pragma unroll
    for (int s = 0; s < NB; ++s) bq[s] = z;
    TR[0] = TR[1] = TR[2] = z;

    constexpr int U = Ring<T, L, RES>::U;
    if constexpr (RES) {
        // check launches: a guard per step and one copy of each loop. Their
        // blocks (up to 24 steps with the residual's arithmetic in each)
        // compiled for over ten minutes per unit in the unguarded form below.
        stream_ramp<T, L, PREV, RES, 0, true>(R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
        for (int t = ramp_steps<L, U>(); t < nsteps; t += U)
            stream_steps<T, L, PREV, RES, 0, -1, true>(t, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
    } else {
        // Whole blocks of U steps without per-step guards (one basic block,
        // which the compiler schedules across steps: 12.3 -> 10.9 us per
        // 8-level launch at 2048^2), then the guarded remainder.
        if (nsteps >= ramp_steps<L, U>())
            stream_ramp<T, L, PREV, RES, 0, false>(R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
        else
            stream_ramp<T, L, PREV, RES, 0, true>(R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
        int t = ramp_steps<L, U>();
        for (; t + U <= nsteps; t += U)
            stream_steps<T, L, PREV, RES, 0, -1, false>(t, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
        if (t < nsteps)
            stream_steps<T, L, PREV, RES, 0, -1, true>(t, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
    }
    cp_async_wait<0>();
}

template <typename T, int G, int L, bool PREV>
__device__ __forceinline__ void stream_task(const StreamArgs<T> &a, int wid, int lane, typename Store<T>::Vec *ring)
{
    FFAcc2 unused[2];
    stream_task<T, G, L, PREV, false>(a, wid, lane, ring, unused);
}

}  // namespace
}  // namespace pfs
