// The fused (temporally blocked) pressure sweep as a warp task, shared by the
// standalone launch (sweep_kernels.cu) and the persistent ensemble kernel
// (ensemble.cu). See sweep_kernels.cu for the design.
#pragma once

#include "cells.cuh"
#include "common.cuh"
#include "kernels.h"
#include "reduce.cuh"
#include "storage.cuh"

namespace pfs {
namespace {

// Level s+1 of the lane's four cells of row r from level s: `c` is row r
// (horizontal neighbours from lanes l-1 / l+1), `up` row r-1, `dn` row r+1.
// Per cell this is ((((l + r) + t) + bo) + b) * 0.25 with one rounding per
// operation, as pfs::jacobi_p. The first add pairs values from different
// lanes and runs as four scalar adds; the remaining adds and the scale act on
// the aligned pairs (x, y) and (z, w) with the packed f32x2 instructions of
// sm_100+ (__fadd2_rn / __fmul2_rn round each element to nearest, like
// __fadd_rn), which halves their issue slots.
__device__ __forceinline__ float4 jacobi4(const float4 &c, const float4 &up, const float4 &dn, const float4 &bb)
{
    const float lft = __shfl_up_sync(0xffffffffu, c.w, 1);
    const float rgt = __shfl_down_sync(0xffffffffu, c.x, 1);
    float2 a = make_float2(__fadd_rn(lft, c.y), __fadd_rn(c.x, c.z));
    float2 z = make_float2(__fadd_rn(c.y, c.w), __fadd_rn(c.z, rgt));
    a = __fadd2_rn(a, make_float2(up.x, up.y));
    z = __fadd2_rn(z, make_float2(up.z, up.w));
    a = __fadd2_rn(a, make_float2(dn.x, dn.y));
    z = __fadd2_rn(z, make_float2(dn.z, dn.w));
    a = __fadd2_rn(a, make_float2(bb.x, bb.y));
    z = __fadd2_rn(z, make_float2(bb.z, bb.w));
    const float2 q = make_float2(0.25f, 0.25f);
    a = __fmul2_rn(a, q);
    z = __fmul2_rn(z, q);
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

// Rows in flight per warp (cp.async prefetch depth).
constexpr int kRP = 4;  // power of two

constexpr int gcd_c(int a, int b) { return b == 0 ? a : gcd_c(b, a % b); }

// Register rings of the pipeline. Level s (0..L-1) keeps rows y-s-2, y-s-1,
// y-s in three register sets whose roles rotate with period 3; the divergence
// rows y-1 .. y-L plus the row being loaded live in a ring of L+1 registers
// (L+2 when the launch also evaluates the residual of level L, which needs b
// one row further back). Unrolling the row loop by U = lcm(3, NB) makes every
// ring index a compile-time register name: no register moves, one
// shared-memory read of b per row instead of one per level.
template <typename T, int L, bool RES = false>
struct Ring {
    static constexpr int NB = L + 1 + (RES ? 1 : 0);
    static constexpr int U = 3 * NB / gcd_c(3, NB);
    static constexpr int vecs_per_warp = 2 * kRP * 32;  // p and b prefetch rings, one vector per lane and row
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

template <typename T>
struct Cursor {
    const T *gp, *gb;      // next row to prefetch (p and b planes, lane column)
    int ld_row;            // its row index (wrapped)
    long long st_off;      // offset of the level-L row of this step, in floats from the lane column
    int st_rel;            // that row minus y0 (stored when 0 <= st_rel < rows)
};

// Issue the cp.async of the next row into ring slot `slot` of p and b.
template <typename T>
__device__ __forceinline__ void prefetch_row(Cursor<T> &cu, typename Store<T>::Vec *pr, typename Store<T>::Vec *br,
                                             int slot, const StreamArgs<T> &a)
{
    constexpr int VB = Store<T>::vec_bytes;
    if (a.pin) cp_async<VB>(pr + slot * 32, cu.gp);
    cp_async<VB>(br + slot * 32, cu.gb);
    if (++cu.ld_row == a.h) {
        cu.ld_row = 0;
        cu.gp -= (size_t)(a.h - 1) * a.ld;
        cu.gb -= (size_t)(a.h - 1) * a.ld;
    } else {
        cu.gp += a.ld;
        cu.gb += a.ld;
    }
}

// One row step t of the pipeline (load row y = ybeg + t); K = t mod U is a
// compile-time constant, so R[K % 3]... and bq[...] name fixed registers.
// With RES, TR keeps the last three level-L rows (period 3) and the step adds
// the exact squared residual of level L at row y-L-1 (the row stored at the
// previous step) into acc, with the per-cell arithmetic of the residual
// kernels (residual_sq), for the stored lanes only.
template <typename T, int L, bool PREV, bool RES, int K>
__device__ __forceinline__ void stream_step(int t, float4 (&R)[3][L], float4 (&bq)[Ring<T, L, RES>::NB],
                                            float4 (&TR)[3], FFAcc2 (&acc)[2], typename Store<T>::Vec *pr,
                                            typename Store<T>::Vec *br, Cursor<T> &cu, const StreamArgs<T> &a,
                                            int nsteps, int rows, T *out, T *outp)
{
    using V = typename Store<T>::Vec;
    constexpr int NB = Ring<T, L, RES>::NB;
    float4(&P)[L] = R[K % 3];
    float4(&Cur)[L] = R[(K + 1) % 3];
    float4(&N)[L] = R[(K + 2) % 3];
    if (t + kRP - 1 < nsteps) prefetch_row(cu, pr, br, (t + kRP - 1) & (kRP - 1), a);
    cp_async_commit();
    cp_async_wait<kRP - 1>();  // row t has landed
    N[0] = a.pin ? Store<T>::to_f4(pr[(t & (kRP - 1)) * 32]) : make_float4(0.f, 0.f, 0.f, 0.f);
    bq[K % NB] = Store<T>::to_f4(br[(t & (kRP - 1)) * 32]);  // b of row y, first used at the next step
    float4 top;
#pragma unroll
    for (int s = 0; s < L; ++s) {
        const float4 &bb = bq[(K + NB * L - s - 1) % NB];  // b of row y-s-1
        const float4 o = jacobi4(Cur[s], P[s], N[s], bb);   // level s+1, row y-s-1
        if (s + 1 < L) N[s + 1] = o;
        else top = o;
    }
    if (out && (unsigned)cu.st_rel < (unsigned)rows) *reinterpret_cast<V *>(out + cu.st_off) = Store<T>::from_f4(top);
    if (PREV && outp && (unsigned)(cu.st_rel + 1) < (unsigned)rows)
        *reinterpret_cast<V *>(outp + cu.st_off + a.ld) = Store<T>::from_f4(N[L - 1]);
    if constexpr (RES) {
        TR[K % 3] = top;                                  // level L, row y-L
        const float4 &c = TR[(K + 2) % 3];                // row y-L-1
        const float4 &up = TR[(K + 1) % 3];               // row y-L-2
        const float4 &bb = bq[(K + NB * (L + 1) - L - 1) % NB];  // b of row y-L-1
        const float lft = __shfl_up_sync(0xffffffffu, c.w, 1);
        const float rgt = __shfl_down_sync(0xffffffffu, c.x, 1);
        if (out && (unsigned)(cu.st_rel - 1) < (unsigned)rows) {
            residual_sq4(acc, bb, lft, c, rgt, up, top);
        }
    }
    cu.st_off += a.ld;
    cu.st_rel += 1;
}

template <typename T, int L, bool PREV, bool RES, int K>
__device__ __forceinline__ void stream_steps(int t, float4 (&R)[3][L], float4 (&bq)[Ring<T, L, RES>::NB],
                                             float4 (&TR)[3], FFAcc2 (&acc)[2], typename Store<T>::Vec *pr,
                                             typename Store<T>::Vec *br, Cursor<T> &cu, const StreamArgs<T> &a,
                                             int nsteps, int rows, T *out, T *outp)
{
    if constexpr (K < Ring<T, L, RES>::U) {
        if (t + K < nsteps) {
            stream_step<T, L, PREV, RES, K>(t + K, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
            stream_steps<T, L, PREV, RES, K + 1>(t, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
        }
    }
}

// Blocks per SM the register budget aims for: the deepest pipelines need
// more than 65536 / (3 * 128) registers per thread without spilling.
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

    V *pr = ring + lane;
    V *br = pr + kRP * 32;

    Cursor<T> cu;
    cu.ld_row = ybeg % a.h;
    if (cu.ld_row < 0) cu.ld_row += a.h;
    cu.gp = a.pin + (size_t)cu.ld_row * a.ld + cx;
    cu.gb = a.b + (size_t)cu.ld_row * a.ld + cx;
    cu.st_rel = -E - L;  // level L at step 0 is row ybeg - L = y0 - E - L
    cu.st_off = (long long)(y0 - E - L) * a.ld;
    T *out = st_lane ? a.pout + cx : nullptr;
    T *outp = (PREV && st_lane) ? a.pprev + cx : nullptr;
#pragma unroll
    for (int k = 0; k < kRP - 1; ++k) {
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

    for (int t = 0; t < nsteps; t += Ring<T, L, RES>::U)
        stream_steps<T, L, PREV, RES, 0>(t, R, bq, TR, acc, pr, br, cu, a, nsteps, rows, out, outp);
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
