// Batched form: an ensemble of independent simulations of uneven grid sizes
// advanced together, one persistent cooperative kernel per timestep.
//
// Each member runs the plain float32 step with viscosity 0 and an even
// diffusion count (where the reference's buffer roles reduce to: advect;
// divergence of the advected velocity; Jacobi from the previous final
// pressure; projection with the final pressure; image advection), with the
// same per-cell arithmetic as the single-simulation kernels (cells.cuh,
// sweep_stream.cuh), so every member's fields are bit-identical to a plain
// session's.
//
// The kernel walks the phases of the step (advect, divergence, fused sweep
// phases of L sweeps, residual checks, projection + image) with a grid
// barrier between phases. A phase is a task list over all members (row tasks,
// sweep strips x chunks, residual strips): warps take tasks in stride, and a
// member that has converged contributes no tasks to later sweep phases. All
// active members advance in lockstep, so the pressure plane a phase reads is
// (start plane + phase index) mod 2 for every member, and no per-member
// barrier is needed.
//
// The grid barrier spins with an iteration limit: on timeout it raises an
// error flag and every block returns, so a fault cannot hang the device.
// Cooperative launch guarantees all blocks are resident.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "cells.cuh"
#include "kernels.h"
#include "nvtx.h"
#include "pfs.h"
#include "reduce.cuh"
#include "sweep_stream.cuh"

namespace pfs {
namespace {

struct Member {
    int w, h, ld;
    float *u[2], *v[2];  // [0] current velocity, [1] advected
    float *p[2];         // pressure ping-pong (the refined form: the float32 correction e)
    float *b;            // divergence (the refined form: the correction's right-hand side r = b - A x)
    float *img[2];       // image ping-pong, c planes of ld*h each
    double *x;           // the refined form: FP64 pressure (else null)
    float *bx;           // the refined form: the divergence b (else null)
    int interval;        // the refined form: sweeps between refinements (f32r_refine_interval)
    int row_task0, nrow;     // row tasks (8 rows): advect, divergence, projection + image
    int sw_task0, nsx, nsy;  // fused sweep tasks
    int rs_task0, rsx, rsy;  // residual strip tasks
};

struct MemberState {
    int cur;      // plane holding the pressure iterate at the start of the step (the final one after it)
    int done;     // pressure solve finished this step
    int sweeps;   // sweeps of this step
    int checks;   // residual evaluations of this step
    int capped;
    int stalled;  // the refined form: the residual stopped falling
    double rel;   // last relative residual
    double bb;    // sum b^2
    // the refined form
    int zero_phase;    // sweep phase whose input correction is zero (the first after a refinement)
    int refine_start;  // sweeps of this step at the last refinement
    int refine;        // refine at the end of this check
    int refines;       // refinements of this step
    double last_rel;   // relative residual at the last refinement
};

struct EnsArgs {
    const Member *mem;
    MemberState *state;
    int nmem;
    const int *row_member, *sw_member, *rs_member;  // task -> member
    int nrow_tasks, nsw_tasks, nrs_tasks;
    double *row_part, *rs_part;  // per-task partial sums
    unsigned *bar_count, *bar_gen;
    int *err;
    int *active;  // members still iterating, one counter per check
    int *refining;  // the refined form: members refining, one counter per check
    float dt, gamma;
    double tol;
    int cap, check_every, chunk, channels, icur;
    int stall_block;  // test hook: this block leaves at once (-1: none); see pfs_ensemble_debug_stall_block
};

// Rows per task of the row phases (advection, divergence, refinement passes,
// projection + image). Each lane walks its columns of a row one after another
// with dependent gathers, so a task is latency-bound; one row per task spreads
// a 2048-row member over 2,048 tasks instead of 256 (at 8 rows per task its
// three row phases took about 2.8 ms per step, most warps idle at the barrier).
constexpr int kRowsPerTask = 1;
// Cells a lane computes at once in the gather-bound row phases (advection,
// projection with image advection).
constexpr int kCellsInFlight = 4;
constexpr long long kBarrierSpinLimit = 1LL << 24;  // ~1-2 s with the back-off below

// Grid-wide barrier with a bounded wait. Returns false (and every later call
// returns false at once) if any block gave up waiting.
__device__ bool grid_sync(const EnsArgs &a)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned *gen = a.bar_gen;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(a.bar_count, 1u) == gridDim.x - 1) {
            *a.bar_count = 0u;
            __threadfence();
            atomicAdd(a.bar_gen, 1u);
        } else {
            long long spins = 0;
            while (*gen == g) {
                if (*(volatile int *)a.err || ++spins > kBarrierSpinLimit) {
                    atomicExch(a.err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*(volatile int *)a.err) ok = 0;
    }
    __syncthreads();
    return ok != 0;
}

// Member state and per-task partials are written by one block and read by
// others later in the same launch: read them around L1 (which is not
// coherent across SMs).
template <typename T>
__device__ __forceinline__ T vload(const T &x) { return *(const volatile T *)&x; }

// A member's (cur, done) in one 8-byte load: every sweep and residual task
// reads both before it starts, and they change between phases.
static_assert(offsetof(MemberState, done) == offsetof(MemberState, cur) + sizeof(int) &&
                  offsetof(MemberState, cur) % 8 == 0 && alignof(MemberState) >= 8,
              "cur and done must share one aligned 8-byte word");
__device__ __forceinline__ int2 state_cur_done(const MemberState &ms)
{
    const unsigned long long v = *reinterpret_cast<const volatile unsigned long long *>(&ms.cur);
    return make_int2((int)(unsigned)(v & 0xffffffffull), (int)(unsigned)(v >> 32));  // little-endian: cur first
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// The refined form's FP64 pieces, with the arithmetic of the refined
// float32 session form (precision.cu: k_lp_refine, k_lp_damp, k_lp_project).
// r = b - A x for cell (i, j): b + xL + xR + xT + xB - 4 x, in FP64.
__device__ __forceinline__ double ref_residual(const double *__restrict__ x, const float *__restrict__ b, int ld, int w,
                                               int h, int i, int j)
{
    const size_t r = (size_t)j * ld;
    double q = __dadd_rn((double)__ldcg(b + r + i), __ldcg(x + r + wm(i, w)));
    q = __dadd_rn(q, __ldcg(x + r + wp(i, w)));
    q = __dadd_rn(q, __ldcg(x + (size_t)wm(j, h) * ld + i));
    q = __dadd_rn(q, __ldcg(x + (size_t)wp(j, h) * ld + i));
    return __fma_rn(-4.0, __ldcg(x + r + i), q);
}

// Projection with the FP64 pressure, ((x_R - x_L) rounded to float) * dt / 2,
// then image advection with the projected velocity (as project_image_cell).
__device__ __forceinline__ void ref_project_image_cell(const float *__restrict__ u, const float *__restrict__ v,
                                                       const double *__restrict__ x, float *__restrict__ uo,
                                                       float *__restrict__ vo, float *__restrict__ pout, int ld, int w,
                                                       int h, float dt, const float *__restrict__ img,
                                                       float *__restrict__ imgo, size_t plane, int c, int i, int j)
{
    const size_t r = (size_t)j * ld, o = r + i;
    const float dx = (float)(__ldcg(x + r + wp(i, w)) - __ldcg(x + r + wm(i, w)));
    const float dy = (float)(__ldcg(x + (size_t)wp(j, h) * ld + i) - __ldcg(x + (size_t)wm(j, h) * ld + i));
    const float un = fsub(u[o], fdiv(fmul(dx, dt), 2.0f));
    const float vn = fsub(v[o], fdiv(fmul(dy, dt), 2.0f));
    uo[o] = un;
    vo[o] = vn;
    pout[o] = (float)__ldcg(x + o);  // the pressure in float32, for downloads
    const Corners k = backtrace<0>(i, j, dt, dt, un, vn, (float)w, (float)h, w, h);
    const size_t r0 = (size_t)k.j0 * ld, r1 = (size_t)k.j1 * ld;
    for (int ch = 0; ch < c; ++ch) {
        const float *sp = img + ch * plane;
        imgo[ch * plane + o] = bilerp(k.sx, k.sy, sp[r0 + k.i0], sp[r0 + k.i1], sp[r1 + k.i0], sp[r1 + k.i1]);
    }
}

// One timestep of every member. REF: the refined float32 form (PFS_PREC_F32R):
// the sweeps iterate a float32 correction e on A e = r, r = b - A x, with the
// pressure x in FP64; at check points a member whose estimate
// ||r - A e|| / ||b|| is below the tolerance, or whose correction has run
// `interval` sweeps, is refined: the correction is filtered by
// PFS_START_DAMP_PASSES damped passes e += (r - A e) / 8, which remove the
// rounding noise it gathered in the modes Jacobi cannot damp (as the refined
// session form does), then x += e, r = b - A x, and the FP64 residual decides.
// Sum of a member's n per-task partials by one warp: lane l adds partials l,
// l + 32, ... in order, then the shuffle tree combines the lanes (a fixed
// order: the same sum every run); the total is on lane 0. One thread walking
// the partials serially cost about 0.8 ms per residual check for a 2048^2
// member (4,096 partials, one L2 round trip after another).
__device__ __forceinline__ double sum_partials(const double *p, int n, int lane)
{
    double s = 0.0;
    for (int t = lane; t < n; t += 32) s += __ldcg(p + t);
    return warp_sum(s);
}

template <int G, int L, bool REF>
__global__ void __launch_bounds__(128, 2) k_ensemble_step(EnsArgs a)
{
    extern __shared__ __align__(16) unsigned char sm_raw[];
    using V = Store<float>::Vec;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * 4 + wib, nw = gridDim.x * 4;
    V *ring = reinterpret_cast<V *>(sm_raw) + wib * Ring<float, L>::vecs_per_warp;
    // test hook: a block that never reaches the first barrier, so the others' bounded wait runs out
    if ((int)blockIdx.x == a.stall_block) return;
    const int ic = a.icur, io = 1 - a.icur;

    // advect every member: u[0], v[0] -> u[1], v[1]
    for (int t = gw; t < a.nrow_tasks; t += nw) {
        const Member &m = a.mem[a.row_member[t]];
        const int r0 = (t - m.row_task0) * kRowsPerTask, r1 = min(m.h, r0 + kRowsPerTask);
        // kCellsInFlight cells per lane at a time, all computed before any is
        // stored, so that their dependent gathers overlap (lanes past the
        // row's end compute its last cell and store nothing)
        for (int j = r0; j < r1; ++j)
            for (int i0 = lane; i0 < m.w; i0 += 32 * kCellsInFlight) {
                float ou[kCellsInFlight], ov[kCellsInFlight];
#pragma unroll
                for (int q = 0; q < kCellsInFlight; ++q)
                    advect_value(m.u[0], m.v[0], m.ld, m.w, m.h, a.dt, min(i0 + 32 * q, m.w - 1), j, ou[q], ov[q]);
#pragma unroll
                for (int q = 0; q < kCellsInFlight; ++q)
                    if (i0 + 32 * q < m.w) {
                        const size_t o = (size_t)j * m.ld + i0 + 32 * q;
                        m.u[1][o] = ou[q];
                        m.v[1][o] = ov[q];
                    }
            }
    }
    if (!grid_sync(a)) return;

    // divergence of the advected velocity (the refined form: into bx), b^2 per task
    for (int t = gw; t < a.nrow_tasks; t += nw) {
        const Member &m = a.mem[a.row_member[t]];
        const int r0 = (t - m.row_task0) * kRowsPerTask, r1 = min(m.h, r0 + kRowsPerTask);
        FFAcc acc;
        float *bo = REF ? m.bx : m.b;
        // kCellsInFlight cells per lane at a time (see the advection phase); b^2 is added in the
        // order of the cells, as one cell at a time would
        for (int j = r0; j < r1; ++j)
            for (int i0 = lane; i0 < m.w; i0 += 32 * kCellsInFlight) {
                float bv[kCellsInFlight];
#pragma unroll
                for (int q = 0; q < kCellsInFlight; ++q)
                    bv[q] = divergence_value(m.u[1], m.v[1], m.ld, m.w, m.h, a.gamma, min(i0 + 32 * q, m.w - 1), j);
#pragma unroll
                for (int q = 0; q < kCellsInFlight; ++q)
                    if (i0 + 32 * q < m.w) {
                        bo[(size_t)j * m.ld + i0 + 32 * q] = bv[q];
                        acc_square(acc, bv[q]);
                    }
            }
        const double s = warp_sum(acc.value());
        if (lane == 0) a.row_part[t] = s;
    }
    if (!grid_sync(a)) return;
    for (int k = gw; k < a.nmem; k += nw) {
        const Member &m = a.mem[k];
        const double s = sum_partials(a.row_part + m.row_task0, m.nrow, lane);
        if (lane != 0) continue;
        volatile MemberState &ms = a.state[k];
        ms.bb = s;
        ms.done = 0;
        ms.sweeps = 0;
        ms.checks = 0;
        ms.capped = 0;
        ms.stalled = 0;
        if (REF) {
            ms.cur = 0;
            ms.zero_phase = 0;
            ms.refine_start = 0;
            ms.refine = 0;
            ms.refines = 0;
        }
    }
    if (!grid_sync(a)) return;

    if (REF) {
        // the residual of the starting pressure (the previous step's x): r = b - A x into m.b
        for (int t = gw; t < a.nrow_tasks; t += nw) {
            const Member &m = a.mem[a.row_member[t]];
            const int r0 = (t - m.row_task0) * kRowsPerTask, r1 = min(m.h, r0 + kRowsPerTask);
            double acc = 0.0;
            for (int j = r0; j < r1; ++j)
                for (int i = lane; i < m.w; i += 32) {
                    const double q = ref_residual(m.x, m.bx, m.ld, m.w, m.h, i, j);
                    m.b[(size_t)j * m.ld + i] = (float)q;
                    acc = __fma_rn(q, q, acc);
                }
            acc = warp_sum(acc);
            if (lane == 0) a.row_part[t] = acc;
        }
        if (!grid_sync(a)) return;
        for (int k = gw; k < a.nmem; k += nw) {
            const Member &m = a.mem[k];
            const double rr = sum_partials(a.row_part + m.row_task0, m.nrow, lane);
            if (lane != 0) continue;
            volatile MemberState &ms = a.state[k];
            const double bb = ms.bb;
            const double rel = bb > 0.0 ? __dsqrt_rn(rr) / __dsqrt_rn(bb) : __dsqrt_rn(rr);
            ms.rel = rel;
            ms.last_rel = rel;
            ms.checks = 1;
            if (rel <= a.tol) ms.done = 1;  // already converged: no sweeps
        }
        if (!grid_sync(a)) return;
    }

    // pressure: phases of L fused sweeps; residual checks every check_every sweeps and at the cap
    int phase = 0, check = 0;
    // The member state a sweep task reads (plane index, done flag, and for the
    // refined form the phase whose correction starts at zero) changes only in
    // the check below, so the warp keeps its first task's reading from one
    // check to the next instead of an L2 round trip per phase.
    int c_mi = 0, c_cur = 0, c_done = 0, c_zero = -1;
    bool cached = false;
    for (int s = 0; s < a.cap;) {
        for (int t = gw; t < a.nsw_tasks; t += nw) {
            int mi, cur, dn, zp;
            if (t == gw && cached) {
                mi = c_mi, cur = c_cur, dn = c_done, zp = c_zero;
            } else {
                mi = a.sw_member[t];
                const int2 cd = state_cur_done(a.state[mi]);  // one L2 round trip for both words
                cur = cd.x;
                dn = cd.y;
                zp = REF ? vload(a.state[mi].zero_phase) : -1;
                if (t == gw) c_mi = mi, c_cur = cur, c_done = dn, c_zero = zp, cached = true;
            }
            if (dn) continue;
            const Member &m = a.mem[mi];
            StreamArgs<float> sa;
            sa.pin = (REF && zp == phase) ? nullptr : m.p[(cur + phase) & 1];
            sa.pout = m.p[(cur + phase + 1) & 1];
            sa.b = m.b;
            sa.pprev = nullptr;
            sa.done = nullptr;
            sa.ld = m.ld;
            sa.w = m.w;
            sa.h = m.h;
            sa.nsx = m.nsx;
            sa.nwork = m.nsx * m.nsy;
            sa.chunk = a.chunk;
            stream_task<float, G, L, false>(sa, t - m.sw_task0, lane, ring);
        }
        ++phase;
        s += L;
        if (!grid_sync(a)) return;
        if (s % a.check_every != 0 && s != a.cap) continue;
        cached = false;  // the check may change done, cur and zero_phase
        for (int t = gw; t < a.nrs_tasks; t += nw) {
            const int mi = a.rs_member[t];
            const int2 cd = state_cur_done(a.state[mi]);  // one L2 round trip for both words
            if (cd.y) continue;
            const int cur = cd.x;
            const Member &m = a.mem[mi];
            const int q = t - m.rs_task0, sx = q % m.rsx, sy = q / m.rsx;
            const int y0 = sy * 8, y1 = min(m.h, y0 + 8);
            FFAcc2 acc[2];
            residual_strip_task(m.p[(cur + phase) & 1], m.b, m.ld, m.w, m.h, sx, y0, y1, lane, acc, nullptr);
            const double v = warp_sum(acc[0].value() + acc[1].value());
            if (lane == 0) a.rs_part[t] = v;
        }
        if (!grid_sync(a)) return;
        for (int k = gw; k < a.nmem; k += nw) {
            volatile MemberState &ms = a.state[k];
            if (__shfl_sync(0xffffffffu, ms.done, 0)) continue;  // the warp takes lane 0's reading
            const Member &m = a.mem[k];
            const double rr = sum_partials(a.rs_part + m.rs_task0, m.rsx * m.rsy, lane);
            if (lane != 0) continue;
            const double bb = ms.bb;
            const double rel = bb > 0.0 ? __dsqrt_rn(rr) / __dsqrt_rn(bb) : __dsqrt_rn(rr);
            ms.checks = ms.checks + 1;
            if (REF) {
                // the estimate of x + e's residual: refine when it meets the tolerance, when the
                // correction has run its interval, or at the cap
                if (rel <= 0.999 * a.tol || s - ms.refine_start >= m.interval || s == a.cap) {
                    ms.refine = 1;
                    atomicAdd(a.refining + check, 1);
                }
                atomicAdd(a.active + check, 1);
                continue;
            }
            ms.rel = rel;
            if (rel <= a.tol || s == a.cap) {
                ms.done = 1;
                ms.sweeps = s;
                ms.capped = (a.tol > 0.0 && rel > a.tol) ? 1 : 0;
                ms.cur = (ms.cur + phase) & 1;
            } else {
                atomicAdd(a.active + check, 1);
            }
        }
        if (!grid_sync(a)) return;
        if (REF && *(volatile int *)(a.refining + check) > 0) {
            // the filter: damped passes e += (r - A e) / 8 on the correction, through the other
            // correction plane (an even count ends back in e's plane)
            for (int pass = 0; pass < PFS_START_DAMP_PASSES; ++pass) {
                for (int t = gw; t < a.nrow_tasks; t += nw) {
                    const int mi = a.row_member[t];
                    if (!vload(a.state[mi].refine)) continue;
                    const Member &m = a.mem[mi];
                    const int ep = (vload(a.state[mi].cur) + phase) & 1;
                    const float *ei = m.p[(pass & 1) ? 1 - ep : ep];
                    float *eo = m.p[(pass & 1) ? ep : 1 - ep];
                    const int r0 = (t - m.row_task0) * kRowsPerTask, r1 = min(m.h, r0 + kRowsPerTask);
                    for (int j = r0; j < r1; ++j)
                        for (int i = lane; i < m.w; i += 32) {
                            const size_t r = (size_t)j * m.ld;
                            const float q = fsub(fadd(fadd(fadd(fadd(__ldcg(m.b + r + i), __ldcg(ei + r + wm(i, m.w))),
                                                                __ldcg(ei + r + wp(i, m.w))),
                                                           __ldcg(ei + (size_t)wm(j, m.h) * m.ld + i)),
                                                      __ldcg(ei + (size_t)wp(j, m.h) * m.ld + i)),
                                                 fmul(4.0f, __ldcg(ei + r + i)));
                            eo[r + i] = fadd(__ldcg(ei + r + i), fmul(q, 0.125f));
                        }
                }
                if (!grid_sync(a)) return;
            }
            // x += e for the refining members
            for (int t = gw; t < a.nrow_tasks; t += nw) {
                const int mi = a.row_member[t];
                if (!vload(a.state[mi].refine)) continue;
                const Member &m = a.mem[mi];
                const float *e = m.p[(vload(a.state[mi].cur) + phase) & 1];
                const int r0 = (t - m.row_task0) * kRowsPerTask, r1 = min(m.h, r0 + kRowsPerTask);
                for (int j = r0; j < r1; ++j)
                    for (int i = lane; i < m.w; i += 32) {
                        const size_t o = (size_t)j * m.ld + i;
                        m.x[o] = __dadd_rn(__ldcg(m.x + o), (double)__ldcg(e + o));
                    }
            }
            if (!grid_sync(a)) return;
            // r = b - A x, sum r^2 per task
            for (int t = gw; t < a.nrow_tasks; t += nw) {
                const int mi = a.row_member[t];
                if (!vload(a.state[mi].refine)) continue;
                const Member &m = a.mem[mi];
                const int r0 = (t - m.row_task0) * kRowsPerTask, r1 = min(m.h, r0 + kRowsPerTask);
                double acc = 0.0;
                for (int j = r0; j < r1; ++j)
                    for (int i = lane; i < m.w; i += 32) {
                        const double q = ref_residual(m.x, m.bx, m.ld, m.w, m.h, i, j);
                        m.b[(size_t)j * m.ld + i] = (float)q;
                        acc = __fma_rn(q, q, acc);
                    }
                acc = warp_sum(acc);
                if (lane == 0) a.row_part[t] = acc;
            }
            if (!grid_sync(a)) return;
            for (int k = gw; k < a.nmem; k += nw) {
                volatile MemberState &ms = a.state[k];
                if (__shfl_sync(0xffffffffu, ms.done || !ms.refine, 0)) continue;  // lane 0's reading
                const Member &m = a.mem[k];
                const double rr = sum_partials(a.row_part + m.row_task0, m.nrow, lane);
                if (lane != 0) continue;
                const double bb = ms.bb;
                const double rel = bb > 0.0 ? __dsqrt_rn(rr) / __dsqrt_rn(bb) : __dsqrt_rn(rr);
                const bool full = s - ms.refine_start >= m.interval;
                ms.rel = rel;
                ms.refine = 0;
                ms.refines = ms.refines + 1;
                if (rel <= a.tol || s == a.cap || (full && !(rel < kStallGain * ms.last_rel))) {
                    ms.done = 1;
                    ms.sweeps = s;
                    ms.capped = rel > a.tol && s == a.cap ? 1 : 0;
                    ms.stalled = rel > a.tol && s != a.cap ? 1 : 0;
                    atomicSub(a.active + check, 1);
                } else {
                    ms.zero_phase = phase;  // the next sweep phase starts the new correction from zero
                    ms.refine_start = s;
                    ms.last_rel = rel;
                }
            }
            if (!grid_sync(a)) return;
        }
        if (*(volatile int *)(a.active + check) == 0) break;
        ++check;
    }

    // projection with the final pressure, then image advection
    for (int t = gw; t < a.nrow_tasks; t += nw) {
        const int mi = a.row_member[t];
        const Member &m = a.mem[mi];
        const size_t plane = (size_t)m.ld * m.h;
        const int r0 = (t - m.row_task0) * kRowsPerTask, r1 = min(m.h, r0 + kRowsPerTask);
        if (REF) {
            for (int j = r0; j < r1; ++j)
                for (int i = lane; i < m.w; i += 32)
                    ref_project_image_cell(m.u[1], m.v[1], m.x, m.u[0], m.v[0], m.p[0], m.ld, m.w, m.h, a.dt,
                                           m.img[ic], m.img[io], plane, a.channels, i, j);
        } else {
            // as project_image_cell, kCellsInFlight cells per lane at a time (see
            // the advection phase)
            const float *pf = m.p[vload(a.state[mi].cur)];
            for (int j = r0; j < r1; ++j)
                for (int i0 = lane; i0 < m.w; i0 += 32 * kCellsInFlight) {
                    float un[kCellsInFlight], vn[kCellsInFlight];
                    Corners kc[kCellsInFlight];
#pragma unroll
                    for (int q = 0; q < kCellsInFlight; ++q)
                        project_cell<0>(m.u[1], m.v[1], pf, m.ld, m.w, m.h, a.dt, min(i0 + 32 * q, m.w - 1), j, un[q],
                                        vn[q]);
#pragma unroll
                    for (int q = 0; q < kCellsInFlight; ++q) {
                        if (i0 + 32 * q < m.w) {
                            const size_t o = (size_t)j * m.ld + i0 + 32 * q;
                            m.u[0][o] = un[q];
                            m.v[0][o] = vn[q];
                        }
                        kc[q] = backtrace<0>(min(i0 + 32 * q, m.w - 1), j, a.dt, a.dt, un[q], vn[q], (float)m.w,
                                             (float)m.h, m.w, m.h);
                    }
                    for (int ch = 0; ch < a.channels; ++ch) {
                        const float *sp = m.img[ic] + ch * plane;
                        float *dp = m.img[io] + ch * plane;
                        float val[kCellsInFlight];
#pragma unroll
                        for (int q = 0; q < kCellsInFlight; ++q) {
                            const size_t r0k = (size_t)kc[q].j0 * m.ld, r1k = (size_t)kc[q].j1 * m.ld;
                            val[q] = bilerp(kc[q].sx, kc[q].sy, sp[r0k + kc[q].i0], sp[r0k + kc[q].i1],
                                            sp[r1k + kc[q].i0], sp[r1k + kc[q].i1]);
                        }
#pragma unroll
                        for (int q = 0; q < kCellsInFlight; ++q)
                            if (i0 + 32 * q < m.w) dp[(size_t)j * m.ld + i0 + 32 * q] = val[q];
                    }
                }
        }
    }
}

}  // namespace

// =============================================================================================
// Host side

struct Ensemble {
    int n = 0, c = 0;
    pfs_params prm{};
    cudaStream_t st = nullptr;
    std::vector<int> w, h, ld;
    std::vector<size_t> off;  // float offset of each member's planes
    float *mem = nullptr;
    size_t floats = 0;
    Member *dmem = nullptr;
    MemberState *dstate = nullptr;
    int *dtasks = nullptr;
    double *dparts = nullptr;
    unsigned *dbar = nullptr;  // count, gen
    int *derr = nullptr, *dactive = nullptr;
    std::vector<Member> hmem;
    int nrow = 0, nsw = 0, nrs = 0;
    int halo = 8, levels = 8, chunk = 32;
    int grid = 0;
    int icur = 0;
    long long steps = 0, total_sweeps = 0, cap_hits = 0;
    float *stage = nullptr;
    size_t stage_bytes = 0;
    float *snap = nullptr;  // state copy for pfs_ensemble_snapshot
    MemberState *snap_state = nullptr;
    int snap_icur = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool graphs_ok = true;
    int *dsel = nullptr;  // member list of pfs_ensemble_image_stats (n ints)
    int stall_block = -1;  // test hook for the next step (pfs_ensemble_debug_stall_block)
    bool refined = false;  // PFS_PREC_F32R members
};

namespace {

int ens_fail(int code, const char *msg)
{
    cudaGetLastError();  // the status carries the error; do not leave it pending for the caller's next CUDA call
    return record_error(code, msg);
}

#define ECK(x)                                                                 \
    do {                                                                       \
        cudaError_t e_ = (x);                                                  \
        if (e_ != cudaSuccess) return ens_fail(PFS_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

int build_tasks(Ensemble &E)
{
    std::vector<int> rowm, swm, rsm;
    const int ow = 128 - 2 * E.halo;
    for (int k = 0; k < E.n; ++k) {
        Member &m = E.hmem[k];
        m.row_task0 = (int)rowm.size();
        m.nrow = (m.h + kRowsPerTask - 1) / kRowsPerTask;
        for (int t = 0; t < m.nrow; ++t) rowm.push_back(k);
        m.sw_task0 = (int)swm.size();
        m.nsx = (m.w + ow - 1) / ow;
        m.nsy = (m.h + E.chunk - 1) / E.chunk;
        for (int t = 0; t < m.nsx * m.nsy; ++t) swm.push_back(k);
        m.rs_task0 = (int)rsm.size();
        m.rsx = (m.w + 127) / 128;
        m.rsy = (m.h + 7) / 8;
        for (int t = 0; t < m.rsx * m.rsy; ++t) rsm.push_back(k);
    }
    E.nrow = (int)rowm.size();
    E.nsw = (int)swm.size();
    E.nrs = (int)rsm.size();
    if (E.dtasks) cudaFree(E.dtasks);
    if (E.dparts) cudaFree(E.dparts);
    E.dtasks = nullptr;
    E.dparts = nullptr;
    ECK(cudaMalloc(&E.dtasks, sizeof(int) * (E.nrow + E.nsw + E.nrs)));
    ECK(cudaMemcpy(E.dtasks, rowm.data(), sizeof(int) * E.nrow, cudaMemcpyHostToDevice));
    ECK(cudaMemcpy(E.dtasks + E.nrow, swm.data(), sizeof(int) * E.nsw, cudaMemcpyHostToDevice));
    ECK(cudaMemcpy(E.dtasks + E.nrow + E.nsw, rsm.data(), sizeof(int) * E.nrs, cudaMemcpyHostToDevice));
    ECK(cudaMalloc(&E.dparts, sizeof(double) * (E.nrow + E.nrs)));
    ECK(cudaMemcpy(E.dmem, E.hmem.data(), sizeof(Member) * E.n, cudaMemcpyHostToDevice));
    return PFS_OK;
}

template <int G, int L, bool REF>
cudaError_t launch_ens(const EnsArgs &a, int grid, cudaStream_t st)
{
    constexpr int smem = Ring<float, L>::bytes_per_block;
    static std::atomic<unsigned long long> attr_done{0};  // per instantiation and device
    const cudaError_t ea = smem_limit_once(k_ensemble_step<G, L, REF>, smem, attr_done);
    if (ea != cudaSuccess) return ea;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr_coop;
    attr_coop.id = cudaLaunchAttributeCooperative;
    attr_coop.val.cooperative = 1;
    cfg.attrs = &attr_coop;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_ensemble_step<G, L, REF>, a);
    if (e == cudaSuccess) launched();
    return e;
}

int grid_for(Ensemble &E)
{
    int dev, sms, per = 0;
    ECK(cudaGetDevice(&dev));
    ECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    auto occ = [&](auto kernel, int smem) -> cudaError_t {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 128, smem);
    };
    if (E.levels == 8)
        ECK(E.refined ? occ(k_ensemble_step<8, 8, true>, Ring<float, 8>::bytes_per_block)
                      : occ(k_ensemble_step<8, 8, false>, Ring<float, 8>::bytes_per_block));
    else
        ECK(E.refined ? occ(k_ensemble_step<4, 4, true>, Ring<float, 4>::bytes_per_block)
                      : occ(k_ensemble_step<4, 4, false>, Ring<float, 4>::bytes_per_block));
    if (per < 1) return ens_fail(PFS_ERR_UNSUPPORTED, "ensemble kernel does not fit on an SM");
    E.grid = per * sms;
    return PFS_OK;
}

EnsArgs make_args(Ensemble &E, int icur)
{
    EnsArgs a;
    a.mem = E.dmem;
    a.state = E.dstate;
    a.nmem = E.n;
    a.row_member = E.dtasks;
    a.sw_member = E.dtasks + E.nrow;
    a.rs_member = E.dtasks + E.nrow + E.nsw;
    a.nrow_tasks = E.nrow;
    a.nsw_tasks = E.nsw;
    a.nrs_tasks = E.nrs;
    a.row_part = E.dparts;
    a.rs_part = E.dparts + E.nrow;
    a.bar_count = E.dbar;
    a.bar_gen = E.dbar + 1;
    a.err = E.derr;
    a.active = E.dactive;
    a.refining = E.dactive + E.prm.max_iters / 4 + 2;
    a.dt = E.prm.dt;
    a.gamma = (float)(-1.0 / (double)E.prm.dt);
    a.tol = E.prm.tol > 0.0 ? E.prm.tol : -1.0;
    a.cap = E.prm.max_iters;
    a.check_every = E.prm.check_every > 0 ? E.prm.check_every : E.prm.max_iters;
    a.chunk = E.chunk;
    a.channels = E.c;
    a.stall_block = E.stall_block;
    a.icur = icur;
    return a;
}

int enqueue_step(Ensemble &E, int icur, cudaStream_t st)
{
    const int nchecks = E.prm.max_iters / E.levels + 2;
    const EnsArgs a = make_args(E, icur);
    ECK(cudaMemsetAsync(a.active, 0, sizeof(int) * nchecks, st));
    if (E.refined) ECK(cudaMemsetAsync(a.refining, 0, sizeof(int) * nchecks, st));
    ECK(cudaMemsetAsync(E.dbar, 0, sizeof(unsigned) * 2, st));
    cudaError_t e;
    if (E.refined) e = E.levels == 8 ? launch_ens<8, 8, true>(a, E.grid, st) : launch_ens<4, 4, true>(a, E.grid, st);
    else e = E.levels == 8 ? launch_ens<8, 8, false>(a, E.grid, st) : launch_ens<4, 4, false>(a, E.grid, st);
    ECK(e);
    return PFS_OK;
}

void drop_graphs(Ensemble &E)
{
    for (auto &g : E.graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

// One CUDA graph per image parity: the step's two memsets and the kernel.
int build_graphs(Ensemble &E)
{
    drop_graphs(E);
    if (!E.graphs_ok) return PFS_OK;
    struct NoStall {  // the captured steps never carry the test hook
        Ensemble &e;
        int saved;
        explicit NoStall(Ensemble &x) : e(x), saved(x.stall_block) { e.stall_block = -1; }
        ~NoStall() { e.stall_block = saved; }
    } no_stall(E);
    cudaStream_t cs;
    ECK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    for (int par = 0; par < 2; ++par) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        int rc = PFS_OK;
        if (e == cudaSuccess) rc = enqueue_step(E, par, cs);
        const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (e == cudaSuccess && rc == PFS_OK && e2 == cudaSuccess) e = cudaGraphInstantiate(&E.graph[par], g, 0);
        else e = cudaErrorStreamCaptureUnsupported;
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {  // no graph support for this launch: run it directly
            cudaGetLastError();
            E.graphs_ok = false;
            drop_graphs(E);
            break;
        }
    }
    cudaStreamDestroy(cs);
    return PFS_OK;
}

}  // namespace

}  // namespace pfs

using pfs::Ensemble;

extern "C" {

int pfs_ensemble_create(pfs_ensemble **out, int n, const int *w, const int *h, int channels, const pfs_params *params,
                        void *stream)
{
    if (!out || n <= 0 || !w || !h || !params || channels < 0)
        return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad ensemble arguments");
    *out = nullptr;
    const pfs_params &p = *params;
    if (!(p.dt > 0.0f) || p.viscosity != 0.0f || p.diffuse_iters < 2 || p.diffuse_iters % 2 ||
        p.boundary != PFS_BOUNDARY_PERIODIC || (p.precision != PFS_PREC_F32 && p.precision != PFS_PREC_F32R))
        return pfs::record_error(PFS_ERR_UNSUPPORTED,
                                 "ensembles run float32 (F32 or F32R) steps with viscosity 0 and an even diffusion "
                                 "count >= 2");
    if (p.precision == PFS_PREC_F32R && !(p.tol > 0.0))
        return pfs::record_error(PFS_ERR_UNSUPPORTED, "refined ensembles iterate to a tolerance (tol > 0)");
    const int L = p.fuse_depth > 0 ? p.fuse_depth : 8;
    if (L != 4 && L != 8) return pfs::record_error(PFS_ERR_UNSUPPORTED, "ensemble fuse_depth must be 4 or 8");
    if (p.max_iters <= 0 || p.max_iters % L || (p.check_every > 0 && p.check_every % L))
        return pfs::record_error(PFS_ERR_UNSUPPORTED, "ensemble sweep cap and check interval must be multiples of "
                                                      "the fuse depth");
    for (int k = 0; k < n; ++k) {
        if (w[k] <= 0 || h[k] <= 0 || w[k] % 4)
            return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "member widths must be positive multiples of 4");
        // the sweep task addresses rows by 32-bit offsets in vectors of four cells (its row pitch is
        // the width rounded up to 32)
        if ((long long)h[k] * ((w[k] + 31) / 32 * 32 / 4) >= (1LL << 31))
            return pfs::record_error(PFS_ERR_UNSUPPORTED, "member planes must hold fewer than 2^33 cells");
    }
    Ensemble *E = new (std::nothrow) Ensemble();
    if (!E) return pfs::record_error(PFS_ERR_CUDA, "out of host memory");
    E->n = n;
    E->c = channels;
    E->prm = p;
    E->st = (cudaStream_t)stream;
    E->levels = L;
    E->halo = L == 8 ? 8 : 4;
    E->chunk = p.chunk_rows > 0 ? p.chunk_rows : 32;
    E->refined = p.precision == PFS_PREC_F32R;
    // per member: u, v x2, p x2, b, image x2 (c planes each); refined: x (FP64, two floats per cell), bx
    const int extra = E->refined ? 3 : 0;
    size_t tot = 0;
    E->hmem.resize(n);
    for (int k = 0; k < n; ++k) {
        E->w.push_back(w[k]);
        E->h.push_back(h[k]);
        const int ld = (w[k] + 31) / 32 * 32;
        E->ld.push_back(ld);
        E->off.push_back(tot);
        tot += (size_t)ld * h[k] * (7 + 2 * channels + extra);
    }
    E->floats = tot;
    int rc = PFS_OK;
    auto bail = [&](int code) {
        pfs_ensemble_destroy(reinterpret_cast<pfs_ensemble *>(E));
        return code;
    };
    if (cudaMalloc(&E->mem, tot * sizeof(float)) != cudaSuccess || cudaMemset(E->mem, 0, tot * sizeof(float)))
        return bail(pfs::record_error(PFS_ERR_CUDA, "ensemble allocation failed"));
    for (int k = 0; k < n; ++k) {
        pfs::Member &m = E->hmem[k];
        m.w = w[k];
        m.h = h[k];
        m.ld = E->ld[k];
        const size_t P = (size_t)m.ld * m.h;
        float *q = E->mem + E->off[k];
        m.u[0] = q;
        m.u[1] = q + P;
        m.v[0] = q + 2 * P;
        m.v[1] = q + 3 * P;
        m.p[0] = q + 4 * P;
        m.p[1] = q + 5 * P;
        m.b = q + 6 * P;
        m.img[0] = q + 7 * P;
        m.img[1] = q + (7 + channels) * P;
        m.x = nullptr;
        m.bx = nullptr;
        m.interval = 0;
        if (E->refined) {  // P is a multiple of 32 floats: the FP64 planes stay 8-byte aligned
            float *r = q + (7 + 2 * channels) * P;
            m.x = reinterpret_cast<double *>(r);
            m.bx = r + 2 * P;
            m.interval = pfs::f32r_refine_interval(std::max(m.w, m.h), p.check_every > 0 ? p.check_every : p.max_iters);
        }
    }
    if (cudaMalloc(&E->dmem, sizeof(pfs::Member) * n) != cudaSuccess ||
        cudaMalloc(&E->dstate, sizeof(pfs::MemberState) * n) != cudaSuccess ||
        cudaMemset(E->dstate, 0, sizeof(pfs::MemberState) * n) != cudaSuccess ||
        cudaMalloc(&E->dbar, 2 * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&E->derr, sizeof(int)) != cudaSuccess || cudaMemset(E->derr, 0, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&E->dactive, 2 * sizeof(int) * (p.max_iters / 4 + 2)) != cudaSuccess)  // any fuse depth (>= 4)
        return bail(pfs::record_error(PFS_ERR_CUDA, "ensemble allocation failed"));
    if ((rc = pfs::build_tasks(*E)) != PFS_OK) return bail(rc);
    if ((rc = pfs::grid_for(*E)) != PFS_OK) return bail(rc);
    *out = reinterpret_cast<pfs_ensemble *>(E);
    return PFS_OK;
}

int pfs_ensemble_destroy(pfs_ensemble *e)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E) return PFS_OK;
    cudaStreamSynchronize(E->st);
    pfs::drop_graphs(*E);
    cudaFree(E->mem);
    cudaFree(E->dmem);
    cudaFree(E->dstate);
    cudaFree(E->dtasks);
    cudaFree(E->dparts);
    cudaFree(E->dbar);
    cudaFree(E->derr);
    cudaFree(E->dactive);
    cudaFree(E->stage);
    cudaFree(E->snap);
    cudaFree(E->snap_state);
    cudaFree(E->dsel);
    delete E;
    return PFS_OK;
}

int pfs_ensemble_snapshot(pfs_ensemble *e, int restore)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "null ensemble");
    const size_t bytes = E->floats * sizeof(float), sbytes = sizeof(pfs::MemberState) * E->n;
    cudaError_t r = cudaSuccess;
    if (!restore) {
        if (!E->snap) r = cudaMalloc(&E->snap, bytes);
        if (r == cudaSuccess && !E->snap_state) r = cudaMalloc(&E->snap_state, sbytes);
        if (r == cudaSuccess) r = cudaMemcpyAsync(E->snap, E->mem, bytes, cudaMemcpyDeviceToDevice, E->st);
        if (r == cudaSuccess) r = cudaMemcpyAsync(E->snap_state, E->dstate, sbytes, cudaMemcpyDeviceToDevice, E->st);
        E->snap_icur = E->icur;
    } else {
        if (!E->snap) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "no snapshot taken");
        r = cudaMemcpyAsync(E->mem, E->snap, bytes, cudaMemcpyDeviceToDevice, E->st);
        if (r == cudaSuccess) r = cudaMemcpyAsync(E->dstate, E->snap_state, sbytes, cudaMemcpyDeviceToDevice, E->st);
        E->icur = E->snap_icur;
    }
    if (r == cudaSuccess) r = cudaStreamSynchronize(E->st);
    return r == cudaSuccess ? PFS_OK : pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(r));
}

static int ens_stage(Ensemble *E, size_t bytes)
{
    if (E->stage_bytes >= bytes) return PFS_OK;
    cudaFree(E->stage);
    E->stage = nullptr;
    E->stage_bytes = 0;
    if (cudaMalloc(&E->stage, bytes) != cudaSuccess) return pfs::record_error(PFS_ERR_CUDA, "staging allocation");
    E->stage_bytes = bytes;
    return PFS_OK;
}

namespace pfs {
namespace {

// Pointwise ensemble statistics of the image: for each pixel and channel, the
// mean and the population variance over the listed members (same grid),
// accumulated in FP64 in list order (deterministic). One thread per pixel;
// member planes are read coalesced, the outputs are interleaved (h, w, c).
__global__ void k_image_stats(const Member *__restrict__ mem, const int *__restrict__ sel, int n, int icur, int c,
                              int w, int h, float *__restrict__ mean, float *__restrict__ var)
{
    const int ld = mem[sel[0]].ld;
    const size_t plane = (size_t)ld * h;
    const double inv = 1.0 / (double)n;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < w * h; e += gridDim.x * blockDim.x) {
        const int i = e % w, j = e / w;
        const size_t o = (size_t)j * ld + i;
        for (int ch = 0; ch < c; ++ch) {
            double s = 0.0, s2 = 0.0;
            for (int k = 0; k < n; ++k) {
                const double x = (double)mem[sel[k]].img[icur][ch * plane + o];
                s += x;
                s2 = fma(x, x, s2);
            }
            const double m = s * inv;
            mean[(size_t)e * c + ch] = (float)m;
            var[(size_t)e * c + ch] = (float)fmax(fma(-m, m, s2 * inv), 0.0);
        }
    }
}

}  // namespace
}  // namespace pfs

#define SCK(x)                                                                  \
    do {                                                                        \
        cudaError_t e_ = (x);                                                   \
        if (e_ != cudaSuccess) {                                                \
            cudaGetLastError();                                                 \
            return pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(e_));     \
        }                                                                       \
    } while (0)

int pfs_ensemble_image_stats(pfs_ensemble *e, const int *members, int n, float *mean, float *var, int where)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E || !members || n <= 0 || n > E->n || !mean || !var || (where != PFS_HOST && where != PFS_DEVICE))
        return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad image statistics arguments");
    if (E->c == 0) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "the ensemble has no image");
    for (int k = 0; k < n; ++k) {
        const int m = members[k];
        if (m < 0 || m >= E->n) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "member index out of range");
        if (E->w[m] != E->w[members[0]] || E->h[m] != E->h[members[0]])
            return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "image statistics need members of one grid size");
    }
    const int w = E->w[members[0]], h = E->h[members[0]];
    const size_t count = (size_t)w * h * E->c;
    if (!E->dsel) SCK(cudaMalloc(&E->dsel, sizeof(int) * E->n));
    SCK(cudaMemcpyAsync(E->dsel, members, sizeof(int) * n, cudaMemcpyHostToDevice, E->st));
    float *M = mean, *V = var;
    if (where == PFS_HOST) {
        const int rc = ens_stage(E, 2 * count * sizeof(float));
        if (rc != PFS_OK) return rc;
        M = E->stage;
        V = E->stage + count;
    }
    const int blocks = (int)std::min<size_t>(((size_t)w * h + 255) / 256, 152 * 8);
    pfs::k_image_stats<<<blocks, 256, 0, E->st>>>(E->dmem, E->dsel, n, E->icur, E->c, w, h, M, V);
    SCK(pfs::launched());
    if (where == PFS_HOST) {
        SCK(cudaMemcpyAsync(mean, M, count * sizeof(float), cudaMemcpyDeviceToHost, E->st));
        SCK(cudaMemcpyAsync(var, V, count * sizeof(float), cudaMemcpyDeviceToHost, E->st));
    }
    SCK(cudaStreamSynchronize(E->st));  // also keeps the member list alive until the kernel has read it
    return PFS_OK;
}

int pfs_ensemble_upload(pfs_ensemble *e, int k, const float *vp, const float *tmp, const float *image, int where)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E || k < 0 || k >= E->n || !vp || !tmp || (E->c > 0 && !image))
        return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad ensemble upload arguments");
    const pfs::Member &m = E->hmem[k];
    const size_t nv = (size_t)m.w * m.h * 4, ni = (size_t)m.w * m.h * E->c;
    const float *A = vp, *B = tmp, *I = image;
    if (where == PFS_HOST) {
        int rc = ens_stage(E, (2 * nv + ni) * sizeof(float));
        if (rc != PFS_OK) return rc;
        cudaMemcpyAsync(E->stage, vp, nv * 4, cudaMemcpyHostToDevice, E->st);
        cudaMemcpyAsync(E->stage + nv, tmp, nv * 4, cudaMemcpyHostToDevice, E->st);
        if (ni) cudaMemcpyAsync(E->stage + 2 * nv, image, ni * 4, cudaMemcpyHostToDevice, E->st);
        A = E->stage;
        B = E->stage + nv;
        I = E->stage + 2 * nv;
    }
    cudaError_t r = pfs::launch_split_velocity(A, m.u[0], m.v[0], m.ld, m.w, m.h, E->st);
    if (r == cudaSuccess) r = pfs::launch_split_channel(B, 2, 4, m.p[0], m.ld, m.w, m.h, E->st);
    if (r == cudaSuccess && E->refined) r = pfs::launch_widen(m.p[0], m.x, (size_t)m.ld * m.h, E->st);
    if (r == cudaSuccess && E->c > 0)
        r = pfs::launch_split_image(I, m.img[E->icur], (size_t)m.ld * m.h, m.ld, m.w, m.h, E->c, E->st);
    pfs::MemberState ms{};
    if (r == cudaSuccess) r = cudaMemcpyAsync(E->dstate + k, &ms, sizeof ms, cudaMemcpyHostToDevice, E->st);
    if (r == cudaSuccess && where == PFS_HOST) r = cudaStreamSynchronize(E->st);
    if (r == cudaSuccess && where != PFS_HOST) r = cudaStreamSynchronize(E->st);  // ms lives on this stack frame
    return r == cudaSuccess ? PFS_OK : pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(r));
}

int pfs_ensemble_step(pfs_ensemble *e, int steps)
{
    pfs::NvtxRange range("pfs.ensemble_step");
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E || steps < 0) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad ensemble step arguments");
    if (E->graphs_ok && !E->graph[0]) {
        int rc = pfs::build_graphs(*E);
        if (rc != PFS_OK) return rc;
    }
    for (int s = 0; s < steps; ++s) {
        cudaError_t r;
        if (E->stall_block >= 0) {  // test hook: a direct launch with the stalling block, once
            int rc = pfs::enqueue_step(*E, E->icur, E->st);
            E->stall_block = -1;
            if (rc != PFS_OK) return rc;
            r = cudaSuccess;
        } else if (E->graphs_ok && E->graph[E->icur]) {
            r = cudaGraphLaunch(E->graph[E->icur], E->st);
            if (r == cudaSuccess) pfs::launched();
        } else {
            int rc = pfs::enqueue_step(*E, E->icur, E->st);
            if (rc != PFS_OK) return rc;
            r = cudaSuccess;
        }
        if (r != cudaSuccess) return pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(r));
        E->icur = 1 - E->icur;
        E->steps += 1;
    }
    int err = 0;
    cudaError_t r = cudaMemcpyAsync(&err, E->derr, sizeof(int), cudaMemcpyDeviceToHost, E->st);
    if (r == cudaSuccess) r = cudaStreamSynchronize(E->st);
    if (r != cudaSuccess) return pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(r));
    if (err) return pfs::record_error(PFS_ERR_DEVICE_TIMEOUT, "ensemble grid barrier timed out");
    return PFS_OK;
}

int pfs_ensemble_debug_stall_block(pfs_ensemble *e, int block)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E || block < 0) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad arguments");
    E->stall_block = block;
    return PFS_OK;
}

int pfs_ensemble_member_stats(pfs_ensemble *e, int k, pfs_stats *out)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E || k < 0 || k >= E->n || !out) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad arguments");
    pfs::MemberState ms;
    cudaError_t r = cudaMemcpyAsync(&ms, E->dstate + k, sizeof ms, cudaMemcpyDeviceToHost, E->st);
    if (r == cudaSuccess) r = cudaStreamSynchronize(E->st);
    if (r != cudaSuccess) return pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(r));
    std::memset(out, 0, sizeof *out);
    out->sweeps = ms.sweeps;
    out->checks = ms.checks;
    out->rel_residual = ms.rel;
    out->bnorm = std::sqrt(ms.bb);
    out->capped = ms.capped;
    out->stalled = ms.stalled;
    out->steps = E->steps;
    return PFS_OK;
}

int pfs_ensemble_download(pfs_ensemble *e, int k, float *vp, float *image, int where)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E || k < 0 || k >= E->n) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad arguments");
    const pfs::Member &m = E->hmem[k];
    const size_t nv = (size_t)m.w * m.h * 4, ni = (size_t)m.w * m.h * E->c;
    float *A = vp, *I = image;
    if (where == PFS_HOST) {
        int rc = ens_stage(E, (nv + ni) * sizeof(float));
        if (rc != PFS_OK) return rc;
        A = vp ? E->stage : nullptr;
        I = image ? E->stage + nv : nullptr;
    }
    pfs::MemberState ms;
    cudaError_t r = cudaMemcpyAsync(&ms, E->dstate + k, sizeof ms, cudaMemcpyDeviceToHost, E->st);
    if (r == cudaSuccess) r = cudaStreamSynchronize(E->st);
    if (r == cudaSuccess && A) r = pfs::launch_merge_velocity(A, m.u[0], m.v[0], m.p[ms.cur], m.b, m.ld, m.w, m.h, E->st);
    if (r == cudaSuccess && I && E->c > 0)
        r = pfs::launch_merge_image(I, m.img[E->icur], (size_t)m.ld * m.h, m.ld, m.w, m.h, E->c, E->st);
    if (r == cudaSuccess && where == PFS_HOST) {
        if (vp) r = cudaMemcpyAsync(vp, A, nv * 4, cudaMemcpyDeviceToHost, E->st);
        if (r == cudaSuccess && image && ni) r = cudaMemcpyAsync(image, I, ni * 4, cudaMemcpyDeviceToHost, E->st);
    }
    if (r == cudaSuccess) r = cudaStreamSynchronize(E->st);
    return r == cudaSuccess ? PFS_OK : pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(r));
}

int pfs_ensemble_config(pfs_ensemble *e, int fuse_depth, int chunk_rows)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E || (fuse_depth != 4 && fuse_depth != 8) || chunk_rows <= 0)
        return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "fuse_depth 4 or 8, chunk_rows > 0");
    if (E->prm.max_iters % fuse_depth || (E->prm.check_every > 0 && E->prm.check_every % fuse_depth))
        return pfs::record_error(PFS_ERR_UNSUPPORTED, "cap / check interval not multiples of the fuse depth");
    cudaStreamSynchronize(E->st);
    E->levels = fuse_depth;
    E->halo = fuse_depth == 8 ? 8 : 4;
    E->chunk = chunk_rows;
    E->prm.fuse_depth = fuse_depth;
    E->prm.chunk_rows = chunk_rows;
    pfs::drop_graphs(*E);
    int rc = pfs::build_tasks(*E);
    if (rc == PFS_OK) rc = pfs::grid_for(*E);
    return rc;
}

int pfs_ensemble_info(pfs_ensemble *e, int *fuse_depth, int *chunk_rows, int *grid_blocks, int *graphs)
{
    Ensemble *E = reinterpret_cast<Ensemble *>(e);
    if (!E) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "null ensemble");
    if (fuse_depth) *fuse_depth = E->levels;
    if (chunk_rows) *chunk_rows = E->chunk;
    if (grid_blocks) *grid_blocks = E->grid;
    if (graphs) *graphs = E->graphs_ok && E->graph[0] ? 1 : 0;
    return PFS_OK;
}

}  // extern "C"
