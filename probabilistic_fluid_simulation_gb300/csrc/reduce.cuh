// Deterministic grid reductions and error-free float arithmetic shared by
// the step kernels and the precision-form kernels.
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace pfs {
namespace {

// Block sum of `acc`, written to red.partials[blockIdx.x * 2 + slot]; the last
// block to finish adds the partials in block order into red.result[slot] and
// re-arms that slot's ticket (one ticket per slot, so two reductions in one
// kernel do not mix their counts). The order of additions is fixed, so the sum is
// reproducible run to run.
__device__ void reduce_blocks(double acc, const Reduce &red, int slot, SolveState *state = nullptr,
                              int sweeps_here = 0, double tol = 0.0, int stall_window = 0)
{
    __shared__ double ws[32];
    __shared__ bool last;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) ws[wid] = acc;
    __syncthreads();
    if (wid == 0) {
        acc = lane < nw ? ws[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            red.partials[blockIdx.x * 2 + slot] = acc;
            __threadfence();
            last = atomicAdd(red.ticket + slot, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (last && wid == 0) {
        __threadfence();
        // lane sums partials lane, lane + 32, ... in that order; the loads are
        // issued eight at a time so the tail does not wait on one L2 round trip
        // per partial (the same additions in the same order as a plain loop)
        double s = 0.0;
        const int n = (int)gridDim.x;
        int k = lane;
        for (; k + 32 * 7 < n; k += 32 * 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = __ldcg(red.partials + (k + 32 * u) * 2 + slot);
#pragma unroll
            for (int u = 0; u < 8; ++u) s += v[u];
        }
        for (; k < n; k += 32) s += __ldcg(red.partials + k * 2 + slot);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) {
            red.result[slot] = s;
            red.ticket[slot] = 0u;
            if (state) {
                const double bb = red.result[1];
                const double rel = bb > 0.0 ? __dsqrt_rn(s) / __dsqrt_rn(bb) : __dsqrt_rn(s);
                state->rr = s;
                state->bb = bb;
                state->rel = rel;
                state->checks += 1;
                if (rel <= tol) {
                    state->sweeps = sweeps_here;
                    state->done = 1;
                } else if (stall_window > 0) {
                    if (state->best == 0.0 || rel < kStallGain * state->best) {
                        state->best = rel;
                        state->best_sweeps = sweeps_here;
                    } else if (sweeps_here - state->best_sweeps >= stall_window) {
                        state->sweeps = sweeps_here;
                        state->done = 2;
                    }
                }
            }
        }
    }
}

// Error-free float transformations (Knuth's TwoSum, and the product error
// from one fused multiply-add) used to evaluate the residual exactly without
// FP64 arithmetic per cell: on GB300 the FP64 pipe runs at a small fraction
// of the FP32 rate.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// Per-thread sum of squares kept as an unevaluated pair hi + lo of floats
// (about 48 significant bits); converted to double once per thread, and the
// block and grid sums are FP64.
struct FFAcc {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float a, float a_lo)
    {
        const FF s = two_sum(hi, a);
        const float e = __fadd_rn(s.lo, __fadd_rn(lo, a_lo));
        hi = __fadd_rn(s.hi, e);
        lo = __fsub_rn(e, __fsub_rn(hi, s.hi));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// x^2 as hi + lo: the product and its exact rounding error (one FMA).
__device__ __forceinline__ void acc_square(FFAcc &acc, float x)
{
    const float sq = __fmul_rn(x, x);
    acc.add(sq, __fmaf_rn(x, x, -sq));
}

// The same transformations on two independent values at once with the packed
// f32x2 instructions of sm_100+ (__fadd2_rn, __fmul2_rn, __ffma2_rn round each
// element to nearest, like their scalar forms), so each element gets exactly
// the bits of the scalar version in half the issue slots. x - y is
// fma(y, -1, x): the product is exact, so it is x - y rounded once.
__device__ __forceinline__ float2 fsub2(float2 x, float2 y) { return __ffma2_rn(y, make_float2(-1.0f, -1.0f), x); }

struct FF2 {
    float2 hi, lo;
};

__device__ __forceinline__ FF2 two_sum2(float2 a, float2 b)
{
    const float2 s = __fadd2_rn(a, b);
    const float2 bb = fsub2(s, a);
    const float2 e = __fadd2_rn(fsub2(a, fsub2(s, bb)), fsub2(b, bb));
    return {s, e};
}

// Two FFAcc chains (element x and element y) advanced together.
struct FFAcc2 {
    float2 hi = make_float2(0.0f, 0.0f), lo = make_float2(0.0f, 0.0f);
    __device__ __forceinline__ void add(float2 a, float2 a_lo)
    {
        const FF2 s = two_sum2(hi, a);
        const float2 e = __fadd2_rn(s.lo, __fadd2_rn(lo, a_lo));
        hi = __fadd2_rn(s.hi, e);
        lo = fsub2(e, fsub2(hi, s.hi));
    }
    // (chain x) + (chain y), each converted as FFAcc::value()
    __device__ __forceinline__ double value() const
    {
        return ((double)hi.x + (double)lo.x) + ((double)hi.y + (double)lo.y);
    }
};

}  // namespace
}  // namespace pfs
