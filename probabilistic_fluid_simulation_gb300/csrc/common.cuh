// Shared device helpers for the GB300 fluid step.
//
// Every float operation that feeds a result goes through an explicit
// round-to-nearest intrinsic (__fadd_rn, __fmul_rn, __fdiv_rn, ...): those are
// never contracted into FMA, so each kernel reproduces the reference's
// single-rounding-per-operation arithmetic (src/fluid.cpp compiled with
// -ffp-contract=off) bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pfs {

// Planar field: one float per cell, rows `ld` floats apart (ld % 4 == 0,
// ld >= w), so every row starts on a 16-byte boundary.
struct Plane {
    float *ptr;
    int ld;
};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// Periodic wrap of a backtraced coordinate, fmod(fmod(x, n) + n, n) in float
// (src/fluid.cpp:48-49,105-106). fmod is exact (its result is always
// representable), so for -n <= x < 2n each fmod reduces to a comparison and
// at most one subtraction of n, which is exact there (Sterbenz); other x take
// CUDA's fmodf, which is exact as well. Same bits either way.
__device__ __forceinline__ float fmod_small(float x, float n)
{
    // x in [-n, 2n]: fmod keeps the sign of x and |result| < n
    if (x >= n) return x == 2.0f * n ? 0.0f : fsub(x, n);
    if (x == -n) return -0.0f;
    return x;
}
__device__ __forceinline__ float wrap_coord(float x, float n)
{
    if (x >= -n && x < 2.0f * n) {
        const float y = fadd(fmod_small(x, n), n);  // in [0, 2n]
        return fmod_small(y, n);
    }
    return fmodf(fadd(fmodf(x, n), n), n);
}

// Bilinear sample with the reference's weights and summation order
// (src/fluid.cpp:62-66): ((a + b) + c) + d, each term ((1-sx)(1-sy)) f.
__device__ __forceinline__ float bilerp(float sx, float sy, float f00, float f10, float f01, float f11)
{
    const float ox = fsub(1.0f, sx), oy = fsub(1.0f, sy);
    const float a = fmul(fmul(ox, oy), f00);
    const float b = fmul(fmul(sx, oy), f10);
    const float c = fmul(fmul(ox, sy), f01);
    const float d = fmul(fmul(sx, sy), f11);
    return fadd(fadd(fadd(a, b), c), d);
}

// Integer cell of a wrapped coordinate in [0, n): truncation as (int)x in
// the reference; clamped so a non-finite input cannot index out of bounds.
__device__ __forceinline__ int cell_of(float x, int n)
{
    int i = __float2int_rz(x);
    return min(max(i, 0), n - 1);
}

// One pressure Jacobi update, src/fluid.cpp:19-21 with alpha = 1, beta = 4
// (src/fluid.cpp:215-216,255): ((((pL + pR) + pT) + pB) + 1*b) / 4. Division
// by 4 is exact, so it is a multiply by 0.25.
__device__ __forceinline__ float jacobi_p(float l, float r, float t, float bo, float b)
{
    return fmul(fadd(fadd(fadd(fadd(l, r), t), bo), b), 0.25f);
}

// One diffusion update, src/fluid.cpp:175-182 (S8): the centre term is the
// current iterate, alpha*neighbours summed in order, divided by beta.
__device__ __forceinline__ float jacobi_d(float l, float r, float t, float bo, float c, float alpha, float beta)
{
    const float s = fadd(fadd(fadd(fmul(alpha, l), fmul(alpha, r)), fmul(alpha, t)), fmul(alpha, bo));
    return fdiv(fadd(s, c), beta);
}

}  // namespace pfs
