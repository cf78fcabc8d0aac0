// Pressure Jacobi sweeps (the hot loop of src/fluid.cpp:239-266) on planar
// float32 fields.
//
//   k_sweep_single  one sweep per launch, any grid size (also the reference
//                   the fused kernel is checked against).
//   k_sweep_stream  L sweeps fused in one launch (temporal blocking). Each
//                   warp owns a strip of 128 columns (4 per lane, float4) and
//                   streams down a chunk of rows. Sweep level s+1 of row r is
//                   computed from level s of rows r-1, r, r+1, which the lane
//                   holds in registers; left/right neighbours come from the
//                   adjacent lanes by warp shuffle. The strip carries G halo
//                   columns per side and the chunk L halo rows per end, which
//                   are recomputed redundantly, so warps never wait on each
//                   other. Global traffic per launch: read p and b once, write
//                   p once (plus the second-to-last level when asked).
//
// Arithmetic per cell is pfs::jacobi_p, bit-identical to the reference, and a
// Jacobi sweep is order-independent, so any fusion depth gives the same bits.
#include "common.cuh"
#include "kernels.h"

namespace pfs {

__global__ void k_sweep_single(const float *__restrict__ pin, const float *__restrict__ b,
                               float *__restrict__ pout, int ld, int w, int h)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= w || j >= h) return;
    const int im = (i == 0) ? w - 1 : i - 1, ip = (i + 1 == w) ? 0 : i + 1;
    const int jm = (j == 0) ? h - 1 : j - 1, jp = (j + 1 == h) ? 0 : j + 1;
    const size_t row = (size_t)j * ld;
    pout[row + i] = jacobi_p(pin[row + im], pin[row + ip], pin[(size_t)jm * ld + i], pin[(size_t)jp * ld + i],
                             b[row + i]);
}

namespace {

__device__ __forceinline__ int wrap_row(int y, int h)
{
    int r = y % h;
    return r < 0 ? r + h : r;
}

__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

// Level s+1 of the lane's four cells of row r from level s: `c` is row r
// (horizontal neighbours from lanes l-1 / l+1), `up` row r-1, `dn` row r+1.
__device__ __forceinline__ float4 jacobi4(const float4 &c, const float4 &up, const float4 &dn, const float4 &bb)
{
    const float lft = __shfl_up_sync(0xffffffffu, c.w, 1);
    const float rgt = __shfl_down_sync(0xffffffffu, c.x, 1);
    float4 o;
    o.x = jacobi_p(lft, c.y, up.x, dn.x, bb.x);
    o.y = jacobi_p(c.x, c.z, up.y, dn.y, bb.y);
    o.z = jacobi_p(c.y, c.w, up.z, dn.z, bb.z);
    o.w = jacobi_p(c.z, rgt, up.w, dn.w, bb.w);
    return o;
}

struct StreamArgs {
    const float *pin;
    const float *b;
    float *pout;
    float *pprev;  // receives level L-1 (the second-to-last iterate) when non-null
    int ld, w, h;
    int nsx, nwork, chunk;
};

// One row step of the pipeline for load row y. P/Cur/N are the three rotating
// register sets (rows y-s-2, y-s-1, y-s of level s); the caller rotates the
// roles by passing them in a different order each step, so no register moves
// are needed.
template <int L, bool PREV>
__device__ __forceinline__ void stream_step(int y, float4 (&P)[L], float4 (&Cur)[L], float4 (&N)[L],
                                            float4 (&bq)[L], float4 &blast, float4 &pn, float4 &bn,
                                            const StreamArgs &a, int cx, bool st_lane, int y0, int y1, int yend)
{
    N[0] = pn;
    const float4 b_y = bn;
    if (y + 1 < yend) {
        const size_t o = (size_t)wrap_row(y + 1, a.h) * a.ld + cx;
        pn = ldg4(a.pin + o);
        bn = ldg4(a.b + o);
    }
#pragma unroll
    for (int s = L - 1; s > 0; --s) bq[s] = bq[s - 1];
    bq[0] = blast;  // b(y-1)
    blast = b_y;
    float4 top;
#pragma unroll
    for (int s = 0; s < L; ++s) {
        const float4 o = jacobi4(Cur[s], P[s], N[s], bq[s]);  // level s+1, row y-s-1
        if (s + 1 < L) N[s + 1] = o;
        else top = o;
    }
    const int r = y - L;  // row of level L
    if (st_lane && r >= y0 && r < y1)
        *reinterpret_cast<float4 *>(a.pout + (size_t)r * a.ld + cx) = top;
    if (PREV) {
        const int rp = y - (L - 1);  // row of level L-1
        if (st_lane && rp >= y0 && rp < y1)
            *reinterpret_cast<float4 *>(a.pprev + (size_t)rp * a.ld + cx) = N[L - 1];
    }
}

template <int G, int L, bool PREV>
__global__ void __launch_bounds__(128) k_sweep_stream(StreamArgs a)
{
    static_assert(L >= 1 && L <= G && G % 4 == 0, "fusion depth must fit the halo");
    const int lane = threadIdx.x & 31;
    const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (wid >= a.nwork) return;  // whole warp
    const int sx = wid % a.nsx, sy = wid / a.nsx;
    const int xo = sx * (128 - 2 * G);
    const int xl = xo - G + 4 * lane;
    int cx = xl % a.w;
    if (cx < 0) cx += a.w;
    const bool st_lane = lane >= G / 4 && lane < 32 - G / 4 && xl < a.w;
    const int y0 = sy * a.chunk;
    const int y1 = min(a.h, y0 + a.chunk);
    const int ybeg = y0 - L, yend = y1 + L;

    float4 R0[L], R1[L], R2[L], bq[L];
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int s = 0; s < L; ++s) R0[s] = R1[s] = R2[s] = bq[s] = z;
    float4 blast = z;
    const size_t o0 = (size_t)wrap_row(ybeg, a.h) * a.ld + cx;
    float4 pn = ldg4(a.pin + o0), bn = ldg4(a.b + o0);

    for (int y = ybeg; y < yend; y += 3) {
        stream_step<L, PREV>(y, R0, R1, R2, bq, blast, pn, bn, a, cx, st_lane, y0, y1, yend);
        if (y + 1 < yend) stream_step<L, PREV>(y + 1, R1, R2, R0, bq, blast, pn, bn, a, cx, st_lane, y0, y1, yend);
        if (y + 2 < yend) stream_step<L, PREV>(y + 2, R2, R0, R1, bq, blast, pn, bn, a, cx, st_lane, y0, y1, yend);
    }
}

template <int G, int L, bool PREV>
cudaError_t launch_stream_t(const StreamArgs &a, cudaStream_t st)
{
    const int blocks = (a.nwork + 3) / 4;
    k_sweep_stream<G, L, PREV><<<blocks, 128, 0, st>>>(a);
    return launched();
}

template <int G, int L>
cudaError_t launch_stream_l(const StreamArgs &a, bool prev, cudaStream_t st)
{
    return prev ? launch_stream_t<G, L, true>(a, st) : launch_stream_t<G, L, false>(a, st);
}

}  // namespace

int stream_strip_width(int halo) { return 128 - 2 * halo; }

cudaError_t launch_sweep_single(const float *pin, const float *b, float *pout, int ld, int w, int h,
                                cudaStream_t st)
{
    dim3 blk(32, 8);
    dim3 grd((w + 31) / 32, (h + 7) / 8);
    k_sweep_single<<<grd, blk, 0, st>>>(pin, b, pout, ld, w, h);
    return launched();
}

// levels in [1, halo]; halo in {4, 8}; w % 4 == 0; ld % 4 == 0; 16-byte aligned planes.
cudaError_t launch_sweep_stream(const float *pin, const float *b, float *pout, float *pprev, int ld, int w,
                                int h, int levels, int halo, int chunk, cudaStream_t st)
{
    StreamArgs a;
    a.pin = pin;
    a.b = b;
    a.pout = pout;
    a.pprev = pprev;
    a.ld = ld;
    a.w = w;
    a.h = h;
    a.chunk = chunk;
    a.nsx = (w + stream_strip_width(halo) - 1) / stream_strip_width(halo);
    a.nwork = a.nsx * ((h + chunk - 1) / chunk);
    const bool prev = pprev != nullptr;
    if (halo == 4) {
        switch (levels) {
        case 1: return launch_stream_l<4, 1>(a, prev, st);
        case 2: return launch_stream_l<4, 2>(a, prev, st);
        case 3: return launch_stream_l<4, 3>(a, prev, st);
        case 4: return launch_stream_l<4, 4>(a, prev, st);
        default: return cudaErrorInvalidValue;
        }
    }
    if (halo == 8) {
        switch (levels) {
        case 1: return launch_stream_l<8, 1>(a, prev, st);
        case 2: return launch_stream_l<8, 2>(a, prev, st);
        case 3: return launch_stream_l<8, 3>(a, prev, st);
        case 4: return launch_stream_l<8, 4>(a, prev, st);
        case 5: return launch_stream_l<8, 5>(a, prev, st);
        case 6: return launch_stream_l<8, 6>(a, prev, st);
        case 7: return launch_stream_l<8, 7>(a, prev, st);
        case 8: return launch_stream_l<8, 8>(a, prev, st);
        default: return cudaErrorInvalidValue;
        }
    }
    return cudaErrorInvalidValue;
}

}  // namespace pfs
