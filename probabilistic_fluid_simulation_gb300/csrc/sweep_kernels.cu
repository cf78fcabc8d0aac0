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
#include "storage.cuh"
#include "sweep_stream.cuh"

namespace pfs {

__global__ void k_sweep_single(const float *__restrict__ pin, const float *__restrict__ b,
                               float *__restrict__ pout, int ld, int w, int h, const int *done)
{
    if (done && *(volatile const int *)done) return;
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

// RES: the launch ends a check interval. Every block (also one whose warps
// have no task) adds its stored cells' squared residual of level L, and the
// grid reduction records the check in a.state (done at or below a.tol), as
// the residual kernels do. `done` is set before the launch starts, so either
// every block returns at once or none does.
template <typename T, int G, int L, bool PREV, bool RES = false>
__global__ void __launch_bounds__(128, RES && L >= 5 ? 2 : min_blocks<L>()) k_sweep_stream(StreamArgs<T> a)
{
    using V = typename Store<T>::Vec;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    V *sm_rings = reinterpret_cast<V *>(sm_raw);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int wid = blockIdx.x * 4 + wib;
    if constexpr (!RES) {
        if (wid >= a.nwork) return;  // whole warp
        if (a.done && *(volatile const int *)a.done) return;
        stream_task<T, G, L, PREV>(a, wid, lane, sm_rings + wib * Ring<T, L>::vecs_per_warp);
    } else {
        if (a.done && *(volatile const int *)a.done) return;  // the whole grid
        FFAcc2 acc[2];
        if (wid < a.nwork)
            stream_task<T, G, L, PREV, true>(a, wid, lane, sm_rings + wib * Ring<T, L, true>::vecs_per_warp, acc);
        reduce_blocks(acc[0].value() + acc[1].value(), a.red, 0, a.state, a.sweeps_here, a.tol);
    }
}

template <typename T, int G, int L, bool PREV, bool RES = false>
cudaError_t launch_stream_t(const StreamArgs<T> &a, cudaStream_t st)
{
    constexpr int smem = Ring<T, L, RES>::bytes_per_block;
    static std::atomic<unsigned long long> attr_done{0};  // per instantiation and device
    const cudaError_t e = smem_limit_once(k_sweep_stream<T, G, L, PREV, RES>, smem, attr_done);
    if (e != cudaSuccess) return e;
    const int blocks = (a.nwork + 3) / 4;  // 4 warps per block: the shared rings are laid out for 4
    if (RES && blocks > a.red.nblocks) return cudaErrorInvalidValue;
    k_sweep_stream<T, G, L, PREV, RES><<<blocks, 128, smem, st>>>(a);
    return launched();
}

template <typename T, int G, int L>
cudaError_t launch_stream_l(const StreamArgs<T> &a, bool prev, cudaStream_t st)
{
    return prev ? launch_stream_t<T, G, L, true>(a, st) : launch_stream_t<T, G, L, false>(a, st);
}

template <typename T>
StreamArgs<T> stream_args(const T *pin, const T *b, T *pout, T *pprev, int ld, int w, int h, int halo, int chunk,
                          const int *done)
{
    StreamArgs<T> a{};
    a.pin = pin;
    a.b = b;
    a.pout = pout;
    a.pprev = pprev;
    a.done = done;
    a.ld = ld;
    a.w = w;
    a.h = h;
    a.chunk = chunk;
    a.nsx = (w + 128 - 2 * halo - 1) / (128 - 2 * halo);
    a.nwork = a.nsx * ((h + chunk - 1) / chunk);
    return a;
}

}  // namespace

int stream_strip_width(int halo) { return 128 - 2 * halo; }

cudaError_t launch_sweep_single(const float *pin, const float *b, float *pout, int ld, int w, int h,
                                const int *done, cudaStream_t st)
{
    dim3 blk(32, 8);
    dim3 grd((w + 31) / 32, (h + 7) / 8);
    k_sweep_single<<<grd, blk, 0, st>>>(pin, b, pout, ld, w, h, done);
    return launched();
}

// levels in [1, halo]; halo in {4, 8}; w % 4 == 0; ld % 4 == 0; 16-byte aligned planes.
cudaError_t launch_sweep_stream(const float *pin, const float *b, float *pout, float *pprev, int ld, int w,
                                int h, int levels, int halo, int chunk, const int *done, cudaStream_t st)
{
    const StreamArgs<float> a = stream_args(pin, b, pout, pprev, ld, w, h, halo, chunk, done);
    const bool prev = pprev != nullptr;
    if (halo == 4) {
        switch (levels) {
        case 1: return launch_stream_l<float, 4, 1>(a, prev, st);
        case 2: return launch_stream_l<float, 4, 2>(a, prev, st);
        case 3: return launch_stream_l<float, 4, 3>(a, prev, st);
        case 4: return launch_stream_l<float, 4, 4>(a, prev, st);
        default: return cudaErrorInvalidValue;
        }
    }
    if (halo == 8) {
        switch (levels) {
        case 1: return launch_stream_l<float, 8, 1>(a, prev, st);
        case 2: return launch_stream_l<float, 8, 2>(a, prev, st);
        case 3: return launch_stream_l<float, 8, 3>(a, prev, st);
        case 4: return launch_stream_l<float, 8, 4>(a, prev, st);
        case 5: return launch_stream_l<float, 8, 5>(a, prev, st);
        case 6: return launch_stream_l<float, 8, 6>(a, prev, st);
        case 7: return launch_stream_l<float, 8, 7>(a, prev, st);
        case 8: return launch_stream_l<float, 8, 8>(a, prev, st);
        default: return cudaErrorInvalidValue;
        }
    }
    return cudaErrorInvalidValue;
}

int sweep_stream_blocks(int w, int h, int chunk)
{
    const long long nsx = (w + 128 - 2 * 8 - 1) / (128 - 2 * 8);
    const long long nwork = nsx * ((h + chunk - 1) / chunk);
    return (int)((nwork + 3) / 4);
}

cudaError_t launch_sweep_stream_check(const float *pin, const float *b, float *pout, float *pprev, int ld, int w,
                                      int h, int levels, int chunk, const Reduce &red, SolveState *state,
                                      int sweeps_here, double tol, const int *done, cudaStream_t st)
{
    StreamArgs<float> a = stream_args(pin, b, pout, pprev, ld, w, h, 8, chunk, done);
    a.red = red;
    a.state = state;
    a.sweeps_here = sweeps_here;
    a.tol = tol;
    const bool prev = pprev != nullptr;
    switch (levels) {
    case 1: return prev ? launch_stream_t<float, 8, 1, true, true>(a, st) : launch_stream_t<float, 8, 1, false, true>(a, st);
    case 2: return prev ? launch_stream_t<float, 8, 2, true, true>(a, st) : launch_stream_t<float, 8, 2, false, true>(a, st);
    case 3: return prev ? launch_stream_t<float, 8, 3, true, true>(a, st) : launch_stream_t<float, 8, 3, false, true>(a, st);
    case 4: return prev ? launch_stream_t<float, 8, 4, true, true>(a, st) : launch_stream_t<float, 8, 4, false, true>(a, st);
    case 5: return prev ? launch_stream_t<float, 8, 5, true, true>(a, st) : launch_stream_t<float, 8, 5, false, true>(a, st);
    case 6: return prev ? launch_stream_t<float, 8, 6, true, true>(a, st) : launch_stream_t<float, 8, 6, false, true>(a, st);
    case 7: return prev ? launch_stream_t<float, 8, 7, true, true>(a, st) : launch_stream_t<float, 8, 7, false, true>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

// 16-bit storage (halo 8, levels 1..8, no second-to-last output): the
// iterate and the right-hand side are stored bf16 / fp16 and every sweep is
// computed in FP32 between the load of the input and the store of the output.
template <typename T>
static cudaError_t launch_sweep_stream_lp(const T *pin, const T *b, T *pout, int ld, int w, int h, int levels,
                                          int chunk, cudaStream_t st)
{
    const StreamArgs<T> a = stream_args<T>(pin, b, pout, nullptr, ld, w, h, 8, chunk, nullptr);
    switch (levels) {
    case 1: return launch_stream_t<T, 8, 1, false>(a, st);
    case 2: return launch_stream_t<T, 8, 2, false>(a, st);
    case 3: return launch_stream_t<T, 8, 3, false>(a, st);
    case 4: return launch_stream_t<T, 8, 4, false>(a, st);
    case 5: return launch_stream_t<T, 8, 5, false>(a, st);
    case 6: return launch_stream_t<T, 8, 6, false>(a, st);
    case 7: return launch_stream_t<T, 8, 7, false>(a, st);
    case 8: return launch_stream_t<T, 8, 8, false>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_sweep_stream_bf16(const __nv_bfloat16 *pin, const __nv_bfloat16 *b, __nv_bfloat16 *pout, int ld,
                                     int w, int h, int levels, int chunk, cudaStream_t st)
{
    return launch_sweep_stream_lp(pin, b, pout, ld, w, h, levels, chunk, st);
}

cudaError_t launch_sweep_stream_f16(const __half *pin, const __half *b, __half *pout, int ld, int w, int h,
                                    int levels, int chunk, cudaStream_t st)
{
    return launch_sweep_stream_lp(pin, b, pout, ld, w, h, levels, chunk, st);
}

}  // namespace pfs
