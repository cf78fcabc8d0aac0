// The fused sweep kernel template and its launch helpers, shared by the
// translation units that instantiate it (sweep_kernels.cu: float sweeps;
// sweep_check_kernels.cu: the check launches; sweep_lp_kernels.cu: 16-bit
// storage). Split so that the many instantiations compile in parallel.
#pragma once

#include "common.cuh"
#include "kernels.h"
#include "storage.cuh"
#include "sweep_stream.cuh"

namespace pfs {

namespace {

// Programmatic dependent launch. The sweep launches of a solve form a chain in
// one stream, each reading the plane the previous one wrote. They are
// launched with cudaLaunchAttributeProgrammaticStreamSerialization, so the
// next launch's blocks can be scheduled while this one drains;
// griddepcontrol.wait then holds every thread until the previous grid has
// completed and its writes are visible, before any global load or store.
// Each grid allows its dependents to launch only after it has passed its own
// wait, so a grid two launches ahead never starts before this one's inputs
// are final. Measured at 2048x2048 (8 sweeps per launch, back to back): 16.5
// to 14.0 us per launch; the kernels' results are unchanged.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void allow_dependent_launch() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// RES: the launch ends a check interval. Every block (also one whose warps
// have no task) adds its stored cells' squared residual of level L, and the
// grid reduction records the check in a.state (done at or below a.tol), as
// the residual kernels do. `done` is set before the launch starts, so either
// every block returns at once or none does.
// The register cap per thread is the same for any kStreamWarps: 65536 over
// (128 * min_blocks) threads.
template <typename T, int G, int L, bool PREV, bool RES = false>
__global__ void __launch_bounds__(32 * kStreamWarps, (RES && L >= 5 ? 2 : min_blocks<L>()) * 4 / kStreamWarps)
    k_sweep_stream(StreamArgs<T> a)
{
    using V = typename Store<T>::Vec;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    V *sm_rings = reinterpret_cast<V *>(sm_raw);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int wid = blockIdx.x * kStreamWarps + wib;
    grid_dependency_wait();
    allow_dependent_launch();
    if constexpr (!RES) {
        if (wid >= a.nwork) return;  // whole warp
        if (a.done && *(volatile const int *)a.done) return;
        stream_task<T, G, L, PREV>(a, wid, lane, sm_rings + wib * Ring<T, L>::vecs_per_warp);
    } else {
        if (a.done && *(volatile const int *)a.done) return;  // the whole grid
        FFAcc2 acc[2];
        if (wid < a.nwork)
            stream_task<T, G, L, PREV, true>(a, wid, lane, sm_rings + wib * Ring<T, L, true>::vecs_per_warp, acc);
        reduce_blocks(acc[0].value() + acc[1].value(), a.red, 0, a.state, a.sweeps_here, a.tol, a.stall_window);
    }
}

template <typename T, int G, int L, bool PREV, bool RES = false>
cudaError_t launch_stream_t(const StreamArgs<T> &a, cudaStream_t st)
{
    // The deepest pipelines (L >= 7) are sized for two blocks per SM
    // (min_blocks; default_chunk fills that wave), and the check launches run
    // on the same chunks. Their register use can fall low enough for a third
    // block, and such a grid then lands unevenly on the SMs (4096^2 at 128-row
    // chunks: 34 -> 44 us per launch; the 4-level check at 148 registers cost
    // 1.5% of a capped 2048^2 step). A shared-memory request above a third of
    // the SM's 228 KB keeps them at two.
    constexpr int ring_bytes = kStreamWarps * Ring<T, L, RES>::vecs_per_warp * Store<T>::vec_bytes;
    constexpr int smem = ((L >= 7 || RES) && ring_bytes < 76 * 1024) ? 76 * 1024 : ring_bytes;
    static std::atomic<unsigned long long> attr_done{0};  // per instantiation and device
    const cudaError_t e = smem_limit_once(k_sweep_stream<T, G, L, PREV, RES>, smem, attr_done);
    if (e != cudaSuccess) return e;
    const int blocks = (a.nwork + kStreamWarps - 1) / kStreamWarps;
    if ((long long)a.h * (a.ld / 4) >= (1LL << 31)) return cudaErrorInvalidValue;  // vector offsets in 32 bits
    if (RES && blocks > a.red.nblocks) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(32 * kStreamWarps);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t le = cudaLaunchKernelEx(&cfg, k_sweep_stream<T, G, L, PREV, RES>, a);
    if (le != cudaSuccess) return le;
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

}  // namespace pfs
