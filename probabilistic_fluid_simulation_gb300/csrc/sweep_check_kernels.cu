// The last launch of a check interval: the fused sweep that also evaluates
// the exact residual of its output (k_sweep_stream with RES; see
// sweep_stream.cuh and sweep_kernels.cu for the design).
#include "common.cuh"
#include "kernels.h"
#include "storage.cuh"
#include "sweep_launch.cuh"

namespace pfs {

int sweep_stream_blocks(int w, int h, int chunk)
{
    const long long nsx = (w + 128 - 2 * 8 - 1) / (128 - 2 * 8);
    const long long nwork = nsx * ((h + chunk - 1) / chunk);
    return (int)((nwork + kStreamWarps - 1) / kStreamWarps);
}

cudaError_t launch_sweep_stream_check(const float *pin, const float *b, float *pout, float *pprev, int ld, int w,
                                      int h, int levels, int chunk, const Reduce &red, SolveState *state,
                                      int sweeps_here, double tol, const int *done, cudaStream_t st,
                                      int stall_window)
{
    StreamArgs<float> a = stream_args(pin, b, pout, pprev, ld, w, h, 8, chunk, done);
    a.red = red;
    a.state = state;
    a.sweeps_here = sweeps_here;
    a.tol = tol;
    a.stall_window = stall_window;
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

}  // namespace pfs
