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
    // without the level L-1 output (the refined forms' correction solves): the
    // other unit, so that the two halves of the instantiations compile in parallel
    if (!pprev)
        return launch_sweep_stream_check_noprev(pin, b, pout, ld, w, h, levels, chunk, red, state, sweeps_here, tol,
                                                done, st, stall_window);
    switch (levels) {
    case 1: return launch_stream_t<float, 8, 1, true, true>(a, st);
    case 2: return launch_stream_t<float, 8, 2, true, true>(a, st);
    case 3: return launch_stream_t<float, 8, 3, true, true>(a, st);
    case 4: return launch_stream_t<float, 8, 4, true, true>(a, st);
    case 5: return launch_stream_t<float, 8, 5, true, true>(a, st);
    case 6: return launch_stream_t<float, 8, 6, true, true>(a, st);
    case 7: return launch_stream_t<float, 8, 7, true, true>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pfs
