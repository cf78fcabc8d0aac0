// The check launches without the level L-1 output (k_sweep_stream with RES,
// PREV false: the refined forms' correction solves), split from
// sweep_check_kernels.cu so that the two halves of the instantiations compile
// in parallel. See sweep_check_kernels.cu and sweep_stream.cuh.
#include "common.cuh"
#include "kernels.h"
#include "storage.cuh"
#include "sweep_launch.cuh"

namespace pfs {

cudaError_t launch_sweep_stream_check_noprev(const float *pin, const float *b, float *pout, int ld, int w, int h,
                                             int levels, int chunk, const Reduce &red, SolveState *state,
                                             int sweeps_here, double tol, const int *done, cudaStream_t st,
                                             int stall_window)
{
    StreamArgs<float> a = stream_args(pin, b, pout, (float *)nullptr, ld, w, h, 8, chunk, done);
    a.red = red;
    a.state = state;
    a.sweeps_here = sweeps_here;
    a.tol = tol;
    a.stall_window = stall_window;
    switch (levels) {
    case 1: return launch_stream_t<float, 8, 1, false, true>(a, st);
    case 2: return launch_stream_t<float, 8, 2, false, true>(a, st);
    case 3: return launch_stream_t<float, 8, 3, false, true>(a, st);
    case 4: return launch_stream_t<float, 8, 4, false, true>(a, st);
    case 5: return launch_stream_t<float, 8, 5, false, true>(a, st);
    case 6: return launch_stream_t<float, 8, 6, false, true>(a, st);
    case 7: return launch_stream_t<float, 8, 7, false, true>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pfs
