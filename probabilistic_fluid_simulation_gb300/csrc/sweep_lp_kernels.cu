// The fused sweep on 16-bit storage (bf16 / fp16 iterate and right-hand
// side, FP32 arithmetic), for the refined precision forms.
#include "common.cuh"
#include "kernels.h"
#include "storage.cuh"
#include "sweep_launch.cuh"

namespace pfs {

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
