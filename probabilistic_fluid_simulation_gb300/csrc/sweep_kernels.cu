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
// Arithmetic per cell is pfs::jacobi_p, bit-identical to the reference (the
// fused kernel's final multiply-add on b/4 equals it throughout float32's
// normal range, see jacobi4), and a Jacobi sweep is order-independent, so any
// fusion depth gives the same bits.
#include "common.cuh"
#include "kernels.h"
#include "storage.cuh"
#include "sweep_launch.cuh"

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
    const long long n = (long long)ld * h;
    (void)n;
    PFS_ST(pout, row + i, n,
           jacobi_p(PFS_LD(pin, row + im, n, kBsSweepSingle), PFS_LD(pin, row + ip, n, kBsSweepSingle),
                    PFS_LD(pin, (size_t)jm * ld + i, n, kBsSweepSingle),
                    PFS_LD(pin, (size_t)jp * ld + i, n, kBsSweepSingle), PFS_LD(b, row + i, n, kBsSweepSingle)),
           kBsSweepSingle);
}

int stream_strip_width(int halo) { return 128 - 2 * halo; }

// Chunk height by grid. A warp task recomputes L(L-1) level rows besides its
// chunk (after the ramp skip), so taller chunks waste less; but a grid with
// more tasks than one wave of resident warps runs a second, mostly empty
// wave, and one with fewer leaves schedulers without their warps. The default
// is the smallest chunk that fits the grid in one wave (four warps per
// block, the blocks per SM the kernel is held to, every SM), at least
// kMinChunkRows. Measured on GB300, 8 sweeps per launch (us per launch, the
// default marked *): 4096^2 128* 33.9, 64 37.3; 2048^2 32* 10.6, 16 13.5;
// 1024^2 9* 5.77, 10 6.0, 16 7.2; 512^2 4* 5.18, 16 5.91; 1536^2 22 8.7,
// 16 10.8.
int default_chunk(int w, int h, int levels)
{
    const int halo = levels <= 4 ? 4 : 8;
    const long long nsx = (w + stream_strip_width(halo) - 1) / stream_strip_width(halo);
    const int sms = device_sms() > 0 ? device_sms() : 1;
    const long long wave = (long long)sms * 4 * (levels >= 7 ? min_blocks<8>() : min_blocks<4>());
    const long long per = std::max(1LL, wave / std::max(1LL, nsx));  // row chunks one wave holds
    const long long c = (h + per - 1) / per;
    return (int)std::max<long long>(kMinChunkRows, std::min<long long>(c, std::max(h, 1)));
}

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

}  // namespace pfs
