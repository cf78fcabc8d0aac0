// Launchers of the device kernels (private to the library; the public
// surface is include/pfs.h).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace pfs {

// Record `msg` as the calling thread's pfs_last_error() and return `code`.
int record_error(int code, const char *msg);

// Kernels launched by this library since it was loaded (pfs_kernel_launches()).
extern std::atomic<long long> g_launches;
inline cudaError_t launched(int n = 1)
{
    g_launches.fetch_add(n, std::memory_order_relaxed);
    return cudaGetLastError();
}

// Raise a kernel's dynamic shared-memory limit once per device (function
// attributes belong to a device's context); `done` holds one bit per device.
template <typename F>
inline cudaError_t smem_limit_once(F *kernel, int bytes, std::atomic<unsigned long long> &done)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_acq_rel);
    return e;
}

// Reduction scratch: one double pair per block plus a ticket, so the last
// block sums the partials in block order (deterministic result).
struct Reduce {
    double *partials;   // [2 * nblocks]
    unsigned *ticket;   // one counter per result slot, zero between launches
    double *result;     // [2]: sum r^2 (or b^2), second slot for the paired sum
    int nblocks;
};

// Capacity of the reduction scratch in blocks (partial-sum slots). The grids
// of the reductions use reduce_grid(): four blocks per SM of the current
// device, at most this many.
constexpr int kReduceBlocks = 608;
int reduce_grid();
// Streaming multiprocessors of the current device (0 if it cannot be read).
int device_sms();

// Device-side state of one pressure solve in residual mode. The residual
// kernel at a check point sets `done` when ||r||/||b|| <= tol, or, with a
// stall window, when the relative residual has not fallen below 0.99 times
// its best value for that many sweeps (the iterate has reached the rounding
// floor of its storage); sweep and residual launches enqueued after that see
// the flag and return at once.
struct SolveState {
    int done;         // 0 iterating, 1 converged, 2 stalled
    int sweeps;       // sweep count at the check that set done
    int checks;       // residual evaluations performed
    int best_sweeps;  // sweep count at the check that last lowered `best`
    double rel;       // last evaluated relative residual
    double rr;        // last evaluated sum r^2
    double bb;        // sum b^2 of this step's divergence
    double best;      // smallest relative residual so far (0: none yet)
};
// A check lowers `best` when its residual is below this fraction of it.
constexpr double kStallGain = 0.99;
// Stall window in sweeps for a grid whose larger side is n, with checks every
// `every` sweeps: long enough that the slowest mode of the exact iteration
// (Jacobi eigenvalue (1 + cos(2 pi / n)) / 2 ~ 1 - pi^2 / n^2 on the periodic
// grid) falls by 3% within it, so only rounding can stop the residual from
// falling 1%, and at least two checks; a multiple of `every`.
inline int auto_stall_window(int n, int every)
{
    const double w = 3.09e-3 * (double)n * (double)n;
    const int e = every > 0 ? every : 1;
    long long k = (long long)((w + e - 1) / e);
    if (k < 2) k = 2;
    if (k > (1 << 30) / e) k = (1 << 30) / e;
    return (int)(k * e);
}

// Sweeps between refinements of the float32 refined form in residual mode
// for a grid whose larger side is n. The float32 correction e can lower its
// residual to about 4.5 * 2^-25 * rms(e) / rms(rt) of its right-hand side
// (the rounding of e); once the residual is smooth, rms(e) / rms(rt) is about
// n^2 / (4 pi^2), a floor of a few percent at 2048^2. In `interval` sweeps
// the slowest mode of the iteration falls by exp(-interval * pi^2 / n^2),
// 0.78 for interval = 0.025 n^2, so the correction is refined long before it
// nears that floor, while the FP64 pass (one read of x, b and e, and the
// damped passes) is rare: one per 105,000 sweeps at 2048^2. A multiple of the
// check interval.
inline int f32r_refine_interval(int n, int every)
{
    const double want = 0.025 * (double)n * (double)n;
    long long k = (long long)((want + every - 1) / every);
    if (k < 1) k = 1;
    if (k > (1 << 30) / every) k = (1 << 30) / every;
    return (int)(k * every);
}

// ---- velocity / image / layout (step_kernels.cu) ----
cudaError_t launch_advect(const float *u, const float *v, float *uo, float *vo, int ld, int w, int h, float dt,
                          cudaStream_t st, int bc = 0);
cudaError_t launch_diffuse_sweep(const float *u, const float *v, float *uo, float *vo, int ld, int w, int h,
                                 float alpha, float beta, cudaStream_t st);
// b = gamma * ((u[i+1]-u[i-1]) + (v[j+1]-v[j-1])); sum b^2 into red.result[1]
cudaError_t launch_divergence(const float *u, const float *v, float *b, int ld, int w, int h, float gamma,
                              const Reduce &red, cudaStream_t st);
cudaError_t launch_project(const float *u, const float *v, const float *p, float *uo, float *vo, int ld, int w,
                           int h, float dt, cudaStream_t st, int bc = 0);
// projection fused with image advection when the image grid equals the velocity grid
cudaError_t launch_project_advect_image(const float *u, const float *v, const float *p, float *uo, float *vo,
                                        int ld, int w, int h, float dt, const float *img, float *imgo,
                                        size_t img_plane, int c, cudaStream_t st, int bc = 0);
// image advection, planar image (c planes of img_plane floats, row pitch ild), planar velocity
cudaError_t launch_advect_image_planar(const float *img, float *imgo, size_t img_plane, int ild, int iw, int ih,
                                       int c, const float *u, const float *v, int vld, int vw, int vh, float dt,
                                       cudaStream_t st, int bc = 0);
// image advection on the reference's interleaved layout (image HWC with c
// channels, velocity HWC with 4 channels)
cudaError_t launch_advect_image_interleaved(const float *img, float *imgo, int iw, int ih, int c,
                                            const float *vel, int vw, int vh, float dt, cudaStream_t st);
// interleaved (h, w, 4) <-> planar
cudaError_t launch_split_velocity(const float *vp, float *u, float *v, int ld, int w, int h, cudaStream_t st);
// interleaved (u, v, p, b) -> planes in one pass (b may be null)
cudaError_t launch_split_vp(const float *vp, float *u, float *v, float *p, float *b, int ld, int w, int h,
                            cudaStream_t st);
cudaError_t launch_split_channel(const float *buf, int ch, int nch, float *plane, int ld, int w, int h,
                                 cudaStream_t st);
cudaError_t launch_merge_velocity(float *out, const float *u, const float *v, const float *p, const float *b,
                                  int ld, int w, int h, cudaStream_t st);
cudaError_t launch_split_image(const float *img, float *planes, size_t plane, int ld, int w, int h, int c,
                               cudaStream_t st);
cudaError_t launch_merge_image(float *img, const float *planes, size_t plane, int ld, int w, int h, int c,
                               cudaStream_t st);

// float32 -> float64, n elements (out may be null: nothing to do)
cudaError_t launch_widen(const float *in, double *out, size_t n, cudaStream_t st);
// pout = p + (b - A p) / 8 (damped Jacobi pass on a predicted pressure start)
cudaError_t launch_damp(const float *pin, const float *b, float *pout, int ld, int w, int h, cudaStream_t st);
// r = b - A p (float, per cell) and p += d: the later passes of a predicted start
cudaError_t launch_residual_field(const float *p, const float *b, float *r, int ld, int w, int h, cudaStream_t st);
cudaError_t launch_add(float *p, const float *d, size_t n, cudaStream_t st);
// Small transfers (bytes a multiple of 4, at most 1 MiB, 4-byte aligned) run
// as a one-warp kernel instead of a copy-engine operation, so they never
// queue behind bulk copies that occupy the copy engines (asynchronous session
// transfers). dst may be device memory or the device alias of mapped pinned
// host memory.
cudaError_t launch_copy_small(const void *src, void *dst, size_t bytes, cudaStream_t st);
cudaError_t launch_zero_small(void *dst, size_t bytes, cudaStream_t st);

// ---- pressure (sweep_kernels.cu, residual_kernels.cu) ----
int stream_strip_width(int halo);
// Rows per warp task of the fused sweep when the caller sets none (see
// sweep_kernels.cu).
int default_chunk(int w, int h, int levels);
// `done` (may be null): skip the launch when *done != 0
cudaError_t launch_sweep_single(const float *pin, const float *b, float *pout, int ld, int w, int h,
                                const int *done, cudaStream_t st);
cudaError_t launch_sweep_stream(const float *pin, const float *b, float *pout, float *pprev, int ld, int w,
                                int h, int levels, int halo, int chunk, const int *done, cudaStream_t st);
// The last launch of a check interval (halo 8, levels 1..7): the fused sweep
// that also evaluates the exact residual of its output over the grid, as
// launch_residual does, recording the check in `state` (done at or below tol,
// with sweeps_here). Needs red.nblocks >= sweep_stream_blocks(w, h, chunk);
// red.result[1] must hold sum b^2.
int sweep_stream_blocks(int w, int h, int chunk);
// launch_sweep_stream_check without the level L-1 output (pprev null), in its own unit.
cudaError_t launch_sweep_stream_check_noprev(const float *pin, const float *b, float *pout, int ld, int w, int h,
                                             int levels, int chunk, const Reduce &red, SolveState *state,
                                             int sweeps_here, double tol, const int *done, cudaStream_t st,
                                             int stall_window);
// Smallest row chunk default_chunk picks (partial sums of the fused check are sized for it).
constexpr int kMinChunkRows = 4;
cudaError_t launch_sweep_stream_check(const float *pin, const float *b, float *pout, float *pprev, int ld, int w,
                                      int h, int levels, int chunk, const Reduce &red, SolveState *state,
                                      int sweeps_here, double tol, const int *done, cudaStream_t st,
                                      int stall_window = 0);
// 16-bit storage, FP32 compute; pin == null means a zero input iterate. levels in [1, 8].
cudaError_t launch_sweep_stream_bf16(const __nv_bfloat16 *pin, const __nv_bfloat16 *b, __nv_bfloat16 *pout, int ld,
                                     int w, int h, int levels, int chunk, cudaStream_t st);
cudaError_t launch_sweep_stream_f16(const __half *pin, const __half *b, __half *pout, int ld, int w, int h,
                                    int levels, int chunk, cudaStream_t st);
// sum over cells of r^2, r = b + pL + pR + pT + pB - 4p (exact per cell), into
// red.result[0]. With `state`: skipped when state->done; otherwise records the
// check (rel = sqrt(r^2)/sqrt(b^2) from red.result[1]) and marks the solve
// done at `sweeps_here` sweeps when rel <= tol.
cudaError_t launch_residual(const float *p, const float *b, int ld, int w, int h, const Reduce &red,
                            SolveState *state, int sweeps_here, double tol, cudaStream_t st, int stall_window = 0);
// both sums in one pass: r^2 into red.result[0], b^2 into red.result[1]
cudaError_t launch_norms(const float *p, const float *b, int ld, int w, int h, const Reduce &red, cudaStream_t st);

}  // namespace pfs
