// pfs_residual_norms_static: the residual/divergence norm reduction of
// pfs_residual_norms (the same kernel) with its cross-block scratch held in a
// fixed array of this library instead of memory the call allocates.
//
// Who needs it: callers that must not allocate device memory. A host
// application whose device memory is entirely reserved by another allocator
// (a framework's caching pool that owns the whole device, for example) gets
// out-of-memory from cudaMalloc even though the work itself needs only a few
// kilobytes; and a caller on a latency-critical path cannot afford cudaMalloc,
// which may synchronize the whole device. pfs_residual_norms allocates its
// scratch on first use (per device and grid size); this entry point allocates
// nothing, ever.
//
// The scratch is g_norms_scratch below: kNormsStaticBytes (10 KiB) per device
// that loads the library, held until the process exits. Every call shares it
// and it keeps the last call's contents: each call clears the reduction
// tickets (the only part that must start at zero) before its launch. Calls
// that overlap on the GPU (issued on different streams and running at the
// same time) race on this array; issue them one after another.
#include <cstdio>

#include "kernels.h"
#include "pfs.h"

namespace {

// Partial sums of up to kReduceBlocks blocks (two slots each), the two
// results, and two reduction tickets.
constexpr size_t kNormsStaticBytes = 10240;
constexpr size_t kPartialBytes = 2 * pfs::kReduceBlocks * sizeof(double);
constexpr size_t kResultOffset = kPartialBytes;
constexpr size_t kTicketOffset = kPartialBytes + 2 * sizeof(double);
static_assert(kTicketOffset + 2 * sizeof(unsigned) <= kNormsStaticBytes, "static norm scratch too small");

// Largest grid this entry point accepts (cells); the reduction itself needs
// the same fixed scratch for any grid, the bound is the library's index range.
constexpr long long kNormsStaticMaxCells = 1LL << 30;

static __device__ __align__(256) unsigned char g_norms_scratch[kNormsStaticBytes];

// Device address of g_norms_scratch in the current context. In host code the
// symbol itself is only a host-side stand-in, not a device address. It is
// looked up on every call (cudaGetSymbolAddress allocates nothing): a cached
// address would outlive a cudaDeviceReset, which reloads the module, and
// would belong to another context when a second driver context is current on
// the same device.
int scratch_for_current_device(void **out, const char **why)
{
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_norms_scratch);
    if (e != cudaSuccess || !ptr) {
        *why = cudaGetErrorString(e);
        return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? PFS_ERR_NO_DEVICE : PFS_ERR_CUDA;
    }
    *out = ptr;
    return PFS_OK;
}

int fail_static(int code, const char *fmt, long long a = 0, long long b = 0, long long c = 0)
{
    char msg[256];
    snprintf(msg, sizeof msg, fmt, a, b, c);
    return pfs::record_error(code, msg);
}

}  // namespace

extern "C" int pfs_residual_norms_static(const float *p, const float *b, int vx, int vy, int ld, double *rr,
                                         double *bb, void *stream)
{
    if (!p || !b || !rr || !bb) return fail_static(PFS_ERR_INVALID_ARGUMENT, "null argument");
    if (vx <= 0 || vy <= 0 || ld < vx)
        return fail_static(PFS_ERR_INVALID_ARGUMENT, "bad dims %lldx%lld (ld %lld)", vx, vy, ld);
    if ((long long)vx * vy > kNormsStaticMaxCells)
        return fail_static(PFS_ERR_INVALID_ARGUMENT,
                           "grid %lldx%lld exceeds the %lld cells pfs_residual_norms_static accepts", vx, vy,
                           kNormsStaticMaxCells);
    void *base = nullptr;
    const char *why = "";
    const int rc = scratch_for_current_device(&base, &why);
    if (rc != PFS_OK) return pfs::record_error(rc, why);
    unsigned char *scratch = static_cast<unsigned char *>(base);
    pfs::Reduce red;
    red.partials = reinterpret_cast<double *>(scratch);
    red.result = reinterpret_cast<double *>(scratch + kResultOffset);
    red.ticket = reinterpret_cast<unsigned *>(scratch + kTicketOffset);
    red.nblocks = pfs::reduce_grid();
    cudaStream_t st = (cudaStream_t)stream;
    double out[2];
    cudaError_t e = cudaMemsetAsync(red.ticket, 0, 2 * sizeof(unsigned), st);
    if (e == cudaSuccess) e = pfs::launch_norms(p, b, ld, vx, vy, red, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, red.result, sizeof out, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return pfs::record_error(PFS_ERR_CUDA, cudaGetErrorString(e));
    *rr = out[0];
    *bb = out[1];
    return PFS_OK;
}
