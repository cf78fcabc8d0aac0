// Device-side bounds checks of the timestep's kernels, compiled in only in the
// bounds-checking build of the library (PFS_BOUNDS_CHECK, libpfs_gb300_bounds.so;
// build.py builds it on request). In that build every checked access tests
// its element index against the extent of the buffer it belongs to (a plane
// of ld * h elements, an interleaved field of w * h * 4, an image of
// w * h * c); an access outside is not performed (a load yields zero) and is
// recorded instead: a count and, for the first one, the site tag, the source
// line, the index and the extent. The host reads and clears the record with
// pfs_bounds_status(). No access can leave its buffer, so a broken index shows
// up as a status, never as a memory fault. In the normal build the macros are
// the plain accesses and the library is unchanged.
//
// Each translation unit keeps its own record (internal linkage: no relocatable
// device code) and registers a reader for it with the host at load time.
#pragma once

#include <cuda_runtime.h>

namespace pfs {

struct BoundsRecord {
    unsigned long long count;  // checked accesses found outside their buffer
    int site;                  // BoundsSite of the first one
    int line;                  // its source line
    long long index;           // its element index (first element of a vector access)
    long long extent;          // the buffer's extent in elements
};

// Site tags of the checked accesses.
enum BoundsSite : int {
    kBsNone = 0,
    kBsSweepLoadP = 1,   // fused sweep: p rows copied into shared memory
    kBsSweepLoadB,       // fused sweep: b rows
    kBsSweepStore,       // fused sweep: level-L row
    kBsSweepStorePrev,   // fused sweep: level L-1 row
    kBsSweepSingle,      // single sweep
    kBsAdvect,           // velocity advection
    kBsDiffuse,          // diffusion sweep
    kBsDivergence,       // divergence
    kBsResidual,         // residual and norms
    kBsProject,          // projection
    kBsImage,            // image advection
    kBsLayout,           // interleaved <-> planar conversion
    kBsAux,              // damped pass, residual field, widen, add, small words
    kBsSites
};

#ifdef PFS_BOUNDS_CHECK

// Host: adds a translation unit's reader (defined in capi.cu).
void bounds_register(int (*read)(BoundsRecord *out, bool clear), const char *unit);

namespace {

__device__ BoundsRecord g_bounds_record;

__device__ __noinline__ void bounds_fail(int site, int line, long long index, long long extent)
{
    if (atomicAdd(&g_bounds_record.count, 1ull) == 0ull) {
        g_bounds_record.site = site;
        g_bounds_record.line = line;
        g_bounds_record.index = index;
        g_bounds_record.extent = extent;
    }
}

__device__ __forceinline__ bool bounds_span(long long i, long long count, long long n, int site, int line)
{
    if (i >= 0 && i + count <= n) return true;
    bounds_fail(site, line, i, n);
    return false;
}

template <typename T>
__device__ __forceinline__ T bounds_load(const T *p, long long i, long long n, int site, int line)
{
    return bounds_span(i, 1, n, site, line) ? p[i] : T{};
}

template <typename T, typename V>
__device__ __forceinline__ void bounds_store(T *p, long long i, long long n, V v, int site, int line)
{
    if (bounds_span(i, 1, n, site, line)) p[i] = v;
}

int bounds_read(BoundsRecord *out, bool clear)
{
    if (cudaMemcpyFromSymbol(out, g_bounds_record, sizeof *out) != cudaSuccess) return 1;
    if (clear) {
        const BoundsRecord zero{};
        if (cudaMemcpyToSymbol(g_bounds_record, &zero, sizeof zero) != cudaSuccess) return 1;
    }
    return 0;
}

struct BoundsRegistration {
    BoundsRegistration() { bounds_register(bounds_read, __BASE_FILE__); }
} g_bounds_registration;

}  // namespace

#define PFS_LD(p, i, n, site) ::pfs::bounds_load((p), (long long)(i), (long long)(n), (site), __LINE__)
#define PFS_ST(p, i, n, v, site) ::pfs::bounds_store((p), (long long)(i), (long long)(n), (v), (site), __LINE__)
#define PFS_SPAN(i, count, n, site) \
    ::pfs::bounds_span((long long)(i), (long long)(count), (long long)(n), (site), __LINE__)

#else

#define PFS_LD(p, i, n, site) ((p)[i])
#define PFS_ST(p, i, n, v, site) ((p)[i] = (v))
#define PFS_SPAN(i, count, n, site) true

#endif

}  // namespace pfs
