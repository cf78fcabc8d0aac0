// C ABI of libpfs_gb300.so (include/pfs.h): drop-in step calls, sessions and
// kernel-level entry points, plus the host orchestration of one timestep.
//
// Buffer roles. The reference ping-pongs two interleaved buffers and swaps
// the caller's pointers (src/fluid.cpp:188-194, 260-266); which buffer ends
// up holding which iterate depends on the sweep counts. Here the fields live
// in planar form: two velocity slots (u, v planes) standing for the
// reference's two buffers, three pressure planes, and one divergence plane.
// The orchestration below tracks, exactly as the reference's pointer swaps
// would, which slot plays "vp" and "tmp" after each phase and which pressure
// plane is each slot's channel 2, so every channel of both buffers can be
// written back as the reference leaves it.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "bounds.cuh"
#include "kernels.h"
#include "nvtx.h"
#include "pfs.h"
#include "precision.h"
#include "unet.h"

using pfs::Reduce;

namespace pfs {
std::atomic<long long> g_launches{0};
}

namespace {

thread_local std::string g_err;
std::mutex g_mu;
int g_iters = 30;
cudaStream_t g_stream = nullptr;

int fail(int code, const char *fmt, ...)
{
    if (code == PFS_ERR_CUDA) cudaGetLastError();  // reported through the status; clear the non-sticky error
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace

int pfs::record_error(int code, const char *msg)
{
    if (code == PFS_ERR_CUDA) cudaGetLastError();  // reported through the status; clear the non-sticky error
    g_err = msg;
    return code;
}

namespace {

#define CK(x)                                                                                              \
    do {                                                                                                   \
        cudaError_t e_ = (x);                                                                              \
        if (e_ != cudaSuccess)                                                                             \
            return fail(PFS_ERR_CUDA, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#define CKS(x)                      \
    do {                            \
        int s_ = (x);               \
        if (s_ != PFS_OK) return s_; \
    } while (0)

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// ---------------------------------------------------------------------------------------------
// Planar fields of one velocity grid.
struct Field {
    int dev = -1, w = 0, h = 0, ld = 0;
    size_t plane = 0;  // floats per plane
    float *mem = nullptr;
    float *u[2] = {nullptr, nullptr}, *v[2] = {nullptr, nullptr}, *p[3] = {nullptr, nullptr, nullptr};
    float *b = nullptr;
    int pidx[2] = {0, 1};  // pressure plane holding channel 2 of velocity slot 0 / 1
    double *rmem = nullptr;
    unsigned *ticket = nullptr;
    double *hres = nullptr;  // pinned and mapped, [2]
    double *hres_d = nullptr;           // its device alias
    pfs::SolveState *dstate = nullptr;  // device
    pfs::SolveState *hstate = nullptr;  // pinned and mapped host copy
    pfs::SolveState *hstate_d = nullptr;
    float *pback = nullptr;             // plain start kept aside while a predicted start is tried
    float *pnet = nullptr;              // the network's correction in the later passes of a predicted start
    Reduce red{};
    // the fused check launches (one block per 4 sweep warp tasks): own partials,
    // red's result and tickets
    double *psweep = nullptr;
    Reduce red_sweep{};
    // check intervals in the first batch of the next residual-mode solve: 1 after a solve that
    // converged (doubling from there), as many as the capped one checked (at most 64) after one
    // that ran to the cap without converging
    int first_batch = 1;
    // residual checks run here, overlapping the sweep launch that follows them
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_check = nullptr, ev_res = nullptr;

    int make_aux()
    {
        if (aux) return PFS_OK;
        CK(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ev_check, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_res, cudaEventDisableTiming));
        return PFS_OK;
    }

    int alloc(int w_, int h_)
    {
        release();
        CK(cudaGetDevice(&dev));
        w = w_;
        h = h_;
        ld = round_up(w, 32);
        plane = (size_t)ld * h;
        CK(cudaMalloc(&mem, plane * 8 * sizeof(float)));
        CK(cudaMemset(mem, 0, plane * 8 * sizeof(float)));
        u[0] = mem;
        u[1] = mem + plane;
        v[0] = mem + 2 * plane;
        v[1] = mem + 3 * plane;
        p[0] = mem + 4 * plane;
        p[1] = mem + 5 * plane;
        p[2] = mem + 6 * plane;
        b = mem + 7 * plane;
        pidx[0] = 0;
        pidx[1] = 1;
        const int nb = pfs::kReduceBlocks;
        CK(cudaMalloc(&rmem, (2 * nb + 2) * sizeof(double) + 16));
        CK(cudaMemset(rmem, 0, (2 * nb + 2) * sizeof(double) + 16));
        ticket = reinterpret_cast<unsigned *>(rmem + 2 * nb + 2);
        // host copies of the check results: mapped, written by a kernel (launch_copy_small)
        CK(cudaHostAlloc(&hres, 2 * sizeof(double), cudaHostAllocMapped));
        CK(cudaHostGetDevicePointer((void **)&hres_d, hres, 0));
        CK(cudaMalloc(&dstate, sizeof(pfs::SolveState)));
        CK(cudaMemset(dstate, 0, sizeof(pfs::SolveState)));
        CK(cudaHostAlloc(&hstate, sizeof(pfs::SolveState), cudaHostAllocMapped));
        CK(cudaHostGetDevicePointer((void **)&hstate_d, hstate, 0));
        red.partials = rmem;
        red.result = rmem + 2 * nb;
        red.ticket = ticket;
        red.nblocks = pfs::reduce_grid();
        // capacity for the fused check launches at chunks of 16 rows or more
        const int ns = std::max(red.nblocks, pfs::sweep_stream_blocks(w, h, pfs::kMinChunkRows));
        CK(cudaMalloc(&psweep, 2 * (size_t)ns * sizeof(double)));
        red_sweep = red;
        red_sweep.partials = psweep;
        red_sweep.nblocks = ns;
        return PFS_OK;
    }
    void release()
    {
        if (mem) cudaFree(mem);
        if (rmem) cudaFree(rmem);
        if (psweep) cudaFree(psweep);
        psweep = nullptr;
        if (hres) cudaFreeHost(hres);
        if (dstate) cudaFree(dstate);
        if (hstate) cudaFreeHost(hstate);
        if (pback) cudaFree(pback);
        pback = nullptr;
        if (pnet) cudaFree(pnet);
        pnet = nullptr;
        if (ev_check) cudaEventDestroy(ev_check);
        if (ev_res) cudaEventDestroy(ev_res);
        if (aux) cudaStreamDestroy(aux);
        aux = nullptr;
        ev_check = ev_res = nullptr;
        mem = nullptr;
        rmem = nullptr;
        hres = nullptr;
        dstate = nullptr;
        hstate = nullptr;
        w = h = 0;
    }
    ~Field() { release(); }
};

struct Tuning {
    int levels = 8;  // sweeps fused per launch
    int halo = 8;    // halo columns per side of a warp strip (>= levels)
    int chunk = 32;  // rows per warp
};

struct StepCfg {
    float dt = 0.1f, visc = 0.0f;
    int D = 30, S = 30;
    double tol = 0.0;
    int check_every = 0;
    bool want_res = false;
    Tuning tun;
    int start_mode = PFS_START_PREVIOUS;
    pfs::unet::Net *net = nullptr;
    int coarsen = 1, passes = 1;  // predicted start: coarsening of the network's grid, network applications
    int bc = PFS_BOUNDARY_PERIODIC;  // boundary mode of the advection (pfs_params.boundary)
    int stall_window = 0;  // residual mode: sweeps without a 1% fall that end the solve (0: never)
};

struct StepOut {
    int sweeps = 0, checks = 0;
    double rel = -1.0, bnorm = -1.0;
    bool capped = false;
    int start_kind = PFS_START_PREVIOUS;
    double rel_start = -1.0;
    int start_passes = 0;
    bool stalled = false;
};

// The fused sweep needs rows of whole float4 vectors and addresses them by
// 32-bit vector offsets (planes below 2^33 cells); other grids take the
// single-sweep kernel.
bool fused_ok(const Field &f) { return f.w % 4 == 0 && (long long)f.h * (f.ld / 4) < (1LL << 31); }

// Sum r^2 of pressure plane `pp` and read back (r^2, b^2) (b^2 from the last divergence).
int residual_host(Field &f, const float *pp, cudaStream_t st, double &rr, double &bb)
{
    CK(pfs::launch_residual(pp, f.b, f.ld, f.w, f.h, f.red, nullptr, 0, 0.0, st));
    CK(pfs::launch_copy_small(f.red.result, f.hres_d, 2 * sizeof(double), st));
    CK(cudaStreamSynchronize(st));
    rr = f.hres[0];
    bb = f.hres[1];
    return PFS_OK;
}

double relative(double rr, double bb) { return bb > 0.0 ? std::sqrt(rr) / std::sqrt(bb) : std::sqrt(rr); }

// Plane roles after the launches that end at one check point.
struct CheckPoint {
    int sweeps, cur, prev;
};

// Pressure iteration of src/fluid.cpp:239-266 from slot X's plane (q_0) with
// Y's plane as the other buffer. Afterwards `cur` holds q_S and `prev` q_{S-1}.
//
// Residual mode: the sweeps are cut at check points (multiples of
// check_every, and the cap); after each, a residual launch evaluates the
// relative residual on the device and raises SolveState::done once it is at
// or below tol, which turns every later sweep and residual launch of the
// solve into an immediate return. The host enqueues check intervals in
// batches that double in size (1, 2, 4, ...; after a capped solve the first
// batch covers all its checks) and reads the state only between batches, then
// takes the plane roles recorded at the converged check point.
//
// With the fused sweep (width a multiple of 4) the last launch of each check
// interval evaluates the exact residual of its output itself
// (launch_sweep_stream_check: fused levels <= 7, so an interval's last
// 8-level launch is split 4 + 4): no second pass over p and b. Otherwise the
// residual launch runs on the field's second stream and overlaps the sweep
// launch that follows it: that launch reads q_S and b, as the residual does,
// and writes only the third plane. The launch after it (which overwrites q_S
// or q_{S-1}), any launch writing the q_{S-1} plane, the host's reads of the
// state and the end of the solve wait for the residual. If the check turns
// out converged, the one launch that ran meanwhile has written only the plane
// no role refers to.
int pressure_solve(Field &f, int X, int Y, const StepCfg &c, StepOut &o, cudaStream_t st, int &cur, int &prev)
{
    pfs::NvtxRange range("pfs.pressure");
    cur = f.pidx[X];
    prev = f.pidx[Y];
    int freep = 3 - cur - prev;
    const bool fused = fused_ok(f);
    const int L = std::max(1, std::min(c.tun.levels, c.tun.halo));
    const bool resid = c.tol > 0.0;
    // the last fused launch of each check interval evaluates the residual itself
    const bool check_fused =
        fused && resid && pfs::sweep_stream_blocks(f.w, f.h, c.tun.chunk) <= f.red_sweep.nblocks;
    const int *done = resid ? &f.dstate->done : nullptr;
    if (resid) CK(pfs::launch_zero_small(f.dstate, sizeof(pfs::SolveState), st));
    if (resid) CKS(f.make_aux());
    bool pending = false;  // a residual launch on f.aux that st has not waited for
    int since = 0;         // sweep launches since the last check
    auto settle = [&]() -> int {
        if (pending) CK(cudaStreamWaitEvent(st, f.ev_res, 0));
        pending = false;
        return PFS_OK;
    };

    CheckPoint marks[64];
    int nmarks = 0, batch = f.first_batch, in_batch = 0;
    int S = 0;
    bool finished = false;
    // predicted start: watch every check; if the residual does not fall, restart from the plain start
    const bool watch = resid && o.start_kind == PFS_START_NETWORK;
    double last_rel = o.rel_start;
    while (S < c.S && !finished) {
        int stop = c.S;
        if (resid && c.check_every > 0) stop = std::min(c.S, (S / c.check_every + 1) * c.check_every);
        while (S < stop) {
            if (!fused) {
                if (pending && since >= 1) CKS(settle());
                CK(pfs::launch_sweep_single(f.p[cur], f.b, f.p[freep], f.ld, f.w, f.h, done, st));
                ++since;
                const int old_prev = prev;
                prev = cur;
                cur = freep;
                freep = old_prev;
                S += 1;
                continue;
            }
            int n = std::min(L, stop - S);
            bool last = (S + n == stop);
            if (check_fused && last && n == 8) {  // the check launch fuses at most 7 levels: 8 = 4 + 4
                n = 4;
                last = false;
            }
            if (pending && (since >= 1 || last)) CKS(settle());
            if (check_fused && last)
                CK(pfs::launch_sweep_stream_check(f.p[cur], f.b, f.p[freep], f.p[prev], f.ld, f.w, f.h, n,
                                                  c.tun.chunk, f.red_sweep, f.dstate, S + n, c.tol, done, st,
                                                  c.stall_window));
            else
                CK(pfs::launch_sweep_stream(f.p[cur], f.b, f.p[freep], last ? f.p[prev] : nullptr, f.ld, f.w, f.h,
                                            n, c.tun.halo, c.tun.chunk, done, st));
            ++since;
            const int old_cur = cur;
            cur = freep;  // q_S; after a `last` launch prev holds q_{S-1}
            freep = old_cur;
            S += n;
        }
        if (!resid) break;
        if (!check_fused) {
            CK(cudaEventRecord(f.ev_check, st));
            CK(cudaStreamWaitEvent(f.aux, f.ev_check, 0));
            CK(pfs::launch_residual(f.p[cur], f.b, f.ld, f.w, f.h, f.red, f.dstate, S, c.tol, f.aux, c.stall_window));
            CK(cudaEventRecord(f.ev_res, f.aux));
            pending = true;
            since = 0;
        }
        marks[nmarks++] = {S, cur, prev};
        if (++in_batch == batch || S == c.S || nmarks == 64 || watch) {
            CKS(settle());
            CK(pfs::launch_copy_small(f.dstate, f.hstate_d, sizeof(pfs::SolveState), st));
            CK(cudaStreamSynchronize(st));
            if (f.hstate->done || S == c.S) finished = true;
            if (watch && !finished && o.start_kind == PFS_START_NETWORK) {
                if (!(f.hstate->rel < last_rel)) {  // the residual failed to fall: the plain start takes over
                    CK(cudaMemcpyAsync(f.p[cur], f.pback, f.plane * sizeof(float), cudaMemcpyDeviceToDevice, st));
                    o.start_kind = PFS_START_FALLBACK;
                }
                last_rel = f.hstate->rel;
            }
            if (nmarks == 64 && !finished) {  // keep the latest mark only
                marks[0] = marks[63];
                nmarks = 1;
            }
            in_batch = 0;
            batch = std::min(batch * 2, 16);
        }
    }
    CKS(settle());
    if (resid && nmarks > 0) {
        const pfs::SolveState &hs = *f.hstate;  // copied at the last sync
        o.checks = hs.checks;
        o.rel = hs.rel;
        o.bnorm = std::sqrt(hs.bb);
        if (hs.done) {
            int k = nmarks - 1;
            while (k > 0 && marks[k].sweeps != hs.sweeps) --k;
            if (marks[k].sweeps != hs.sweeps) return fail(PFS_ERR_CUDA, "lost the converged check point");
            S = hs.sweeps;
            cur = marks[k].cur;
            prev = marks[k].prev;
        }
    }
    o.sweeps = S;
    o.stalled = resid && nmarks > 0 && f.hstate->done == 2;
    o.capped = resid && S == c.S && !(o.rel <= c.tol) && !o.stalled;
    // a solve that ran to the cap is likely followed by another: enqueue all its checks in one batch
    // (one host read of the state instead of five for 20 checks); any converged solve resets to
    // doubling from 1, so at most one step after a change enqueues intervals that return at once
    if (resid) f.first_batch = o.capped ? std::max(1, std::min(64, o.checks)) : 1;
    if (c.want_res && !resid) {
        double rr, bb;
        CKS(residual_host(f, f.p[cur], st, rr, bb));
        o.bnorm = std::sqrt(bb);
        o.rel = relative(rr, bb);
    }
    return PFS_OK;
}

// Advection, diffusion, divergence and pressure of one step
// (src/fluid.cpp:298-304). `vp`/`tmp` are the velocity slots playing the
// reference's vp/tmp on entry. On return Z (the buffer projection reads, the
// reference's tmp after computePressure) and W (the one it writes, the
// reference's vp) are set; the caller projects Z -> W.
int velocity_phase(Field &f, int vp, int tmp, const StepCfg &c, StepOut &o, cudaStream_t st, int &Z, int &W)
{
    pfs::NvtxRange range("pfs.velocity");
    const int A = vp, B = tmp;
    // advect(vp, tmp): src/fluid.cpp:300
    CK(pfs::launch_advect(f.u[A], f.v[A], f.u[B], f.v[B], f.ld, f.w, f.h, c.dt, st, c.bc));

    // diffuse(tmp, vp): src/fluid.cpp:301. X ends as the reference's vp (it holds
    // the last diffusion iterate), Y as its tmp.
    int X = A, Y = B;
    if (c.D > 0) {
        if (c.visc == 0.0f) {
            // alpha = 0, beta = 1: every sweep returns its input (up to the sign
            // of zero), so all iterates equal the advected field; both slots get it.
            CK(cudaMemcpyAsync(f.u[A], f.u[B], f.plane * sizeof(float), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(f.v[A], f.v[B], f.plane * sizeof(float), cudaMemcpyDeviceToDevice, st));
            X = (c.D % 2) ? A : B;
            Y = (X == A) ? B : A;
        } else {
            const float alpha = c.visc * c.dt;
            const float beta = (float)(1.0 + 4.0 * (double)alpha);
            int src = B, dst = A;
            for (int k = 0; k < c.D; ++k) {
                CK(pfs::launch_diffuse_sweep(f.u[src], f.v[src], f.u[dst], f.v[dst], f.ld, f.w, f.h, alpha, beta, st));
                if (k != c.D - 1) std::swap(src, dst);
            }
            X = dst;
            Y = src;
        }
    }

    // computePressure(vp, tmp): src/fluid.cpp:303
    const float gamma = (float)(-1.0 / (double)c.dt);
    CK(pfs::launch_divergence(f.u[X], f.v[X], f.b, f.ld, f.w, f.h, gamma, f.red, st));
    o.start_kind = c.start_mode;
    if (c.start_mode == PFS_START_ZERO) {
        CK(cudaMemsetAsync(f.p[f.pidx[X]], 0, f.plane * sizeof(float), st));
    } else if (c.start_mode == PFS_START_NETWORK) {
        if (!f.pback) CK(cudaMalloc(&f.pback, f.plane * sizeof(float)));
        float *px = f.p[f.pidx[X]];
        CK(cudaMemcpyAsync(f.pback, px, f.plane * sizeof(float), cudaMemcpyDeviceToDevice, st));
        // damped passes go through the free plane (an even count ends in px)
        float *scratch = f.p[3 - f.pidx[X] - f.pidx[Y]];
        o.start_passes = 0;
        for (int pass = 0; pass < c.passes; ++pass) {
            if (pass == 0) {
                CKS(pfs::unet::predict_coarse(c.net, f.b, f.ld, px, f.ld, f.h, f.w, c.coarsen, st));
            } else {  // correction for the residual: A e = r, added to the start
                if (!f.pnet) CK(cudaMalloc(&f.pnet, f.plane * sizeof(float)));
                CK(pfs::launch_residual_field(px, f.b, scratch, f.ld, f.w, f.h, st));
                CKS(pfs::unet::predict_coarse(c.net, scratch, f.ld, f.pnet, f.ld, f.h, f.w, c.coarsen, st));
                CK(pfs::launch_add(px, f.pnet, f.plane, st));
            }
            for (int k = 0; k < PFS_START_DAMP_PASSES; ++k) {
                const bool even = (k % 2) == 0;
                CK(pfs::launch_damp(even ? px : scratch, f.b, even ? scratch : px, f.ld, f.w, f.h, st));
            }
            o.start_passes += PFS_START_DAMP_PASSES;
        }
        double rr, bb;
        CKS(residual_host(f, px, st, rr, bb));
        const double rel_net = relative(rr, bb);
        CKS(residual_host(f, f.pback, st, rr, bb));
        const double rel_plain = relative(rr, bb);
        if (rel_net <= PFS_START_SLACK * rel_plain) {
            o.rel_start = rel_net;
        } else {  // a broken prediction (or not finite): keep the plain start
            CK(cudaMemcpyAsync(px, f.pback, f.plane * sizeof(float), cudaMemcpyDeviceToDevice, st));
            o.start_kind = PFS_START_FALLBACK;
            o.rel_start = rel_plain;
        }
    }
    int cur = f.pidx[X], prev = f.pidx[Y];
    CKS(pressure_solve(f, X, Y, c, o, st, cur, prev));
    const int S = o.sweeps;
    if (S == 0) {
        Z = Y;
        W = X;
    } else {
        Z = (S % 2) ? Y : X;  // the reference's tmp after S-1 swaps
        W = (Z == X) ? Y : X;
        f.pidx[Z] = cur;
        f.pidx[W] = prev;
    }
    return PFS_OK;
}

// ---------------------------------------------------------------------------------------------
// Drop-in scratch: one Field per (device, grid), plus interleaved staging for host buffers.
struct Workspace {
    Field f;
    float *stage = nullptr;  // host-call staging: 2 velocity buffers
    size_t stage_bytes = 0;
    ~Workspace()
    {
        if (stage) cudaFree(stage);
    }
};
std::map<int, Workspace *> g_ws;  // keyed by device

int get_workspace(int w, int h, Workspace **out)
{
    int dev;
    CK(cudaGetDevice(&dev));
    Workspace *&ws = g_ws[dev];
    if (!ws) ws = new (std::nothrow) Workspace();
    if (!ws) return fail(PFS_ERR_CUDA, "out of host memory");
    if (ws->f.w != w || ws->f.h != h) CKS(ws->f.alloc(w, h));
    *out = ws;
    return PFS_OK;
}

// Scratch of pfs_residual_norms: the reduction's per-block partials, results
// and tickets (about 10 KB) and a pinned result pair, one set per device,
// sized for any grid; kept apart from the drop-in step's planar workspace so
// that norms at one grid size never reallocate the step's scratch.
struct NormScratch {
    double *rmem = nullptr;
    double *hres = nullptr;
    pfs::Reduce red{};
    ~NormScratch()
    {
        if (rmem) cudaFree(rmem);
        if (hres) cudaFreeHost(hres);
    }
};
std::map<int, NormScratch *> g_norms;  // keyed by device

int get_norm_scratch(NormScratch **out)
{
    int dev;
    CK(cudaGetDevice(&dev));
    NormScratch *&ns = g_norms[dev];
    if (!ns) {
        NormScratch *n = new (std::nothrow) NormScratch();
        if (!n) return fail(PFS_ERR_CUDA, "out of host memory");
        const int nb = pfs::kReduceBlocks;
        const size_t bytes = (2 * nb + 2) * sizeof(double) + 16;
        cudaError_t e = cudaMalloc(&n->rmem, bytes);
        if (e == cudaSuccess) e = cudaMemset(n->rmem, 0, bytes);
        if (e == cudaSuccess) e = cudaMallocHost(&n->hres, 2 * sizeof(double));
        if (e != cudaSuccess) {
            delete n;
            return fail(PFS_ERR_CUDA, "norm scratch: %s", cudaGetErrorString(e));
        }
        n->red.partials = n->rmem;
        n->red.result = n->rmem + 2 * nb;
        n->red.ticket = reinterpret_cast<unsigned *>(n->rmem + 2 * nb + 2);
        n->red.nblocks = pfs::reduce_grid();
        ns = n;
    }
    *out = ns;
    return PFS_OK;
}

int check_dims(int vx, int vy, int vz, float dt)
{
    if (vx <= 0 || vy <= 0) return fail(PFS_ERR_INVALID_ARGUMENT, "grid %dx%d must be positive", vx, vy);
    if ((long long)vx * vy > (1LL << 30)) return fail(PFS_ERR_INVALID_ARGUMENT, "grid %dx%d too large", vx, vy);
    if (vz != 4) return fail(PFS_ERR_INVALID_ARGUMENT, "velocity fields have 4 channels, got vz=%d", vz);
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(PFS_ERR_INVALID_ARGUMENT, "dt must be finite and > 0");
    return PFS_OK;
}

// The interleaved velocity kernels move one cell as a float4.
int check_aligned(const void *p, const char *what)
{
    if (((uintptr_t)p) % 16 != 0)
        return fail(PFS_ERR_INVALID_ARGUMENT, "%s must be 16-byte aligned (cudaMalloc pointers are)", what);
    return PFS_OK;
}

StepCfg dropin_cfg(float dt, float visc)
{
    StepCfg c;
    c.dt = dt;
    c.visc = visc;
    c.D = g_iters;
    c.S = g_iters;
    return c;
}

// Device-pointer step on interleaved buffers A (vp) and B (tmp).
int dropin_step(float *A, float *B, int w, int h, float dt, float visc, cudaStream_t st)
{
    Workspace *ws;
    CKS(get_workspace(w, h, &ws));
    Field &f = ws->f;
    f.pidx[0] = 0;
    f.pidx[1] = 1;
    CK(pfs::launch_split_velocity(A, f.u[0], f.v[0], f.ld, w, h, st));
    CK(pfs::launch_split_channel(A, 2, 4, f.p[0], f.ld, w, h, st));
    CK(pfs::launch_split_channel(B, 2, 4, f.p[1], f.ld, w, h, st));
    StepCfg c = dropin_cfg(dt, visc);
    StepOut o;
    int Z, W;
    CKS(velocity_phase(f, 0, 1, c, o, st, Z, W));
    // subtractPressureGradient(tmp, vp): src/fluid.cpp:304
    CK(pfs::launch_project(f.u[Z], f.v[Z], f.p[f.pidx[Z]], f.u[W], f.v[W], f.ld, w, h, dt, st));
    // With equal diffusion and pressure counts the roles always come back as
    // W = vp, Z = tmp, so the caller's pointers keep their buffers.
    CK(pfs::launch_merge_velocity(A, f.u[W], f.v[W], f.p[f.pidx[W]], f.b, f.ld, w, h, st));
    CK(pfs::launch_merge_velocity(B, f.u[Z], f.v[Z], f.p[f.pidx[Z]], f.b, f.ld, w, h, st));
    return PFS_OK;
}

}  // namespace

// =============================================================================================
// Public C ABI
// =============================================================================================

struct pfs_session {
    int dev = 0;
    cudaStream_t st = nullptr;
    Field f;
    int vpSlot = 0, tmpSlot = 1;
    int iw = 0, ih = 0, ic = 0, ild = 0;
    size_t iplane = 0;
    float *img_mem = nullptr;
    float *img[2] = {nullptr, nullptr};
    int icur = 0;
    float *stage = nullptr;
    size_t stage_bytes = 0;
    pfs_params prm{};
    pfs_stats stats{};
    pfs::LpState *lp = nullptr;  // precision forms other than F32
    int start_mode = PFS_START_PREVIOUS;
    pfs::unet::Net *net = nullptr;
    int net_coarsen = 1, net_passes = 1;
    // asynchronous host transfers: two device staging slots each way, copies on
    // the session's own copy streams, ordered against the compute stream by events
    struct IoSlot {
        float *buf = nullptr;
        cudaEvent_t copied = nullptr;  // upload: host-to-device copy done; download: device-to-host copy done
        cudaEvent_t used = nullptr;    // upload: split into the state done; download: merge into buf done
    };
    IoSlot up[PFS_IO_SLOTS], down[PFS_IO_SLOTS];
    cudaStream_t up_st = nullptr, down_st = nullptr;
    int up_head = 0, up_count = 0, down_next = 0;
    size_t io_floats = 0;  // floats per slot: vp, tmp, image
    ~pfs_session()
    {
        if (up_st) cudaStreamSynchronize(up_st);
        if (down_st) cudaStreamSynchronize(down_st);
        for (IoSlot *k : {&up[0], &up[1], &down[0], &down[1]}) {
            if (k->buf) cudaFree(k->buf);
            if (k->copied) cudaEventDestroy(k->copied);
            if (k->used) cudaEventDestroy(k->used);
        }
        if (up_st) cudaStreamDestroy(up_st);
        if (down_st) cudaStreamDestroy(down_st);
        if (img_mem) cudaFree(img_mem);
        if (stage) cudaFree(stage);
        if (lp) pfs::lp_destroy(lp);
    }
};
static_assert(PFS_IO_SLOTS == 2, "the slot destructor loop lists two slots each way");

extern "C" {

const char *pfs_status_string(int s)
{
    switch (s) {
    case PFS_OK: return "ok";
    case PFS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PFS_ERR_CUDA: return "CUDA error";
    case PFS_ERR_NOT_FINITE: return "non-finite input";
    case PFS_ERR_UNSUPPORTED: return "unsupported";
    case PFS_ERR_NO_DEVICE: return "no CUDA device";
    case PFS_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

const char *pfs_last_error(void) { return g_err.c_str(); }

int pfs_version(void) { return 200; }

long long pfs_kernel_launches(void) { return pfs::g_launches.load(std::memory_order_relaxed); }

#ifdef PFS_BOUNDS_CHECK
extern "C++" {
namespace pfs {
namespace {
struct BoundsUnit {
    int (*read)(BoundsRecord *, bool);
    const char *unit;
};
std::mutex &bounds_mu()
{
    static std::mutex m;
    return m;
}
std::vector<BoundsUnit> &bounds_units()
{
    static std::vector<BoundsUnit> v;
    return v;
}
}  // namespace
void bounds_register(int (*read)(BoundsRecord *, bool), const char *unit)
{
    std::lock_guard<std::mutex> lk(bounds_mu());
    bounds_units().push_back({read, unit});
}
}  // namespace pfs
}  // extern "C++"
#endif

int pfs_bounds_status(long long out[5])
{
#ifndef PFS_BOUNDS_CHECK
    (void)out;
    return fail(PFS_ERR_UNSUPPORTED, "this build has no bounds checks (libpfs_gb300_bounds.so has them)");
#else
    if (!out) return fail(PFS_ERR_INVALID_ARGUMENT, "null output");
    for (int k = 0; k < 5; ++k) out[k] = 0;
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(PFS_ERR_CUDA, "cudaDeviceSynchronize: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(pfs::bounds_mu());
    for (const pfs::BoundsUnit &u : pfs::bounds_units()) {
        pfs::BoundsRecord r{};
        if (u.read(&r, true) != 0) return fail(PFS_ERR_CUDA, "reading the bounds record of %s failed", u.unit);
        if (r.count == 0) continue;
        if (out[0] == 0) {
            out[1] = r.site;
            out[2] = r.line;
            out[3] = r.index;
            out[4] = r.extent;
        }
        out[0] += (long long)r.count;
    }
    return PFS_OK;
#endif
}

int pfs_set_jacobi_iters(int n)
{
    if (n < 0) return fail(PFS_ERR_INVALID_ARGUMENT, "sweep count must be >= 0");
    std::lock_guard<std::mutex> lk(g_mu);
    g_iters = n;
    return PFS_OK;
}

int pfs_get_jacobi_iters(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    return g_iters;
}

int pfs_set_stream(void *stream)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_stream = (cudaStream_t)stream;
    return PFS_OK;
}

int pfs_release_workspace(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    int dev;
    CK(cudaGetDevice(&dev));
    auto it = g_ws.find(dev);
    if (it != g_ws.end()) {
        CK(cudaDeviceSynchronize());
        delete it->second;
        g_ws.erase(it);
    }
    auto jt = g_norms.find(dev);
    if (jt != g_norms.end()) {
        CK(cudaDeviceSynchronize());
        delete jt->second;
        g_norms.erase(jt);
    }
    return PFS_OK;
}

int pfs_simulate_fluid_step(float **vp, float **tmp, float dt, float viscosity, int vx, int vy, int vz)
{
    pfs::NvtxRange range("pfs.simulate_fluid_step");
    if (!vp || !tmp || !*vp || !*tmp) return fail(PFS_ERR_INVALID_ARGUMENT, "null buffer");
    if (*vp == *tmp) return fail(PFS_ERR_INVALID_ARGUMENT, "vp and tmp must be distinct buffers");
    CKS(check_dims(vx, vy, vz, dt));
    if (!std::isfinite(viscosity)) return fail(PFS_ERR_NOT_FINITE, "viscosity must be finite");
    CKS(check_aligned(*vp, "vp"));
    CKS(check_aligned(*tmp, "tmp"));
    std::lock_guard<std::mutex> lk(g_mu);
    return dropin_step(*vp, *tmp, vx, vy, dt, viscosity, g_stream);
}

int pfs_advect_color_step(float **image, float **itmp, float **vp, float dt, int ix, int iy, int iz, int vx, int vy,
                          int vz)
{
    if (!image || !itmp || !vp || !*image || !*itmp || !*vp) return fail(PFS_ERR_INVALID_ARGUMENT, "null buffer");
    if (*image == *itmp) return fail(PFS_ERR_INVALID_ARGUMENT, "image and itmp must be distinct buffers");
    if (ix <= 0 || iy <= 0 || iz <= 0) return fail(PFS_ERR_INVALID_ARGUMENT, "bad image dims");
    CKS(check_dims(vx, vy, vz, dt));
    CKS(check_aligned(*vp, "vp"));
    cudaStream_t st;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        st = g_stream;
    }
    CK(pfs::launch_advect_image_interleaved(*image, *itmp, ix, iy, iz, *vp, vx, vy, dt, st));
    std::swap(*image, *itmp);  // src/fluid.cpp:317-319
    return PFS_OK;
}

int pfs_simulate_fluid_step_host(pfs_vp_field *vp, pfs_vp_field *tmp, float dt, float viscosity)
{
    if (!vp || !tmp || !vp->data || !tmp->data) return fail(PFS_ERR_INVALID_ARGUMENT, "null buffer");
    if (vp->x != tmp->x || vp->y != tmp->y || vp->z != tmp->z)
        return fail(PFS_ERR_INVALID_ARGUMENT, "vp and tmp dims differ");
    CKS(check_dims(vp->x, vp->y, vp->z, dt));
    if (!std::isfinite(viscosity)) return fail(PFS_ERR_NOT_FINITE, "viscosity must be finite");
    std::lock_guard<std::mutex> lk(g_mu);
    const int w = vp->x, h = vp->y;
    Workspace *ws;
    CKS(get_workspace(w, h, &ws));
    const size_t bytes = (size_t)w * h * 4 * sizeof(float);
    if (ws->stage_bytes < 2 * bytes) {
        if (ws->stage) cudaFree(ws->stage);
        ws->stage = nullptr;
        ws->stage_bytes = 0;
        CK(cudaMalloc(&ws->stage, 2 * bytes));
        ws->stage_bytes = 2 * bytes;
    }
    float *A = ws->stage, *B = ws->stage + (size_t)w * h * 4;
    cudaStream_t st = g_stream;
    CK(cudaMemcpyAsync(A, vp->data, bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B, tmp->data, bytes, cudaMemcpyHostToDevice, st));
    CKS(dropin_step(A, B, w, h, dt, viscosity, st));
    CK(cudaMemcpyAsync(vp->data, A, bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(tmp->data, B, bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return PFS_OK;
}

int pfs_advect_color_step_host(pfs_vp_field *image, pfs_vp_field *itmp, pfs_vp_field *vp, float dt)
{
    if (!image || !itmp || !vp || !image->data || !itmp->data || !vp->data)
        return fail(PFS_ERR_INVALID_ARGUMENT, "null buffer");
    if (image->x <= 0 || image->y <= 0 || image->z <= 0) return fail(PFS_ERR_INVALID_ARGUMENT, "bad image dims");
    if (itmp->x != image->x || itmp->y != image->y || itmp->z != image->z)
        return fail(PFS_ERR_INVALID_ARGUMENT, "image and itmp dims differ");
    CKS(check_dims(vp->x, vp->y, vp->z, dt));
    std::lock_guard<std::mutex> lk(g_mu);
    Workspace *ws;
    CKS(get_workspace(vp->x, vp->y, &ws));
    const size_t vbytes = (size_t)vp->x * vp->y * 4 * sizeof(float);
    const size_t ibytes = (size_t)image->x * image->y * image->z * sizeof(float);
    const size_t need = vbytes + 2 * ibytes;
    if (ws->stage_bytes < need) {
        if (ws->stage) cudaFree(ws->stage);
        ws->stage = nullptr;
        ws->stage_bytes = 0;
        CK(cudaMalloc(&ws->stage, need));
        ws->stage_bytes = need;
    }
    float *V = ws->stage, *I = ws->stage + vbytes / sizeof(float), *T = I + ibytes / sizeof(float);
    cudaStream_t st = g_stream;
    CK(cudaMemcpyAsync(V, vp->data, vbytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(I, image->data, ibytes, cudaMemcpyHostToDevice, st));
    CK(pfs::launch_advect_image_interleaved(I, T, image->x, image->y, image->z, V, vp->x, vp->y, dt, st));
    CK(cudaMemcpyAsync(itmp->data, T, ibytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::swap(image->data, itmp->data);  // src/fluid.cpp:317-319
    return PFS_OK;
}

// ---- sessions ------------------------------------------------------------------------------

void pfs_params_default(pfs_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->dt = 0.1f;
    p->viscosity = 0.0f;
    p->diffuse_iters = 30;
    p->max_iters = 30;
    p->tol = 0.0;
    p->check_every = 0;
    p->fuse_depth = 0;
    p->chunk_rows = 0;
    p->want_residual = 0;
    p->boundary = PFS_BOUNDARY_PERIODIC;
    p->stall_sweeps = 0;
}

static int check_params(const pfs_params *p)
{
    if (!p) return fail(PFS_ERR_INVALID_ARGUMENT, "null params");
    if (!(p->dt > 0.0f) || !std::isfinite(p->dt)) return fail(PFS_ERR_INVALID_ARGUMENT, "dt must be finite and > 0");
    if (!std::isfinite(p->viscosity)) return fail(PFS_ERR_NOT_FINITE, "viscosity must be finite");
    if (p->diffuse_iters < 0 || p->max_iters < 0 || p->check_every < 0)
        return fail(PFS_ERR_INVALID_ARGUMENT, "sweep counts must be >= 0");
    if (p->fuse_depth < 0 || p->fuse_depth > 8) return fail(PFS_ERR_INVALID_ARGUMENT, "fuse_depth in [0, 8]");
    if (p->chunk_rows < 0) return fail(PFS_ERR_INVALID_ARGUMENT, "chunk_rows must be >= 0");
    if (std::isnan(p->tol)) return fail(PFS_ERR_NOT_FINITE, "tol is NaN");
    if (p->boundary < PFS_BOUNDARY_PERIODIC || p->boundary > PFS_BOUNDARY_WALLS)
        return fail(PFS_ERR_INVALID_ARGUMENT, "unknown boundary mode %d", p->boundary);
    if (p->boundary != PFS_BOUNDARY_PERIODIC && p->precision != PFS_PREC_F32)
        return fail(PFS_ERR_UNSUPPORTED, "boundary modes other than periodic run in the F32 form");
    if (p->precision < PFS_PREC_F32 || p->precision > PFS_PREC_F32R)
        return fail(PFS_ERR_INVALID_ARGUMENT, "unknown precision form %d", p->precision);
    if (p->precision != PFS_PREC_F32) {
        if (p->viscosity != 0.0f)
            return fail(PFS_ERR_UNSUPPORTED, "precision forms other than F32 run with viscosity 0");
        if (p->diffuse_iters < 2 || p->diffuse_iters % 2)
            return fail(PFS_ERR_UNSUPPORTED, "precision forms other than F32 need an even diffusion count >= 2");
    }
    return PFS_OK;
}

static StepCfg session_cfg(const pfs_session *s)
{
    StepCfg c;
    c.dt = s->prm.dt;
    c.visc = s->prm.viscosity;
    c.D = s->prm.diffuse_iters;
    c.S = s->prm.max_iters;
    c.tol = s->prm.tol;
    c.check_every = s->prm.check_every;
    c.want_res = s->prm.want_residual != 0;
    if (s->prm.fuse_depth > 0) c.tun.levels = s->prm.fuse_depth;
    c.tun.halo = c.tun.levels <= 4 ? 4 : 8;
    c.tun.chunk = s->prm.chunk_rows > 0 ? s->prm.chunk_rows : pfs::default_chunk(s->f.w, s->f.h, c.tun.levels);
    c.start_mode = s->start_mode;
    c.net = s->net;
    c.coarsen = s->net_coarsen;
    c.passes = s->net_passes;
    c.bc = s->prm.boundary;
    if (c.tol > 0.0 && s->prm.stall_sweeps != 0)
        c.stall_window = s->prm.stall_sweeps > 0 ? s->prm.stall_sweeps
                                                 : pfs::auto_stall_window(std::max(s->f.w, s->f.h), c.check_every);
    return c;
}

int pfs_session_create(pfs_session **out, int vx, int vy, int ix, int iy, int iz, const pfs_params *params,
                       void *stream)
{
    if (!out) return fail(PFS_ERR_INVALID_ARGUMENT, "null output");
    *out = nullptr;
    pfs_params def;
    pfs_params_default(&def);
    const pfs_params *p = params ? params : &def;
    CKS(check_params(p));
    CKS(check_dims(vx, vy, 4, p->dt));
    if (iz < 0 || (iz > 0 && (ix <= 0 || iy <= 0))) return fail(PFS_ERR_INVALID_ARGUMENT, "bad image dims");
    if (p->boundary != PFS_BOUNDARY_PERIODIC && (vx < 2 || vy < 2 || (iz > 0 && (ix < 2 || iy < 2))))
        return fail(PFS_ERR_INVALID_ARGUMENT, "clamped boundaries need grid sides of at least 2");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(PFS_ERR_NO_DEVICE, "no CUDA device");
    pfs_session *s = new (std::nothrow) pfs_session();
    if (!s) return fail(PFS_ERR_CUDA, "out of host memory");
    s->prm = *p;
    s->st = (cudaStream_t)stream;
    if ((p->precision == PFS_PREC_BF16 || p->precision == PFS_PREC_F16 || p->precision == PFS_PREC_F32R) &&
        vx % 4 != 0) {
        delete s;
        return fail(PFS_ERR_UNSUPPORTED, "the refined forms need a grid width divisible by 4");
    }
    if (p->precision != PFS_PREC_F32) {
        int rc = pfs::lp_create(&s->lp, p->precision, vx, vy, iz > 0 ? ix : 0, iz > 0 ? iy : 0, iz);
        if (rc == PFS_OK) CK(cudaGetDevice(&s->dev));
        if (rc != PFS_OK) {
            delete s;
            return rc;
        }
        s->f.w = vx;  // dims only; the planar F32 fields are not allocated for these forms
        s->f.h = vy;
        s->iw = ix;
        s->ih = iy;
        s->ic = iz;
        *out = s;
        return PFS_OK;
    }
    int rc = s->f.alloc(vx, vy);
    if (rc == PFS_OK) CK(cudaGetDevice(&s->dev));
    if (rc == PFS_OK && iz > 0) {
        s->iw = ix;
        s->ih = iy;
        s->ic = iz;
        s->ild = round_up(ix, 32);
        s->iplane = (size_t)s->ild * iy;
        cudaError_t e = cudaMalloc(&s->img_mem, 2 * s->iplane * iz * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(s->img_mem, 0, 2 * s->iplane * iz * sizeof(float));
        if (e != cudaSuccess) rc = fail(PFS_ERR_CUDA, "image allocation: %s", cudaGetErrorString(e));
        s->img[0] = s->img_mem;
        s->img[1] = s->img_mem + s->iplane * iz;
    }
    if (rc != PFS_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return PFS_OK;
}

int pfs_session_set_params(pfs_session *s, const pfs_params *params)
{
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    CKS(check_params(params));
    if (params->precision != s->prm.precision)
        return fail(PFS_ERR_INVALID_ARGUMENT, "the precision form is fixed at session creation");
    if (params->boundary != PFS_BOUNDARY_PERIODIC &&
        (s->f.w < 2 || s->f.h < 2 || (s->ic > 0 && (s->iw < 2 || s->ih < 2))))
        return fail(PFS_ERR_INVALID_ARGUMENT, "clamped boundaries need grid sides of at least 2");
    s->prm = *params;
    return PFS_OK;
}

static int session_stage(pfs_session *s, size_t bytes)
{
    if (s->stage_bytes >= bytes) return PFS_OK;
    if (s->stage) cudaFree(s->stage);
    s->stage = nullptr;
    s->stage_bytes = 0;
    CK(cudaMalloc(&s->stage, bytes));
    s->stage_bytes = bytes;
    return PFS_OK;
}

// The state from interleaved device buffers (vp, tmp, image), queued on the
// session stream.
static int apply_state(pfs_session *s, const float *A, const float *B, const float *I)
{
    if (s->lp) return pfs::lp_upload(s->lp, A, B, I, s->st);
    Field &f = s->f;
    f.pidx[0] = 0;
    f.pidx[1] = 1;
    s->vpSlot = 0;
    s->tmpSlot = 1;
    CK(pfs::launch_split_vp(A, f.u[0], f.v[0], f.p[0], f.b, f.ld, f.w, f.h, s->st));
    CK(pfs::launch_split_vp(B, f.u[1], f.v[1], f.p[1], nullptr, f.ld, f.w, f.h, s->st));
    if (s->ic > 0) {
        s->icur = 0;
        CK(pfs::launch_split_image(I, s->img[0], s->iplane, s->ild, s->iw, s->ih, s->ic, s->st));
    }
    return PFS_OK;
}

// The state into interleaved device buffers (any of them null: skipped), in
// the reference's layout, queued on the session stream.
static int merge_state(pfs_session *s, float *A, float *B, float *I)
{
    if (s->lp) {
        // (u, v, final pressure, divergence) into both velocity buffers
        if (A) CKS(pfs::lp_download(s->lp, A, I, s->st));
        if (B) CKS(pfs::lp_download(s->lp, B, A ? nullptr : I, s->st));
        if (!A && !B && I) CKS(pfs::lp_download(s->lp, nullptr, I, s->st));
        return PFS_OK;
    }
    Field &f = s->f;
    const int W = s->vpSlot, Z = s->tmpSlot;
    if (A) CK(pfs::launch_merge_velocity(A, f.u[W], f.v[W], f.p[f.pidx[W]], f.b, f.ld, f.w, f.h, s->st));
    if (B) CK(pfs::launch_merge_velocity(B, f.u[Z], f.v[Z], f.p[f.pidx[Z]], f.b, f.ld, f.w, f.h, s->st));
    if (I && s->ic > 0) CK(pfs::launch_merge_image(I, s->img[s->icur], s->iplane, s->ild, s->iw, s->ih, s->ic, s->st));
    return PFS_OK;
}

// A synchronous upload is refused while asynchronous ones wait for a step:
// the next step would replace its state by the oldest of them.
static int no_queued_upload(pfs_session *s)
{
    if (s->up_count > 0)
        return fail(PFS_ERR_INVALID_ARGUMENT, "an asynchronous upload is queued: step the session first");
    return PFS_OK;
}

int pfs_session_upload(pfs_session *s, const float *vp, const float *tmp, const float *image, int where)
{
    if (!s || !vp || !tmp) return fail(PFS_ERR_INVALID_ARGUMENT, "null argument");
    if (s->ic > 0 && !image) return fail(PFS_ERR_INVALID_ARGUMENT, "session has an image: pass it");
    CKS(no_queued_upload(s));
    Field &f = s->f;
    const size_t vcount = (size_t)f.w * f.h * 4, icount = (size_t)s->iw * s->ih * s->ic;
    const float *A = vp, *B = tmp, *I = image;
    if (where == PFS_HOST) {
        CKS(session_stage(s, (2 * vcount + icount) * sizeof(float)));
        float *dA = s->stage, *dB = s->stage + vcount, *dI = s->stage + 2 * vcount;
        CK(cudaMemcpyAsync(dA, vp, vcount * sizeof(float), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(dB, tmp, vcount * sizeof(float), cudaMemcpyHostToDevice, s->st));
        if (icount) CK(cudaMemcpyAsync(dI, image, icount * sizeof(float), cudaMemcpyHostToDevice, s->st));
        A = dA;
        B = dB;
        I = dI;
    } else if (where != PFS_DEVICE) {
        return fail(PFS_ERR_INVALID_ARGUMENT, "where must be PFS_HOST or PFS_DEVICE");
    } else {
        CKS(check_aligned(vp, "vp"));
        CKS(check_aligned(tmp, "tmp"));
    }
    CKS(apply_state(s, A, B, I));
    if (where == PFS_HOST) CK(cudaStreamSynchronize(s->st));
    return PFS_OK;
}

// Copy streams, events and the staging slots of the asynchronous transfers,
// made on first use.
static int io_init(pfs_session *s)
{
    if (s->up_st) return PFS_OK;  // made last: everything else is in place
    const size_t vcount = (size_t)s->f.w * s->f.h * 4, icount = (size_t)s->iw * s->ih * s->ic;
    s->io_floats = 2 * vcount + icount;
    // each piece only if missing, so a call after a failed one completes the set without leaking
    for (pfs_session::IoSlot *k : {&s->up[0], &s->up[1], &s->down[0], &s->down[1]}) {
        if (!k->buf) CK(cudaMalloc(&k->buf, s->io_floats * sizeof(float)));
        if (!k->copied) CK(cudaEventCreateWithFlags(&k->copied, cudaEventDisableTiming));
        if (!k->used) CK(cudaEventCreateWithFlags(&k->used, cudaEventDisableTiming));
    }
    if (!s->down_st) CK(cudaStreamCreateWithFlags(&s->down_st, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&s->up_st, cudaStreamNonBlocking));
    return PFS_OK;
}

int pfs_session_upload_async(pfs_session *s, const float *vp, const float *tmp, const float *image)
{
    pfs::NvtxRange range("pfs.upload_async");
    if (!s || !vp || !tmp) return fail(PFS_ERR_INVALID_ARGUMENT, "null argument");
    if (s->ic > 0 && !image) return fail(PFS_ERR_INVALID_ARGUMENT, "session has an image: pass it");
    if (s->up_count == PFS_IO_SLOTS)
        return fail(PFS_ERR_INVALID_ARGUMENT, "%d asynchronous uploads are queued already", PFS_IO_SLOTS);
    CKS(io_init(s));
    const size_t vcount = (size_t)s->f.w * s->f.h * 4, icount = (size_t)s->iw * s->ih * s->ic;
    pfs_session::IoSlot &k = s->up[(s->up_head + s->up_count) % PFS_IO_SLOTS];
    // the slot's previous contents must have been split into the state (no wait before the first use)
    CK(cudaStreamWaitEvent(s->up_st, k.used, 0));
    CK(cudaMemcpyAsync(k.buf, vp, vcount * sizeof(float), cudaMemcpyHostToDevice, s->up_st));
    CK(cudaMemcpyAsync(k.buf + vcount, tmp, vcount * sizeof(float), cudaMemcpyHostToDevice, s->up_st));
    if (icount)
        CK(cudaMemcpyAsync(k.buf + 2 * vcount, image, icount * sizeof(float), cudaMemcpyHostToDevice, s->up_st));
    CK(cudaEventRecord(k.copied, s->up_st));
    s->up_count++;
    return PFS_OK;
}

// The oldest queued upload becomes the state (queued on the session stream
// behind its copy).
static int apply_queued_upload(pfs_session *s)
{
    if (s->up_count == 0) return PFS_OK;
    const size_t vcount = (size_t)s->f.w * s->f.h * 4;
    pfs_session::IoSlot &k = s->up[s->up_head];
    CK(cudaStreamWaitEvent(s->st, k.copied, 0));
    CKS(apply_state(s, k.buf, k.buf + vcount, k.buf + 2 * vcount));
    CK(cudaEventRecord(k.used, s->st));
    s->up_head = (s->up_head + 1) % PFS_IO_SLOTS;
    s->up_count--;
    return PFS_OK;
}

int pfs_session_download_async(pfs_session *s, float *vp, float *tmp, float *image)
{
    pfs::NvtxRange range("pfs.download_async");
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    CKS(io_init(s));
    const size_t vcount = (size_t)s->f.w * s->f.h * 4, icount = (size_t)s->iw * s->ih * s->ic;
    pfs_session::IoSlot &k = s->down[s->down_next];
    s->down_next = (s->down_next + 1) % PFS_IO_SLOTS;
    // the slot's previous contents must have reached the host before the merge overwrites them
    CK(cudaStreamWaitEvent(s->st, k.copied, 0));
    float *A = vp ? k.buf : nullptr, *B = tmp ? k.buf + vcount : nullptr;
    float *I = (image && icount) ? k.buf + 2 * vcount : nullptr;
    CKS(merge_state(s, A, B, I));
    CK(cudaEventRecord(k.used, s->st));
    CK(cudaStreamWaitEvent(s->down_st, k.used, 0));
    if (A) CK(cudaMemcpyAsync(vp, A, vcount * sizeof(float), cudaMemcpyDeviceToHost, s->down_st));
    if (B) CK(cudaMemcpyAsync(tmp, B, vcount * sizeof(float), cudaMemcpyDeviceToHost, s->down_st));
    if (I) CK(cudaMemcpyAsync(image, I, icount * sizeof(float), cudaMemcpyDeviceToHost, s->down_st));
    CK(cudaEventRecord(k.copied, s->down_st));
    return PFS_OK;
}

int pfs_session_wait_io(pfs_session *s)
{
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    if (s->up_st) CK(cudaStreamSynchronize(s->up_st));
    if (s->down_st) CK(cudaStreamSynchronize(s->down_st));
    return PFS_OK;
}

int pfs_session_step(pfs_session *s, int n)
{
    if (!s || n < 0) return fail(PFS_ERR_INVALID_ARGUMENT, "bad session or step count");
    if (n > 0) CKS(apply_queued_upload(s));
    if (s->lp) {
        pfs::LpParams lp;
        lp.dt = s->prm.dt;
        lp.max_iters = s->prm.max_iters;
        lp.tol = s->prm.tol;
        lp.check_every = s->prm.check_every;
        lp.levels = s->prm.fuse_depth > 0 ? s->prm.fuse_depth : 8;
        lp.chunk = s->prm.chunk_rows > 0 ? s->prm.chunk_rows : pfs::default_chunk(s->f.w, s->f.h, lp.levels);
        lp.start_mode = s->start_mode;
        lp.net = s->net;
        lp.coarsen = s->net_coarsen;
        lp.passes = s->net_passes;
        if (lp.tol > 0.0 && s->prm.stall_sweeps != 0)
            lp.stall_window = s->prm.stall_sweeps > 0
                                  ? s->prm.stall_sweeps
                                  : pfs::auto_stall_window(std::max(s->f.w, s->f.h),
                                                           lp.check_every > 0 ? lp.check_every : 32);
        for (int k = 0; k < n; ++k) {
            pfs::NvtxRange range("pfs.step");
            pfs::LpOut o;
            CKS(pfs::lp_step(s->lp, lp, s->st, o));
            s->stats.start_kind = o.start_kind;
            s->stats.rel_start = o.rel_start;
            s->stats.start_passes = o.start_passes;
            s->stats.sweeps = o.sweeps;
            s->stats.checks = o.checks;
            s->stats.rel_residual = o.rel;
            s->stats.bnorm = o.bnorm;
            s->stats.capped = o.capped ? 1 : 0;
            s->stats.stalled = o.stalled ? 1 : 0;
            s->stats.steps += 1;
            s->stats.total_sweeps += o.sweeps;
            s->stats.cap_hits += o.capped ? 1 : 0;
        }
        return PFS_OK;
    }
    Field &f = s->f;
    const StepCfg c = session_cfg(s);
    for (int k = 0; k < n; ++k) {
        pfs::NvtxRange range("pfs.step");
        StepOut o;
        int Z, W;
        CKS(velocity_phase(f, s->vpSlot, s->tmpSlot, c, o, s->st, Z, W));
        pfs::NvtxRange project_range("pfs.project_image");
        const float *pz = f.p[f.pidx[Z]];
        if (s->ic > 0 && s->iw == f.w && s->ih == f.h) {
            float *src = s->img[s->icur], *dst = s->img[1 - s->icur];
            CK(pfs::launch_project_advect_image(f.u[Z], f.v[Z], pz, f.u[W], f.v[W], f.ld, f.w, f.h, c.dt, src, dst,
                                                s->iplane, s->ic, s->st, c.bc));
            s->icur = 1 - s->icur;
        } else {
            CK(pfs::launch_project(f.u[Z], f.v[Z], pz, f.u[W], f.v[W], f.ld, f.w, f.h, c.dt, s->st, c.bc));
            if (s->ic > 0) {
                float *src = s->img[s->icur], *dst = s->img[1 - s->icur];
                CK(pfs::launch_advect_image_planar(src, dst, s->iplane, s->ild, s->iw, s->ih, s->ic, f.u[W], f.v[W],
                                                   f.ld, f.w, f.h, c.dt, s->st, c.bc));
                s->icur = 1 - s->icur;
            }
        }
        s->vpSlot = W;
        s->tmpSlot = Z;
        s->stats.sweeps = o.sweeps;
        s->stats.checks = o.checks;
        s->stats.rel_residual = o.rel;
        s->stats.bnorm = o.bnorm;
        s->stats.capped = o.capped ? 1 : 0;
        s->stats.stalled = o.stalled ? 1 : 0;
        s->stats.steps += 1;
        s->stats.total_sweeps += o.sweeps;
        s->stats.cap_hits += o.capped ? 1 : 0;
        s->stats.start_kind = o.start_kind;
        s->stats.rel_start = o.rel_start;
        s->stats.start_passes = o.start_passes;
    }
    return PFS_OK;
}

int pfs_session_set_start_network(pfs_session *s, pfs_unet *u, int coarsen, int passes)
{
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    if (!u) return fail(PFS_ERR_INVALID_ARGUMENT, "network start needs a network");
    if (coarsen < 1 || passes < 1 || passes > 8)
        return fail(PFS_ERR_INVALID_ARGUMENT, "coarsen must be >= 1 and passes in [1, 8]");
    if (s->prm.precision == PFS_PREC_F64)
        return fail(PFS_ERR_UNSUPPORTED, "the F64 form has no network start (the network reads float32 divergence)");
    if (s->f.w % coarsen || s->f.h % coarsen || (s->f.w / coarsen) % 128 || (s->f.h / coarsen) % 128)
        return fail(PFS_ERR_UNSUPPORTED, "network start needs grid sides / coarsen that are multiples of 128");
    s->start_mode = PFS_START_NETWORK;
    s->net = reinterpret_cast<pfs::unet::Net *>(u);
    s->net_coarsen = coarsen;
    s->net_passes = passes;
    return PFS_OK;
}

int pfs_session_set_start(pfs_session *s, int mode, pfs_unet *u)
{
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    if (mode < PFS_START_PREVIOUS || mode > PFS_START_NETWORK)
        return fail(PFS_ERR_INVALID_ARGUMENT, "start mode must be PFS_START_PREVIOUS, _ZERO or _NETWORK");
    if (mode == PFS_START_NETWORK) return pfs_session_set_start_network(s, u, 1, 1);
    s->start_mode = mode;
    s->net = nullptr;
    return PFS_OK;
}

int pfs_session_download(pfs_session *s, float *vp, float *tmp, float *image, int where)
{
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    Field &f = s->f;
    const size_t vcount = (size_t)f.w * f.h * 4, icount = (size_t)s->iw * s->ih * s->ic;
    float *A = vp, *B = tmp, *I = image;
    if (where == PFS_HOST) {
        CKS(session_stage(s, (2 * vcount + icount) * sizeof(float)));
        A = vp ? s->stage : nullptr;
        B = tmp ? s->stage + vcount : nullptr;
        I = (image && icount) ? s->stage + 2 * vcount : nullptr;
    } else if (where != PFS_DEVICE) {
        return fail(PFS_ERR_INVALID_ARGUMENT, "where must be PFS_HOST or PFS_DEVICE");
    } else {
        if (vp) CKS(check_aligned(vp, "vp"));
        if (tmp) CKS(check_aligned(tmp, "tmp"));
    }
    CKS(merge_state(s, A, B, I));
    if (where == PFS_HOST) {
        if (vp) CK(cudaMemcpyAsync(vp, A, vcount * sizeof(float), cudaMemcpyDeviceToHost, s->st));
        if (tmp) CK(cudaMemcpyAsync(tmp, B, vcount * sizeof(float), cudaMemcpyDeviceToHost, s->st));
        if (I) CK(cudaMemcpyAsync(image, I, icount * sizeof(float), cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
    }
    return PFS_OK;
}

int pfs_session_download_f64(pfs_session *s, double *vp, double *image, int where)
{
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    if (where != PFS_HOST && where != PFS_DEVICE)
        return fail(PFS_ERR_INVALID_ARGUMENT, "where must be PFS_HOST or PFS_DEVICE");
    const size_t vcount = (size_t)s->f.w * s->f.h * 4, icount = (size_t)s->iw * s->ih * s->ic;
    double *A = vp, *I = image;
    if (where == PFS_HOST) {
        CKS(session_stage(s, (vcount + icount) * sizeof(double)));
        A = vp ? reinterpret_cast<double *>(s->stage) : nullptr;
        I = (image && icount) ? reinterpret_cast<double *>(s->stage) + vcount : nullptr;
    }
    if (s->lp) {
        CKS(pfs::lp_download_f64(s->lp, A, I, s->st));
    } else {
        // F32 form: the buffers in float32 (vp's velocity, tmp's final pressure), widened
        Field &f = s->f;
        float *tmp32 = nullptr;
        CK(cudaMallocAsync(&tmp32, (vcount * 2 + icount) * sizeof(float), s->st));
        const int W = s->vpSlot, Z = s->tmpSlot;
        CK(pfs::launch_merge_velocity(tmp32, f.u[W], f.v[W], f.p[f.pidx[Z]], f.b, f.ld, f.w, f.h, s->st));
        if (icount)
            CK(pfs::launch_merge_image(tmp32 + vcount, s->img[s->icur], s->iplane, s->ild, s->iw, s->ih, s->ic,
                                       s->st));
        CK(pfs::launch_widen(tmp32, A, vcount, s->st));
        if (I && icount) CK(pfs::launch_widen(tmp32 + vcount, I, icount, s->st));
        CK(cudaFreeAsync(tmp32, s->st));
    }
    if (where == PFS_HOST) {
        if (vp) CK(cudaMemcpyAsync(vp, A, vcount * sizeof(double), cudaMemcpyDeviceToHost, s->st));
        if (I) CK(cudaMemcpyAsync(image, I, icount * sizeof(double), cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
    }
    return PFS_OK;
}

int pfs_session_stats(pfs_session *s, pfs_stats *out)
{
    if (!s || !out) return fail(PFS_ERR_INVALID_ARGUMENT, "null argument");
    *out = s->stats;
    return PFS_OK;
}

int pfs_session_sync(pfs_session *s)
{
    if (!s) return fail(PFS_ERR_INVALID_ARGUMENT, "null session");
    CK(cudaStreamSynchronize(s->st));
    return pfs_session_wait_io(s);
}

int pfs_session_destroy(pfs_session *s)
{
    if (!s) return PFS_OK;
    cudaStreamSynchronize(s->st);
    delete s;
    return PFS_OK;
}

// ---- kernel-level entry points -------------------------------------------------------------

int pfs_pressure_sweeps(const float *p_in, const float *b, float *p_out, float *p_prev, int vx, int vy, int ld,
                        int levels, int fused, int chunk_rows, void *stream)
{
    if (!p_in || !b || !p_out) return fail(PFS_ERR_INVALID_ARGUMENT, "null plane");
    if (vx <= 0 || vy <= 0 || ld < vx) return fail(PFS_ERR_INVALID_ARGUMENT, "bad dims");
    if (levels < 1) return fail(PFS_ERR_INVALID_ARGUMENT, "levels must be >= 1");
    if (p_in == p_out || (p_prev && (p_prev == p_in || p_prev == p_out)))
        return fail(PFS_ERR_INVALID_ARGUMENT, "planes must be distinct");
    cudaStream_t st = (cudaStream_t)stream;
    if (fused) {
        if (vx % 4 || ld % 4 || ((uintptr_t)p_in | (uintptr_t)b | (uintptr_t)p_out | (uintptr_t)p_prev) % 16)
            return fail(PFS_ERR_UNSUPPORTED, "fused sweeps need vx %% 4 == 0, ld %% 4 == 0, 16-byte planes");
        if (levels > 8) return fail(PFS_ERR_UNSUPPORTED, "fused sweeps: at most 8 levels per call");
        if ((long long)vy * (ld / 4) >= (1LL << 31))
            return fail(PFS_ERR_UNSUPPORTED, "fused sweeps: planes must hold fewer than 2^33 cells");
        const int halo = levels <= 4 ? 4 : 8;
        CK(pfs::launch_sweep_stream(p_in, b, p_out, p_prev, ld, vx, vy, levels, halo,
                                    chunk_rows > 0 ? chunk_rows : pfs::default_chunk(vx, vy, levels), nullptr, st));
        return PFS_OK;
    }
    if (levels > 1 && !p_prev) return fail(PFS_ERR_INVALID_ARGUMENT, "unfused multi-sweep needs p_prev as scratch");
    // ping-pong so that the last sweep lands in p_out and the one before in p_prev
    const float *src = p_in;
    for (int k = 0; k < levels; ++k) {
        float *dst = ((levels - 1 - k) % 2 == 0) ? p_out : p_prev;
        CK(pfs::launch_sweep_single(src, b, dst, ld, vx, vy, nullptr, st));
        src = dst;
    }
    return PFS_OK;
}

int pfs_residual_norms(const float *p, const float *b, int vx, int vy, int ld, double *rr, double *bb, void *stream)
{
    if (!p || !b || !rr || !bb) return fail(PFS_ERR_INVALID_ARGUMENT, "null argument");
    if (vx <= 0 || vy <= 0 || ld < vx) return fail(PFS_ERR_INVALID_ARGUMENT, "bad dims");
    std::lock_guard<std::mutex> lk(g_mu);
    NormScratch *ns;
    CKS(get_norm_scratch(&ns));
    cudaStream_t st = (cudaStream_t)stream;
    CK(pfs::launch_norms(p, b, ld, vx, vy, ns->red, st));
    CK(cudaMemcpyAsync(ns->hres, ns->red.result, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *rr = ns->hres[0];
    *bb = ns->hres[1];
    return PFS_OK;
}

}  // extern "C"
