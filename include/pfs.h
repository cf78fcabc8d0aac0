/*
 * pfs.h - C ABI of the GB300 (sm_103a) fluid step library libpfs_gb300.so.
 *
 * Drop-in replacement for the per-timestep update of
 * mdushkoff/Probabilistic_Fluid_Simulation: simulate_fluid_step and
 * advect_color_step, declared in includes/fluid.hpp:106-119 and implemented
 * on the CPU in src/fluid.cpp:298-320 (the semantics reproduced here) and on
 * the GPU in src/fluid.cu:282-317.
 *
 * Conventions (kept from the reference):
 *   - Fields are interleaved HWC float32: velocity (vy, vx, 4) with channels
 *     u, v, pressure, divergence (src/fluid.cpp:15-17, 234-235, 255); image
 *     (iy, ix, iz) with any channel count iz.
 *   - Boundaries are periodic everywhere (src/fluid.cpp:43-57, 159-162).
 *   - The caller owns every buffer. Calls may swap the caller's pointers, as
 *     the reference does (src/fluid.cpp:188-194, 260-266, 317-319).
 *   - Channels 2-3 of both velocity buffers are solver state carried between
 *     steps: the pressure iteration starts from the previous step's pressure.
 *
 * Differences from the reference:
 *   - Every call returns a status (PFS_OK == 0); the reference returns void
 *     and never checks a launch. pfs_last_error() describes the last failure
 *     of the calling thread.
 *   - NUM_JACOBI_ITERS (includes/fluid.hpp:11, a compile-time 30) is a
 *     runtime setting, pfs_set_jacobi_iters().
 *   - Work is issued on the stream set by pfs_set_stream() (default: the
 *     legacy default stream, as in the reference).
 *
 * No torch or CUDA C++ types appear in this interface; streams are passed as
 * void* (a cudaStream_t).
 */
#ifndef PFS_H_
#define PFS_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ---------------------------------------------------------------- */
enum {
    PFS_OK = 0,
    PFS_ERR_INVALID_ARGUMENT = 1, /* bad dims, null pointers, dt <= 0, ...        */
    PFS_ERR_CUDA = 2,             /* a CUDA call failed; see pfs_last_error()     */
    PFS_ERR_NOT_FINITE = 3,       /* NaN/Inf in an input that was checked         */
    PFS_ERR_UNSUPPORTED = 4,      /* option not available for these sizes         */
    PFS_ERR_NO_DEVICE = 5,        /* no CUDA device visible                        */
    PFS_ERR_DEVICE_TIMEOUT = 6    /* a bounded device-side wait ran out            */
};

/* Human-readable name of a status code. */
const char *pfs_status_string(int status);
/* Message of the calling thread's last failed call ("" if none). */
const char *pfs_last_error(void);
/* Library version as 10000*major + 100*minor + patch. */
int pfs_version(void);
/* Number of CUDA kernels this library has launched since it was loaded. */
long long pfs_kernel_launches(void);
/* Bounds-checking build (libpfs_gb300_bounds.so) only: the timestep's kernels
 * (fused and single sweeps, advection, diffusion, divergence, projection, image
 * advection, residuals, layout conversion) test each global access against the
 * extent of its buffer, skip one that falls outside (a load yields zero) and
 * record it. This call waits for the device, then reads and clears that record
 * over every kernel run since the previous call: out[0] the number of accesses
 * found outside, and for the first of them out[1] its site (1 fused-sweep p
 * row, 2 fused-sweep b row, 3 fused-sweep store, 4 fused-sweep level L-1
 * store, 5 single sweep, 6 advection, 7 diffusion, 8 divergence, 9 residual,
 * 10 projection, 11 image advection, 12 layout conversion, 13 auxiliary
 * passes), out[2] its source line, out[3] its element index and out[4] the
 * buffer's extent in elements. The normal build returns PFS_ERR_UNSUPPORTED. */
int pfs_bounds_status(long long out[5]);

/* ---- global settings --------------------------------------------------------- */
/* Sweep count of both diffusion and pressure per step; replaces
 * NUM_JACOBI_ITERS (includes/fluid.hpp:11). Default 30. n >= 0. */
int pfs_set_jacobi_iters(int n);
int pfs_get_jacobi_iters(void);
/* Stream for the drop-in calls below (a cudaStream_t, NULL = legacy default). */
int pfs_set_stream(void *stream);
/* Free the cached scratch of the drop-in calls and of pfs_residual_norms on
 * the current device. */
int pfs_release_workspace(void);

/* ---- drop-in: CUDA branch of includes/fluid.hpp -------------------------------- */
/*
 * One timestep on device buffers. Replaces
 *   void simulate_fluid_step(float **vp, float **tmp, float dt, float viscosity,
 *                            int vx, int vy, int vz);        (includes/fluid.hpp:107)
 * with the semantics of src/fluid.cpp:298-310: after the call channels 0-1 of
 * *vp hold the projected velocity, channel 2 of *tmp the final pressure and
 * channel 2 of *vp the one before it, channel 3 of both the divergence. vz
 * must be 4. Asynchronous on the library stream. The scratch (planar copies
 * of the fields) is allocated on first use per device and grid size and kept
 * until pfs_release_workspace().
 */
int pfs_simulate_fluid_step(float **vp, float **tmp, float dt, float viscosity, int vx, int vy, int vz);

/*
 * Image advection on device buffers, then swap *image and *itmp. Replaces
 *   void advect_color_step(float **image, float **itmp, float **vp, float dt,
 *                          int ix, int iy, int iz, int vx, int vy, int vz);
 *                                                            (includes/fluid.hpp:116)
 * with the semantics of src/fluid.cpp:72-127,312-320. Allocates nothing.
 */
int pfs_advect_color_step(float **image, float **itmp, float **vp, float dt, int ix, int iy, int iz, int vx, int vy,
                          int vz);

/* ---- drop-in: CPU branch of includes/fluid.hpp (host buffers, GPU compute) ----- */
/* Same layout as vp_field (includes/fluid.hpp:17-22). */
typedef struct {
    int x;
    int y;
    int z;
    float *data;
} pfs_vp_field;

/*
 * Replaces void simulate_fluid_step(vp_field *vp, vp_field *tmp, float dt,
 * float viscosity) (includes/fluid.hpp:109): host buffers in, host buffers
 * out, computed on the GPU (copies in, step, copies out; returns when the
 * host buffers hold the result). Pinned host memory copies fastest.
 */
int pfs_simulate_fluid_step_host(pfs_vp_field *vp, pfs_vp_field *tmp, float dt, float viscosity);
/* Replaces void advect_color_step(vp_field *image, vp_field *itmp, vp_field *vp,
 * float dt) (includes/fluid.hpp:118); swaps image->data and itmp->data. */
int pfs_advect_color_step_host(pfs_vp_field *image, pfs_vp_field *itmp, pfs_vp_field *vp, float dt);

/* ---- sessions: state kept on the device across steps ----------------------------- */
/*
 * A session holds one simulation resident in HBM in planar layout (one plane
 * per channel) and advances it many steps per call. It generalises the
 * reference loop (src/main.cpp:219-246: simulate_fluid_step then
 * advect_color_step) with:
 *   - separate diffusion and pressure sweep counts,
 *   - an optional residual stop: the pressure iteration ends at the first
 *     check point (every check_every sweeps, and at max_iters) where
 *     ||b - A p||_2 / ||b||_2 <= tol, A the 5-point periodic operator of
 *     src/fluid.cpp:239-257, evaluated per cell in FP64,
 *   - the buffer roles of src/fluid.cpp kept exactly (which buffer's
 *     pressure seeds the next solve depends on the sweep-count parities).
 * With tol <= 0 and diffuse_iters == max_iters == N, a step equals the
 * reference built with NUM_JACOBI_ITERS = N.
 */
enum { PFS_HOST = 0, PFS_DEVICE = 1 };

/* Storage / arithmetic form of a session:
 *   PFS_PREC_F32   the reference's float32 arithmetic, bit-exact (default; the fused sweep's
 *                  final multiply-add on b/4 rounds as the reference does for every value in
 *                  float32's normal range, above about 5e-38 in magnitude);
 *   PFS_PREC_BF16  velocity, image and the pressure correction stored bf16,
 *                  computed in FP32; the pressure held as a pair of floats
 *                  (about 48 significant bits), its residual and the
 *                  refinement update x += e evaluated exactly enough in
 *                  error-free float32 arithmetic (iterative refinement: the
 *                  same Jacobi iteration, different rounding);
 *   PFS_PREC_F16   the same with fp16 storage (the right-hand side of each
 *                  correction solve is scaled by 1/max|r| into fp16 range);
 *   PFS_PREC_F64   every field and operation in FP64: the FP64 run of the
 *                  same method, the yardstick for the others' error;
 *   PFS_PREC_F32R  velocity, image and the pressure correction stored
 *                  float32, the correction sweeps in FP32 (the fused sweep
 *                  kernel of the F32 form), the pressure pair and its
 *                  residual by the same refinement as BF16 / F16. Unlike F32,
 *                  whose float pressure stops falling near a relative residual
 *                  of 1e-4 on a 256x256 vortex grid and 1e-3 at 2048x2048, it
 *                  reaches tolerances far below 1e-5 (the pair's 48 bits).
 * The non-F32 forms run with viscosity 0 and an even diffusion count (the
 * reference's buffer roles then reduce to: pressure iteration from the
 * previous final pressure, projection with the final pressure); other
 * settings return PFS_ERR_UNSUPPORTED. check_every sets the sweeps between
 * refinements of the refined forms (0 means 32), except for F32R in residual
 * mode (tol > 0): there the correction sweeps run with the F32 form's fused
 * residual checks every check_every sweeps, and the refinement runs when
 * the correction's residual reaches the tolerance or every 0.025 * n^2 sweeps
 * (n the larger grid side; long before the float32 correction nears its
 * rounding floor), so the refinement pass is rare and the sweeps run at the F32
 * form's rate. */
enum { PFS_PREC_F32 = 0, PFS_PREC_BF16 = 1, PFS_PREC_F16 = 2, PFS_PREC_F64 = 3, PFS_PREC_F32R = 4 };

typedef struct {
    float dt;
    float viscosity;
    int diffuse_iters;  /* diffusion sweeps per step (reference: NUM_JACOBI_ITERS) */
    int max_iters;      /* pressure sweeps (fixed mode) or cap (residual mode)      */
    double tol;         /* > 0: residual mode; <= 0: exactly max_iters sweeps       */
    int check_every;    /* residual check interval in sweeps (0: only at the cap)   */
    int fuse_depth;     /* sweeps fused per launch, 0 = tuned default              */
    int chunk_rows;     /* rows per warp in the fused sweep, 0 = tuned default      */
    int want_residual;  /* fixed mode: also report the final residual              */
    int precision;      /* PFS_PREC_*                                              */
    int boundary;       /* PFS_BOUNDARY_* (sessions of the F32 form)               */
    int stall_sweeps;   /* residual mode: end the solve when the relative residual
                           has not fallen below 0.99 x its lowest value for this
                           many sweeps (the iterate has reached the rounding floor
                           of its storage; stats.stalled); < 0 picks a window
                           from the grid size, long enough that the exact
                           iteration's slowest mode falls 3% within it; 0 (the
                           default) never stops early                            */
} pfs_params;

/* Boundary mode of the advection (velocity and image):
 *   PFS_BOUNDARY_PERIODIC  the reference's wrapping mode (src/fluid.cpp:47-52,
 *                          105-106), default; every other operator is
 *                          periodic in all modes, as in the reference;
 *   PFS_BOUNDARY_CLAMP     the reference's commented-out clamp mode
 *                          (src/fluid.cpp:43-45, 100-102): the backtraced
 *                          coordinate is std::max(0.5f, std::min<float>(n - 1.5, x))
 *                          instead of wrapped;
 *   PFS_BOUNDARY_WALLS     clamp, and zero velocity on the boundary cells
 *                          (first and last row and column) after advection
 *                          and after projection: fixed zero-velocity walls.
 * The non-periodic modes need grid sides of at least 2; the drop-in calls and
 * ensembles are periodic. */
enum { PFS_BOUNDARY_PERIODIC = 0, PFS_BOUNDARY_CLAMP = 1, PFS_BOUNDARY_WALLS = 2 };

typedef struct {
    int sweeps;          /* pressure sweeps of the last step               */
    int checks;          /* residual evaluations of the last step          */
    double rel_residual; /* last evaluated relative residual (-1 if none)   */
    double bnorm;        /* ||b||_2 of the last step                        */
    int capped;          /* last step stopped at max_iters above tol        */
    long long steps;     /* steps run by this session                       */
    long long total_sweeps;
    long long cap_hits;
    int start_kind;      /* initial pressure of the last step: PFS_START_* */
    double rel_start;    /* relative residual of that initial pressure (-1 if not evaluated) */
    int start_passes;    /* damped passes applied to a predicted start in the last step    */
    int stalled;         /* last step ended because its residual stopped falling
                            (pfs_params.stall_sweeps)                                     */
} pfs_stats;

typedef struct pfs_session pfs_session;

/* Defaults: dt 0.1, viscosity 0, 30/30 sweeps, fixed mode. */
void pfs_params_default(pfs_params *p);
/* vx, vy: velocity grid; ix, iy, iz: image (iz = 0 for no image). */
int pfs_session_create(pfs_session **out, int vx, int vy, int ix, int iy, int iz, const pfs_params *params,
                       void *stream);
int pfs_session_set_params(pfs_session *s, const pfs_params *params);
/* Load state from interleaved buffers (vp, tmp: (vy, vx, 4); image (iy, ix, iz)),
 * host or device pointers per `where`. image may be NULL when iz == 0. */
int pfs_session_upload(pfs_session *s, const float *vp, const float *tmp, const float *image, int where);
/* Advance n steps (asynchronous unless the residual mode needs a host decision). */
int pfs_session_step(pfs_session *s, int n);
/* Write the state back in the reference layout (the buffers the reference's
 * vp, tmp and image pointers would designate after the same steps). */
int pfs_session_download(pfs_session *s, float *vp, float *tmp, float *image, int where);
/* The state in float64, interleaved: vp (u, v, pressure, divergence) and the
 * image. For the F32 form the pressure is the final iterate (tmp's channel 2). */
int pfs_session_download_f64(pfs_session *s, double *vp, double *image, int where);
int pfs_session_stats(pfs_session *s, pfs_stats *out);
/* Waits for the steps and for the asynchronous transfers queued so far. */
int pfs_session_sync(pfs_session *s);
int pfs_session_destroy(pfs_session *s);

/* ---- asynchronous host transfers ------------------------------------------------------ */
/*
 * For a stream of states in and results out, with the copies running on the
 * session's own copy streams beside the steps (the reference's CLI declares
 * NUM_STREAMS for this and never uses it, src/main.cpp:30,198-200). Host
 * buffers should be pinned (page-locked): pageable ones work, but their copies
 * cannot overlap the steps.
 *
 * pfs_session_upload_async queues a state, host buffers laid out as for
 * pfs_session_upload. Its host-to-device copy starts at once; the state
 * replaces the session's state when the next pfs_session_step begins (each
 * pfs_session_step call takes the oldest queued state, if any). At most
 * PFS_IO_SLOTS states can be queued; one more returns
 * PFS_ERR_INVALID_ARGUMENT. The buffers must stay unchanged until
 * pfs_session_wait_io or pfs_session_sync returns.
 *
 * pfs_session_download_async queues a copy of the state as it stands after
 * the steps queued so far into host buffers (any may be NULL), laid out as
 * for pfs_session_download, and returns at once; the buffers hold the result
 * when pfs_session_wait_io or pfs_session_sync returns. Up to PFS_IO_SLOTS
 * downloads are in flight; a further one makes the device (not the host)
 * wait for the oldest.
 *
 * pfs_session_wait_io waits for every transfer queued so far, not for steps
 * queued after them. Downloads of any kind read the state as it stands,
 * whatever uploads are queued; pfs_session_upload returns
 * PFS_ERR_INVALID_ARGUMENT while a queued upload has not been taken by a step.
 */
enum { PFS_IO_SLOTS = 2 };
int pfs_session_upload_async(pfs_session *s, const float *vp, const float *tmp, const float *image);
int pfs_session_download_async(pfs_session *s, float *vp, float *tmp, float *image);
int pfs_session_wait_io(pfs_session *s);

/* ---- learned warm start -------------------------------------------------------------- */
/*
 * A 4-level U-Net (3x3 circular convolutions, 16/32/64/64 channels, bf16
 * weights and activations, fp32 accumulation) mapping the divergence of a
 * step, normalised by its rms, to the pressure, normalised the same way. Its
 * forward and backward kernels are the library's own (tensor-core implicit
 * GEMM convolutions); training is forward_backward + adam_step on batches of
 * (b, p) pairs. Grids must have height and width multiples of 128. No
 * counterpart in the reference (whose pressure iteration always starts from
 * the previous pressure).
 */
typedef struct pfs_unet pfs_unet;
/* buffers for up to max_pixels pixels per batch (images x height x width) */
int pfs_unet_create(pfs_unet **out, long long max_pixels);
int pfs_unet_destroy(pfs_unet *u);
long long pfs_unet_num_params(pfs_unet *u);
int pfs_unet_set_params(pfs_unet *u, const float *host_params);
int pfs_unet_get_params(pfs_unet *u, float *host_params);
int pfs_unet_get_grads(pfs_unet *u, float *host_grads);
/* mean squared error of the prediction for n (b, p) pairs (dense float32
 * device arrays, n x h x w, already normalised) and the gradients of all
 * parameters; *loss receives the loss (blocking) if non-NULL */
int pfs_unet_forward_backward(pfs_unet *u, const float *b, const float *p, int n, int h, int w, float *loss,
                              void *stream);
int pfs_unet_adam_step(pfs_unet *u, float lr, void *stream);
/* p = rms(b) * net(b / rms(b)) for one plane (row pitches ldb, ldp floats) */
int pfs_unet_predict(pfs_unet *u, const float *b, int ldb, float *p, int ldp, int h, int w, void *stream);
/* the same with the network run on the grid coarsened `coarsen` times: b
 * averaged over coarsen x coarsen blocks, the prediction interpolated back
 * (periodic bilinear, fine cell i at coarse coordinate (i + 1/2)/coarsen - 1/2)
 * and scaled by coarsen^2 (the 5-point operator in cell units scales with the
 * cell size squared). Lets a network trained at side N serve grids of side
 * coarsen * N, whose features are coarsen times larger in cells. */
int pfs_unet_predict_coarse(pfs_unet *u, const float *b, int ldb, float *p, int ldp, int h, int w, int coarsen,
                            void *stream);

/* Initial pressure of each step's iteration:
 *   PFS_START_PREVIOUS  the previous step's pressure (the reference, default)
 *   PFS_START_ZERO      zero
 *   PFS_START_NETWORK   the network's prediction followed by
 *                       PFS_START_DAMP_PASSES damped Jacobi passes
 *                       p += (b - A p) / 8 (the undamped iteration cannot
 *                       reduce the checkerboard component of an error, which
 *                       a predicted start carries). If the residual of that
 *                       start is not finite or above PFS_START_SLACK times the
 *                       previous pressure's (a broken prediction), or the
 *                       residual stops falling between checks, the iteration
 *                       continues from the previous pressure (stats.start_kind
 *                       then reads PFS_START_FALLBACK). The slack is there
 *                       because the residual at the start overweights fine-scale
 *                       error, which the sweeps remove within tens of sweeps;
 *                       the sweeps needed are set by the smooth error. The
 *                       session keeps a pointer to u. Not available in the F64
 *                       form (the network reads float32 divergence). */
enum { PFS_START_PREVIOUS = 0, PFS_START_ZERO = 1, PFS_START_NETWORK = 2, PFS_START_FALLBACK = 3 };
enum { PFS_START_DAMP_PASSES = 8, PFS_START_SLACK = 4 };
int pfs_session_set_start(pfs_session *s, int mode, pfs_unet *u);
/* PFS_START_NETWORK with the network run on the grid coarsened `coarsen`
 * times (pfs_unet_predict_coarse; 1 = the session's grid) and applied
 * `passes` times (1..8): pass 1 predicts the pressure from b, each later pass
 * predicts the correction e of A e = r for the start's residual r = b - A p
 * and adds it (A is linear); every pass is followed by the damped passes.
 * pfs_session_set_start(s, PFS_START_NETWORK, u) is (coarsen 1, passes 1). */
int pfs_session_set_start_network(pfs_session *s, pfs_unet *u, int coarsen, int passes);

/* ---- ensembles: many independent simulations in one persistent kernel ------------ */
/*
 * n members with their own grid sizes (widths multiples of 4) and a common
 * image channel count, advanced together: each timestep of all members is one
 * cooperative launch (replayed from a CUDA graph where the driver accepts the
 * capture) that walks advection, divergence, phases of fused sweeps, residual
 * checks and projection + image advection with grid-wide barriers between
 * phases; members that converge stop taking sweep work. Each member's fields
 * are bit-identical to a session with the same parameters. Float32, viscosity
 * 0, even diffusion count; max_iters and check_every multiples of the fuse
 * depth (4 or 8). No counterpart in the reference, which runs one simulation.
 */
typedef struct pfs_ensemble pfs_ensemble;
int pfs_ensemble_create(pfs_ensemble **out, int n, const int *vx, const int *vy, int channels,
                        const pfs_params *params, void *stream);
/* member k's state in the reference layout (vp, tmp: (vy, vx, 4); image (vy, vx, channels)) */
int pfs_ensemble_upload(pfs_ensemble *e, int k, const float *vp, const float *tmp, const float *image, int where);
int pfs_ensemble_step(pfs_ensemble *e, int steps);
/* member k: vp = (u, v, final pressure, divergence) and the image */
int pfs_ensemble_download(pfs_ensemble *e, int k, float *vp, float *image, int where);
int pfs_ensemble_member_stats(pfs_ensemble *e, int k, pfs_stats *out);
/* tile configuration of the sweep phases (the autotuner's knobs) */
int pfs_ensemble_config(pfs_ensemble *e, int fuse_depth, int chunk_rows);
int pfs_ensemble_info(pfs_ensemble *e, int *fuse_depth, int *chunk_rows, int *grid_blocks, int *graphs);
/* restore == 0: copy the whole state aside (device to device); 1: put it back */
int pfs_ensemble_snapshot(pfs_ensemble *e, int restore);
/* Test hook for the bounded grid barrier: in the next pfs_ensemble_step,
 * block `block` of the step kernel leaves at once without reaching the first
 * barrier, so the other blocks' bounded wait runs out (about 1-2 s), they
 * return, and the step returns PFS_ERR_DEVICE_TIMEOUT (no fault, no hang).
 * The ensemble then stays failed: every later step returns the same status. */
int pfs_ensemble_debug_stall_block(pfs_ensemble *e, int block);
/* Ensemble statistics of the image field: for every pixel and channel, the
 * mean and the population variance (divide by n) over the n listed members,
 * which must share one grid size; FP64 accumulation in list order, float32
 * results interleaved (vy, vx, channels), host or device buffers per `where`.
 * Returns when the results are written. */
int pfs_ensemble_image_stats(pfs_ensemble *e, const int *members, int n, float *mean, float *var, int where);
int pfs_ensemble_destroy(pfs_ensemble *e);

/* ---- kernel-level entry points (tests, tuning, benchmarks) ------------------------ */
/*
 * `levels` pressure Jacobi sweeps (src/fluid.cpp:239-257) on planar fields:
 * p_out = J^levels(p_in) with divergence plane b; planes have row pitch ld
 * floats. fused != 0 uses the temporally blocked kernel (requires vx % 4 == 0,
 * ld % 4 == 0, 16-byte aligned planes); p_prev, if non-NULL, receives
 * J^(levels-1)(p_in). No allocation.
 */
int pfs_pressure_sweeps(const float *p_in, const float *b, float *p_out, float *p_prev, int vx, int vy, int ld,
                        int levels, int fused, int chunk_rows, void *stream);
/* ||b - A p||_2^2 and ||b||_2^2 (FP64) of planar p, b; blocking. The
 * reduction's scratch (about 10 KB per device, any grid size) is allocated on
 * the first call on a device and kept until pfs_release_workspace(). Any
 * pointer alignment is accepted: 16-byte aligned planes with vx and ld
 * multiples of 4 take a vector-load kernel, others a scalar one (the sums agree
 * to rounding). */
int pfs_residual_norms(const float *p, const float *b, int vx, int vy, int ld, double *rr, double *bb,
                       void *stream);

/*
 * pfs_residual_norms without any device allocation. No counterpart in the
 * reference (whose step allocates nothing and reports no residual); it exists
 * for callers that must not allocate device memory: a host application whose
 * device memory is entirely reserved by another allocator (a framework's
 * caching pool that owns the device) would get out-of-memory from cudaMalloc,
 * and a caller on a latency-critical path cannot afford cudaMalloc, which may
 * synchronize the device. pfs_residual_norms allocates its scratch on first use
 * per device; this call allocates nothing.
 *
 * Same kernel and same results as pfs_residual_norms. Its cross-block scratch
 * is a fixed 10 KiB array inside the library, present on every device that
 * loads the library until the process exits; each call looks up its address
 * in the current context. Not capturable in a CUDA graph: the call waits for
 * its results (cudaStreamSynchronize). Every call shares the array
 * and clears the part that must start at zero itself; calls that overlap on
 * the GPU (different streams running at the same time) race on it, so issue
 * them one after another. Grids above 2^30 cells are rejected with
 * PFS_ERR_INVALID_ARGUMENT. Blocking, like pfs_residual_norms.
 */
int pfs_residual_norms_static(const float *p, const float *b, int vx, int vy, int ld, double *rr, double *bb,
                              void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PFS_H_ */
