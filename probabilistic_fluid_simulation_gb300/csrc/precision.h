// Host interface of the precision forms (precision.cu), used by the session
// calls in capi.cu.
#pragma once

#include <cuda_runtime.h>

#include "pfs.h"

namespace pfs {
namespace unet {
struct Net;
}

struct LpState;

struct LpParams {
    float dt;
    int max_iters;    // sweep cap (fixed count when tol <= 0)
    double tol;       // relative residual target (<= 0: fixed count)
    int check_every;  // sweeps between refinements / checks (0: 32 for the refined forms, only at the cap for FP64)
    int levels;       // sweeps fused per launch (refined forms)
    int chunk;        // rows per warp in the fused sweep
    int start_mode = PFS_START_PREVIOUS;  // PFS_START_PREVIOUS / _ZERO / _NETWORK
    unet::Net *net = nullptr;             // the network of a PFS_START_NETWORK start
    int coarsen = 1;                      // network run on the grid coarsened this many times
    int passes = 1;                       // network applications (later ones on the residual)
    int stall_window = 0;                 // residual mode: sweeps without a 1% fall that end the solve
};

struct LpOut {
    int sweeps = 0, checks = 0;
    double rel = -1.0, bnorm = -1.0;
    bool capped = false;
    int start_kind = PFS_START_PREVIOUS;
    double rel_start = -1.0;
    int start_passes = 0;
    bool stalled = false;
};

int lp_create(LpState **out, int form, int w, int h, int iw, int ih, int ic);
void lp_destroy(LpState *s);
// vp, tmp, image: interleaved float32 device buffers (the reference layout);
// the pressure iteration starts from channel 2 of tmp, as the reference's does
// with an even diffusion count.
int lp_upload(LpState *s, const float *vp, const float *tmp, const float *image, cudaStream_t st);
int lp_step(LpState *s, const LpParams &p, cudaStream_t st, LpOut &o);
// (u, v, pressure, divergence) and the image, interleaved, float32 or float64
int lp_download(LpState *s, float *vp, float *image, cudaStream_t st);
int lp_download_f64(LpState *s, double *vp, double *image, cudaStream_t st);

}  // namespace pfs
