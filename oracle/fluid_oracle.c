/*
 * CPU oracle for the per-timestep fluid update of
 * mdushkoff/Probabilistic_Fluid_Simulation (src/fluid.cpp:24-320).
 *
 * TEST INFRASTRUCTURE. This is a restatement of the reference algorithm used
 * only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as
 * the checker of the CUDA path. The product never links or calls it.
 *
 * Pinning: the float instantiation is checked bit-for-bit against the
 * reference's own src/fluid.cpp (compiled unmodified by oracle/Makefile into
 * oracle/_ref/) and against golden vectors produced by that build
 * (tests/golden/). Build flags: -O2 -ffp-contract=off (no FMA contraction on
 * any host, so x86-64 and aarch64 give identical bits).
 *
 * Symbols: pfso_*_f32 (float, the reference's arithmetic) and pfso_*_f64
 * (double, the FP64 run of the same method).
 */
#include <math.h>
#include <stdlib.h>

#ifdef _OPENMP
#include <omp.h>
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

typedef struct {
    int sweeps;          /* pressure sweeps performed this step */
    int checks;          /* residual evaluations performed */
    double rel_residual; /* last evaluated ||b - A p||/||b|| (-1 if none) */
    double bnorm;        /* ||b||_2 at the last evaluation (-1 if none) */
    int capped;          /* residual mode only: stopped at max_iters above tol */
} pfso_stats;

int pfso_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void pfso_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

#define REAL float
#define SFX _f32
#define FMOD fmodf
#include "fluid_oracle_body.h"
#undef REAL
#undef SFX
#undef FMOD

#define REAL double
#define SFX _f64
#define FMOD fmod
#include "fluid_oracle_body.h"
#undef REAL
#undef SFX
#undef FMOD
