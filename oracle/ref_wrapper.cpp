/*
 * Builds the reference's own src/fluid.cpp, unmodified, into a shared
 * library so tests can run it beside the oracle restatement.
 *
 * TEST INFRASTRUCTURE ONLY (output goes to oracle/_ref/, which is not part of
 * the product and is not committed).
 *
 * NUM_JACOBI_ITERS is a plain #define in includes/fluid.hpp:11 with no
 * #ifndef guard, so it cannot be overridden with -D. Instead this wrapper
 * defines the macro and the vp_field type itself (same layout as
 * includes/fluid.hpp:17-22) and pre-claims the header guard FLUID_HPP_
 * (includes/fluid.hpp:7-8) before including the .cpp, whose own
 * #include "../includes/fluid.hpp" then expands to nothing.
 *
 * The reference source path is passed as PFS_REF_SRC (a string literal) and
 * the sweep count as PFS_REF_ITERS by oracle/Makefile.
 */
#include <algorithm>  // std::max / std::min of the reference's clamp mode (the clamp build only)
#define NUM_JACOBI_ITERS (PFS_REF_ITERS)
typedef struct {
    int x;
    int y;
    int z;
    float *data;
} vp_field;
#define FLUID_HPP_
void advect(vp_field *vp, vp_field *vp_out, float dt);
void advect_color(vp_field *image, vp_field *out, vp_field *vp, float dt);
void diffuse(vp_field *vp, vp_field *vp_out, float viscosity, float dt);
void addForces(vp_field *vp, float *forces);
void computePressure(vp_field *vp, vp_field *vp_out, float dt);
void subtractPressureGradient(vp_field *vp, vp_field *vp_out, float dt);
void simulate_fluid_step(vp_field *vp, vp_field *tmp, float dt, float viscosity);
void advect_color_step(vp_field *image, vp_field *itmp, vp_field *vp, float dt);

#include PFS_REF_SRC

extern "C" {

int pfsref_num_jacobi_iters(void) { return NUM_JACOBI_ITERS; }

/* includes/fluid.hpp:109 (CPU branch), with the swapped data pointers
 * written back to the caller. */
void pfsref_simulate_fluid_step(float **vp, float **tmp, int w, int h, float dt, float viscosity)
{
    vp_field a = {w, h, 4, *vp};
    vp_field b = {w, h, 4, *tmp};
    simulate_fluid_step(&a, &b, dt, viscosity);
    *vp = a.data;
    *tmp = b.data;
}

/* includes/fluid.hpp:118 (CPU branch). */
void pfsref_advect_color_step(float **image, float **itmp, int iw, int ih, int ic,
                              float *vel, int vw, int vh, float dt)
{
    vp_field im = {iw, ih, ic, *image};
    vp_field it = {iw, ih, ic, *itmp};
    vp_field v = {vw, vh, 4, vel};
    advect_color_step(&im, &it, &v, dt);
    *image = im.data;
    *itmp = it.data;
}

} /* extern "C" */
