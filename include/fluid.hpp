/*
 * fluid.hpp - drop-in for the reference's includes/fluid.hpp
 * (mdushkoff/Probabilistic_Fluid_Simulation), backed by the GB300 library
 * libpfs_gb300.so through its C ABI (pfs.h).
 *
 * The reference header declares one of two signatures per call, chosen by
 * USE_CUDA (includes/fluid.hpp:106-119): host vp_field buffers for the CPU
 * build, device float** buffers for the CUDA build. Both are provided here as
 * overloads, host-only (no __global__ declarations), so a plain C++ compiler
 * can include this file. Semantics follow src/fluid.cpp:298-320 exactly,
 * including the swaps of the caller's pointers.
 *
 * Differences from the reference: failures throw pfs::error (the reference
 * has no error reporting); NUM_JACOBI_ITERS (includes/fluid.hpp:11) is the
 * runtime value pfs_set_jacobi_iters() sets, 30 unless changed.
 */
#ifndef PFS_FLUID_HPP_
#define PFS_FLUID_HPP_

#include <stdexcept>
#include <string>

#include "pfs.h"

/* Same layout as the reference's vp_field (includes/fluid.hpp:17-22). */
typedef pfs_vp_field vp_field;

namespace pfs {

struct error : std::runtime_error {
    int status;
    error(int s, const char *what) : std::runtime_error(std::string(pfs_status_string(s)) + ": " + what), status(s)
    {
    }
};

inline void check(int status)
{
    if (status != PFS_OK) throw error(status, pfs_last_error());
}

}  // namespace pfs

/* CPU branch (includes/fluid.hpp:109): host buffers, computed on the GPU. */
inline void simulate_fluid_step(vp_field *vp, vp_field *tmp, float dt, float viscosity)
{
    pfs::check(pfs_simulate_fluid_step_host(vp, tmp, dt, viscosity));
}

/* CPU branch (includes/fluid.hpp:118). */
inline void advect_color_step(vp_field *image, vp_field *itmp, vp_field *vp, float dt)
{
    pfs::check(pfs_advect_color_step_host(image, itmp, vp, dt));
}

/* CUDA branch (includes/fluid.hpp:107): device buffers, asynchronous. */
inline void simulate_fluid_step(float **vp, float **tmp, float dt, float viscosity, int vx, int vy, int vz)
{
    pfs::check(pfs_simulate_fluid_step(vp, tmp, dt, viscosity, vx, vy, vz));
}

/* CUDA branch (includes/fluid.hpp:116). */
inline void advect_color_step(float **image, float **itmp, float **vp, float dt, int ix, int iy, int iz, int vx,
                              int vy, int vz)
{
    pfs::check(pfs_advect_color_step(image, itmp, vp, dt, ix, iy, iz, vx, vy, vz));
}

#endif /* PFS_FLUID_HPP_ */
