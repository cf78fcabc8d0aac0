// A host program written against include/fluid.hpp the way the reference's
// src/main.cpp drives its CPU build (src/main.cpp:219-246): host vp_field
// buffers, simulate_fluid_step then advect_color_step each timestep.
//
//   dropin_main <in.bin> <out.bin> <steps> <dt> <viscosity> <iters>
//
// in.bin: int32 w, h, iw, ih, ic, then float32 vp (h*w*4), tmp (h*w*4),
// image (ih*iw*ic). out.bin: the same layout after the steps, buffers in the
// roles the calls leave them (vp, tmp, image, itmp).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fluid.hpp"

int main(int argc, char **argv)
{
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s in.bin out.bin steps dt viscosity iters\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int dims[5];
    if (std::fread(dims, sizeof(int), 5, f) != 5) return 2;
    const int w = dims[0], h = dims[1], iw = dims[2], ih = dims[3], ic = dims[4];
    const size_t nv = (size_t)w * h * 4, ni = (size_t)iw * ih * ic;
    std::vector<float> a(nv), b(nv), im(ni), it(ni, 0.0f);
    if (std::fread(a.data(), 4, nv, f) != nv || std::fread(b.data(), 4, nv, f) != nv ||
        std::fread(im.data(), 4, ni, f) != ni)
        return 2;
    std::fclose(f);

    vp_field vp = {w, h, 4, a.data()}, vtmp = {w, h, 4, b.data()};
    vp_field image = {iw, ih, ic, im.data()}, itmp = {iw, ih, ic, it.data()};
    const int steps = std::atoi(argv[3]);
    const float dt = (float)std::atof(argv[4]), visc = (float)std::atof(argv[5]);
    pfs::check(pfs_set_jacobi_iters(std::atoi(argv[6])));
    try {
        for (int i = 0; i < steps; ++i) {
            simulate_fluid_step(&vp, &vtmp, dt, visc);
            advect_color_step(&image, &itmp, &vp, dt);
        }
    } catch (const pfs::error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    std::fwrite(dims, sizeof(int), 5, o);
    std::fwrite(vp.data, 4, nv, o);
    std::fwrite(vtmp.data, 4, nv, o);
    std::fwrite(image.data, 4, ni, o);
    std::fwrite(itmp.data, 4, ni, o);
    std::fclose(o);
    return 0;
}
