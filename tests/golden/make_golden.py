"""Generate golden vectors by running the reference's own src/fluid.cpp.

Run in a checkout where the reference sources exist (default
/root/reference, override with PFS_REFERENCE):

    make -C oracle REF=<reference> && python tests/golden/make_golden.py

It builds nothing itself: oracle/Makefile compiles src/fluid.cpp unmodified
per NUM_JACOBI_ITERS into oracle/_ref/. Each case stores its inputs and the
reference's outputs, so the fixtures check the oracle and the CUDA path on
any host without the reference present.

Cases follow the shapes the reference's own tests use (3x3 and 2x2 fields
with channels 0-2 set to 1, src/test/test_pressure.cpp:9-37,52-75, and the
(-1,-1,-1,+1) scratch initialisation of src/main.cpp:186-195), plus seeded
vortex fields covering even and odd sweep counts, viscosity, rectangular
grids, an image whose resolution differs from the velocity grid, and
non-zero initial pressure in both buffers (the implicit warm start).
golden/clamp/ holds two cases of the reference's clamp mode (its commented
clamp lines enabled by oracle/Makefile).
The 256x256 / 40-sweep / 100-step workload is stored as SHA-256 digests of
the final buffers.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from probabilistic_fluid_simulation_gb300 import synthetic as S  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def run_ref(iters, vp, tmp, img, itmp, dt, visc, steps, snap_steps, variant=""):
    vp, tmp, img, itmp = vp.copy(), tmp.copy(), img.copy(), itmp.copy()
    snaps = {}
    for s in range(1, steps + 1):
        vp, tmp = O.ref_step(iters, vp, tmp, dt, visc, variant)
        img, itmp = O.ref_advect_color_step(iters, img, itmp, vp, dt, variant)
        if s in snap_steps:
            snaps[s] = (vp.copy(), tmp.copy(), img.copy(), itmp.copy())
    return snaps


def save_case(name, iters, vp, tmp, img, itmp, dt, visc, steps, snap_steps, variant="", out=OUT):
    snaps = run_ref(iters, vp, tmp, img, itmp, dt, visc, steps, snap_steps, variant)
    arrays = dict(in_vp=vp, in_tmp=tmp, in_img=img, in_itmp=itmp)
    for s, (a, b, c, d) in snaps.items():
        arrays[f"vp_s{s}"] = a
        arrays[f"tmp_s{s}"] = b
        arrays[f"img_s{s}"] = c
        arrays[f"itmp_s{s}"] = d
    meta = dict(iters=iters, dt=dt, viscosity=visc, steps=steps, snaps=sorted(snaps))
    if variant:
        meta["variant"] = variant
    os.makedirs(out, exist_ok=True)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), meta=json.dumps(meta), **arrays)
    print("wrote", name, {k: v.shape for k, v in arrays.items() if k.startswith("in_")})


def ones_fixture(n):
    vp = np.zeros((n, n, 4), np.float32)
    vp[..., 0:3] = 1.0
    tmp = np.empty_like(vp)
    tmp[..., 0:3] = -1.0
    tmp[..., 3] = 1.0
    img = np.linspace(0.0, 1.0, n * n * 4, dtype=np.float32).reshape(n, n, 4)
    return vp, tmp, img, np.zeros_like(img)


def noisy_scratch(shape, seed):
    rng = S.SplitMix64(seed)
    vals = np.array([rng.uniform(-1.0, 1.0) for _ in range(int(np.prod(shape)))], np.float32)
    return vals.reshape(shape)


def main():
    for it in (1, 2, 3, 30, 40):
        if not O.ref_available(it):
            sys.exit(f"oracle/_ref/libfluidref_it{it}.so missing: run make -C oracle first")

    # Reference-test shapes (src/test/test_pressure.cpp) with src/main.cpp scratch init.
    save_case("ones3x3_it30", 30, *ones_fixture(3), dt=0.1, visc=0.0, steps=2, snap_steps=(1, 2))
    save_case("ones2x2_it30", 30, *ones_fixture(2), dt=0.1, visc=0.0, steps=2, snap_steps=(1, 2))

    # Seeded vortex fields.
    vp, tmp, img, itmp = S.initial_state(32, 24, 3, seed=11)
    save_case("vortex32x24_it40", 40, vp, tmp, img, itmp, dt=0.1, visc=0.0, steps=4, snap_steps=(1, 4))

    for it, seed in ((1, 12), (2, 13), (3, 14)):
        vp = S.vortex_field(20, 14, seed)
        # non-zero initial pressure / divergence in both buffers: pins which
        # buffer's channel 2 seeds the pressure iteration for odd and even counts
        vp[..., 2:4] = noisy_scratch((14, 20, 2), seed)
        tmp = noisy_scratch((14, 20, 4), seed + 100)
        img = S.blob_image(30, 21, 4, seed)  # image grid differs from velocity grid
        itmp = np.zeros_like(img)
        save_case(f"vortex20x14_it{it}_visc", it, vp, tmp, img, itmp, dt=0.1, visc=0.05, steps=3,
                  snap_steps=(1, 3))

    # The reference's clamp mode (its commented-out lines of src/fluid.cpp:44-45,101-102 enabled,
    # oracle/Makefile): kept apart in golden/clamp/, since the drop-in calls are periodic only.
    for it in (3, 30):
        if not O.ref_available(it, "_clamp"):
            sys.exit(f"oracle/_ref/libfluidref_clamp_it{it}.so missing: run make -C oracle first")
    clamp_dir = os.path.join(OUT, "clamp")
    vp, tmp, img, itmp = S.initial_state(32, 24, 3, seed=21)
    save_case("clamp_vortex32x24_it30", 30, vp, tmp, img, itmp, dt=0.1, visc=0.0, steps=3, snap_steps=(1, 3),
              variant="_clamp", out=clamp_dir)
    vp = S.vortex_field(20, 14, 22)
    vp[..., 2:4] = noisy_scratch((14, 20, 2), 22)
    tmp = noisy_scratch((14, 20, 4), 122)
    img = S.blob_image(30, 21, 4, 22)
    save_case("clamp_vortex20x14_it3_visc", 3, vp, tmp, img, np.zeros_like(img), dt=0.1, visc=0.05, steps=3,
              snap_steps=(1, 3), variant="_clamp", out=clamp_dir)

    # 256x256, 40 sweeps, dt=0.1, 100 steps, 3-channel image, seed 0: digests only.
    vp, tmp, img, itmp = S.initial_state(256, 256, 3, seed=0)
    inputs = {k: hashlib.sha256(a.tobytes()).hexdigest() for k, a in
              (("vp", vp), ("tmp", tmp), ("img", img), ("itmp", itmp))}
    snaps = run_ref(40, vp, tmp, img, itmp, 0.1, 0.0, 100, (1, 100))
    digests = {}
    for s, arrs in snaps.items():
        digests[str(s)] = {k: hashlib.sha256(a.tobytes()).hexdigest()
                           for k, a in zip(("vp", "tmp", "img", "itmp"), arrs)}
    rec = dict(w=256, h=256, channels=3, seed=0, iters=40, dt=0.1, viscosity=0.0, steps=100,
               input_digests=inputs, digests=digests,
               note="SHA-256 of float32 little-endian bytes of each buffer, roles after the step's swaps")
    with open(os.path.join(OUT, "c0_256_it40_digests.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print("wrote c0_256_it40_digests.json")


if __name__ == "__main__":
    main()
