"""Runs the timestep's entry points through the bounds-checking build of the
library (PFS_LIBRARY must name libpfs_gb300_bounds.so) and prints one JSON
line per case: the device-side bounds record after it (pfs_bounds_status) and,
where the case has golden vectors of the reference, whether the results still
equal them. Used by test_gpu_bounds.py in a subprocess; needs a GPU."""
import json
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from golden_util import cases, load  # noqa: E402
from probabilistic_fluid_simulation_gb300 import fluid as F  # noqa: E402
from probabilistic_fluid_simulation_gb300 import synthetic as S  # noqa: E402

GRIDS = [(2, 1), (3, 5), (7, 3), (13, 11), (64, 48), (127, 61), (260, 5), (128, 130), (516, 36), (1000, 3)]


def emit(case, **kw):
    rec = F.bounds_status()
    print(json.dumps({"case": case, **rec, **kw}), flush=True)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def golden_dropin():
    for name in cases():
        meta, arrays = load(name)
        F.set_jacobi_iters(meta["iters"])
        vp, tmp = dev(arrays["in_vp"]), dev(arrays["in_tmp"])
        img, itmp = dev(arrays["in_img"]), dev(arrays["in_itmp"])
        equal = True
        for s in range(1, meta["steps"] + 1):
            vp, tmp = F.simulate_fluid_step(vp, tmp, meta["dt"], meta["viscosity"])
            img, itmp = F.advect_color_step(img, itmp, vp, meta["dt"])
            if s in meta["snaps"]:
                for k, t in (("vp", vp), ("tmp", tmp), ("img", img)):
                    equal &= bool(np.array_equal(t.cpu().numpy(), arrays[f"{k}_s{s}"]))
        emit("dropin " + name, equal=equal)
    F.set_jacobi_iters(30)


def sessions():
    for w, h in GRIDS:
        for bc in (0, 1, 2):
            vp, tmp, img, _ = S.initial_state(w, h, 3, seed=w + h)
            try:
                with F.Session(w, h, (h, w, 3), tol=1e-5, check_every=16, max_iters=200, boundary=bc) as s:
                    s.upload(vp, tmp, img)
                    s.step(2)
                    s.download(vp.copy(), tmp.copy(), img.copy())
            except F.PFSError as e:  # e.g. clamped boundaries on a side of 1: rejected on the host
                emit(f"session {w}x{h} boundary {bc}", rejected=str(e))
                continue
            emit(f"session {w}x{h} boundary {bc}")
    # an image grid unlike the velocity grid (drop-in image advection on its own grid)
    vp, tmp, _, _ = S.initial_state(100, 36, 3, seed=3)
    img = np.random.default_rng(0).random((72, 50, 4), dtype=np.float32)
    dv, dt_ = dev(vp), dev(tmp)
    dv, dt_ = F.simulate_fluid_step(dv, dt_, 0.1, 0.0)
    F.advect_color_step(dev(img), dev(np.zeros_like(img)), dv, 0.1)
    emit("dropin image 50x72x4 on velocity 100x36")


def precision_forms():
    for prec in (1, 2, 3, 4):  # the forms of include/pfs.h other than plain float32
        for w, h in ((260, 36), (128, 130)):
            vp, tmp, img, _ = S.initial_state(w, h, 3, seed=5)
            try:
                with F.Session(w, h, (h, w, 3), tol=1e-5, check_every=32, max_iters=300, precision=prec) as s:
                    s.upload(vp, tmp, img)
                    s.step(2)
            except F.PFSError as e:
                emit(f"precision {prec} {w}x{h}", rejected=str(e))
                continue
            emit(f"precision {prec} {w}x{h}")


def sweeps_and_norms():
    rng = np.random.default_rng(1)
    for w, h, ld in ((516, 37, 516), (260, 9, 264), (128, 1, 128), (1000, 130, 1008)):
        p = dev(rng.standard_normal((h, ld), dtype=np.float32))
        b = dev(rng.standard_normal((h, ld), dtype=np.float32))
        q = torch.empty_like(p)
        prev = torch.empty_like(p)
        rejected = []
        calls = [(lambda lv=lv, ch=ch: F.pressure_sweeps(p, b, q, prev, lv, fused=True, chunk_rows=ch, w=w), f"fused {lv}/{ch}")
                 for lv in range(1, 9) for ch in (0, 16, 7)]
        calls += [(lambda: F.pressure_sweeps(p, b, q, prev, 3, fused=False, w=w), "single"),
                  (lambda: F.residual_norms(p, b, w=w), "norms"), (lambda: F.residual_norms_static(p, b, w=w), "static")]
        for call, what in calls:
            try:
                call()
            except F.PFSError as e:  # a size the entry point does not take: rejected on the host
                rejected.append(f"{what}: {e}")
        emit(f"sweeps and norms {w}x{h} ld {ld}", rejected=rejected)


def ensemble():
    sizes = [(64, 64), (100, 36), (128, 130), (260, 5)]
    with F.Ensemble(sizes, 3, tol=1e-5, check_every=16, max_iters=200) as e:
        for k, (w, h) in enumerate(sizes):
            vp, tmp, img, _ = S.initial_state(w, h, 3, seed=k)
            e.upload(k, vp, tmp, img)
        e.step(2)
    emit("ensemble of 4")


if __name__ == "__main__":
    torch.cuda.set_device(0)
    golden_dropin()
    sessions()
    precision_forms()
    sweeps_and_norms()
    ensemble()
