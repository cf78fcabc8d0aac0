"""Boundary modes of sessions (pfs_params.boundary) against the oracle and the
reference's own clamp mode (golden/clamp, made from src/fluid.cpp with its
commented clamp lines enabled), bit for bit."""
import numpy as np
import pytest

from golden_util import clamp_cases, load
from probabilistic_fluid_simulation_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", clamp_cases())
def test_clamp_sessions_match_reference_clamp_golden(cuda_device, pfs_lib, name):
    meta, arr = load(name)
    h, w, _ = arr["in_vp"].shape
    img = arr["in_img"]
    with pfs_lib.Session(w, h, image_shape=img.shape, dt=meta["dt"], viscosity=meta["viscosity"],
                         diffuse_iters=meta["iters"], max_iters=meta["iters"],
                         boundary=pfs_lib.BOUNDARY_CLAMP) as s:
        s.upload(arr["in_vp"], arr["in_tmp"], img)
        done = 0
        for snap in meta["snaps"]:
            s.step(snap - done)
            done = snap
            a, b, c = np.empty_like(arr["in_vp"]), np.empty_like(arr["in_tmp"]), np.empty_like(img)
            s.download(a, b, c)
            assert np.array_equal(a, arr[f"vp_s{snap}"]), (name, snap, "vp")
            assert np.array_equal(b, arr[f"tmp_s{snap}"]), (name, snap, "tmp")
            assert np.array_equal(c, arr[f"img_s{snap}"]), (name, snap, "img")


CASES = [  # w, h, image (w, h, c), viscosity, tol
    (64, 48, (64, 48, 3), 0.0, 0.0),      # image on the velocity grid: fused projection + image kernel
    (48, 40, (72, 56, 4), 0.0, 0.0),      # separate image grid
    (40, 32, (40, 32, 3), 0.05, 0.0),     # diffusion sweeps
    (128, 96, (128, 96, 3), 0.0, 1e-4),   # residual stop, fused sweeps
]


@pytest.mark.parametrize("boundary", [1, 2])
@pytest.mark.parametrize("w,h,img_shape,visc,tol", CASES)
def test_boundary_sessions_match_oracle(cuda_device, pfs_lib, oracle_mod, boundary, w, h, img_shape, visc, tol):
    vp, tmp, _, _ = S.initial_state(w, h, 3, seed=w + boundary)
    vp[..., 0:2] *= 300.0  # backtraces that leave the grid by several cells
    iw, ih, ic = img_shape
    img = S.blob_image(iw, ih, ic, seed=5)
    itmp = np.zeros_like(img)
    kw = dict(diffuse_iters=4, max_iters=40 if tol == 0 else 4000, tol=tol, check_every=100 if tol else 0)
    ov, ot, oi, oit = vp.copy(), tmp.copy(), img.copy(), itmp.copy()
    for _ in range(3):
        ov, ot, _ = oracle_mod.step(ov, ot, 0.1, visc, boundary=boundary, **kw)
        oi, oit = oracle_mod.advect_color_step(oi, oit, ov, 0.1, boundary=boundary)
    with pfs_lib.Session(w, h, image_shape=img.shape, dt=0.1, viscosity=visc, boundary=boundary, **kw) as s:
        s.upload(vp, tmp, img)
        s.step(3)
        a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
        s.download(a, b, c)
    assert np.array_equal(a, ov) and np.array_equal(b, ot) and np.array_equal(c, oi)
    if boundary == 2:
        for ch in (0, 1):
            u = a[..., ch]
            assert not u[0].any() and not u[-1].any() and not u[:, 0].any() and not u[:, -1].any()


def test_boundary_modes_rejected_where_unsupported(cuda_device, pfs_lib):
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.Session(64, 64, boundary=3)
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.Session(64, 64, boundary=1, diffuse_iters=2, precision=pfs_lib.PREC_BF16)
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.Session(1, 8, boundary=1)
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.Ensemble([(64, 64)], 3, diffuse_iters=2, boundary=1)
