"""The CPU oracle against the reference: golden vectors made by the reference's
own src/fluid.cpp (tests/golden), the reference build itself where it is
present (oracle/_ref), and the oracle's generalisations (residual stop, FP64)."""
import hashlib

import numpy as np
import pytest

from golden_util import c0_digests, cases, load
from probabilistic_fluid_simulation_gb300 import synthetic as S


def run_oracle(O, arrays, meta, steps=None, dtype=np.float32):
    vp, tmp = arrays["in_vp"].astype(dtype), arrays["in_tmp"].astype(dtype)
    img, itmp = arrays["in_img"].astype(dtype), arrays["in_itmp"].astype(dtype)
    snaps = {}
    n = meta["iters"]
    for s in range(1, (steps or meta["steps"]) + 1):
        vp, tmp, _ = O.step(vp, tmp, meta["dt"], meta["viscosity"], diffuse_iters=n, max_iters=n)
        img, itmp = O.advect_color_step(img, itmp, vp, meta["dt"])
        snaps[s] = (vp.copy(), tmp.copy(), img.copy(), itmp.copy())
    return snaps


@pytest.mark.parametrize("name", cases())
def test_oracle_matches_golden_bitwise(oracle_mod, name):
    meta, arrays = load(name)
    snaps = run_oracle(oracle_mod, arrays, meta)
    for s in meta["snaps"]:
        for k, got in zip(("vp", "tmp", "img", "itmp"), snaps[s]):
            want = arrays[f"{k}_s{s}"]
            assert got.shape == want.shape
            assert np.array_equal(got, want), f"{name} step {s} buffer {k}: max |d| = {np.abs(got - want).max()}"


def test_golden_covers_reference_quirks():
    names = cases()
    # odd and even sweep counts, viscosity, the reference-test 2x2 / 3x3 shapes
    assert {"ones2x2_it30", "ones3x3_it30", "vortex20x14_it1_visc", "vortex20x14_it2_visc",
            "vortex20x14_it3_visc", "vortex32x24_it40"} <= set(names)


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.slow
def test_oracle_c0_256_100_steps_digests(oracle_mod):
    """256x256, 40 sweeps, dt 0.1, 100 steps (the CPU-runnable workload):
    every buffer after steps 1 and 100 equals the reference's, by SHA-256."""
    rec = c0_digests()
    vp, tmp, img, itmp = S.initial_state(rec["w"], rec["h"], rec["channels"], rec["seed"])
    assert {k: _digest(a) for k, a in (("vp", vp), ("tmp", tmp), ("img", img), ("itmp", itmp))} == \
        rec["input_digests"], "synthetic generator is not bit-reproducible on this host"
    n = rec["iters"]
    for s in range(1, rec["steps"] + 1):
        vp, tmp, _ = oracle_mod.step(vp, tmp, rec["dt"], rec["viscosity"], diffuse_iters=n, max_iters=n)
        img, itmp = oracle_mod.advect_color_step(img, itmp, vp, rec["dt"])
        if str(s) in rec["digests"]:
            got = {k: _digest(a) for k, a in (("vp", vp), ("tmp", tmp), ("img", img), ("itmp", itmp))}
            assert got == rec["digests"][str(s)], f"step {s}"


@pytest.mark.parametrize("iters", [1, 2, 3, 30, 40])
@pytest.mark.parametrize("shape,visc,img_shape", [((16, 16), 0.0, (16, 16, 3)), ((13, 9), 0.05, (20, 11, 4)),
                                                    ((1, 5), 0.0, (3, 2, 1))])
def test_oracle_matches_reference_build(oracle_mod, iters, shape, visc, img_shape):
    """Bitwise against src/fluid.cpp compiled unmodified (only where the
    reference sources were available to build oracle/_ref)."""
    if not oracle_mod.ref_available(iters):
        pytest.skip("reference build oracle/_ref not present on this host")
    w, h = shape
    vp = S.vortex_field(w, h, seed=iters)
    vp[..., 2] = np.linspace(-1, 1, w * h, dtype=np.float32).reshape(h, w)
    tmp = np.full_like(vp, -1.0)
    tmp[..., 3] = 1.0
    iw, ih, ic = img_shape
    img = S.blob_image(iw, ih, ic, seed=3)
    itmp = np.zeros_like(img)
    a = [vp.copy(), tmp.copy(), img.copy(), itmp.copy()]
    b = [vp.copy(), tmp.copy(), img.copy(), itmp.copy()]
    for _ in range(3):
        a[0], a[1] = oracle_mod.ref_step(iters, a[0], a[1], 0.1, visc)
        a[2], a[3] = oracle_mod.ref_advect_color_step(iters, a[2], a[3], a[0], 0.1)
        b[0], b[1], _ = oracle_mod.step(b[0], b[1], 0.1, visc, diffuse_iters=iters, max_iters=iters)
        b[2], b[3] = oracle_mod.advect_color_step(b[2], b[3], b[0], 0.1)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_residual_stop_rule(oracle_mod):
    """Residual mode stops at the first check point at or below tol, and the
    state equals a fixed-count run of that many sweeps."""
    vp0 = S.vortex_field(32, 32, seed=5)
    tmp0 = np.zeros_like(vp0)
    tol = 1e-3
    vp, tmp, st = oracle_mod.step(vp0.copy(), tmp0.copy(), 0.1, 0.0, diffuse_iters=2, max_iters=5000, tol=tol,
                                  check_every=10)
    assert st.sweeps % 10 == 0 and 0 < st.sweeps < 5000
    assert st.rel_residual <= tol and not st.capped
    vq, tq, st2 = oracle_mod.step(vp0.copy(), tmp0.copy(), 0.1, 0.0, diffuse_iters=2, max_iters=st.sweeps,
                                  want_residual=True)
    assert np.array_equal(vp, vq) and np.array_equal(tmp, tq)
    assert st2.rel_residual == pytest.approx(st.rel_residual, rel=1e-12)
    # one check earlier the residual was still above tol
    _, _, st3 = oracle_mod.step(vp0.copy(), tmp0.copy(), 0.1, 0.0, diffuse_iters=2, max_iters=st.sweeps - 10,
                                want_residual=True)
    assert st3.rel_residual > tol


def test_residual_cap(oracle_mod):
    vp0 = S.vortex_field(64, 64, seed=6)
    _, _, st = oracle_mod.step(vp0, np.zeros_like(vp0), 0.1, 0.0, diffuse_iters=2, max_iters=50, tol=1e-12,
                               check_every=20)
    assert st.sweeps == 50 and st.capped and st.checks == 3


def test_fp64_oracle_tracks_fp32(oracle_mod):
    """The FP64 run of the same method stays close to the FP32 run; used to
    measure the error of every result."""
    vp, tmp, img, itmp = S.initial_state(48, 40, 3, seed=9)
    v32, t32, i32, j32 = vp.copy(), tmp.copy(), img.copy(), itmp.copy()
    v64, t64, i64, j64 = (a.astype(np.float64) for a in (vp, tmp, img, itmp))
    for _ in range(5):
        v32, t32, _ = oracle_mod.step(v32, t32, 0.1, 0.0, diffuse_iters=40, max_iters=40)
        i32, j32 = oracle_mod.advect_color_step(i32, j32, v32, 0.1)
        v64, t64, _ = oracle_mod.step(v64, t64, 0.1, 0.0, diffuse_iters=40, max_iters=40)
        i64, j64 = oracle_mod.advect_color_step(i64, j64, v64, 0.1)
    for a, b in ((v32, v64), (t32, t64), (i32, i64)):
        scale = np.abs(b).max()
        assert np.abs(a - b).max() <= 1e-4 * scale


def test_oracle_threads_do_not_change_results(oracle_mod):
    vp, tmp, _, _ = S.initial_state(40, 24, 3, seed=2)
    old = oracle_mod.lib().pfso_num_threads()
    oracle_mod.set_threads(1)
    a = oracle_mod.step(vp.copy(), tmp.copy(), 0.1, 0.0, diffuse_iters=4, max_iters=100, tol=1e-6, check_every=7)
    oracle_mod.set_threads(4)
    b = oracle_mod.step(vp.copy(), tmp.copy(), 0.1, 0.0, diffuse_iters=4, max_iters=100, tol=1e-6, check_every=7)
    oracle_mod.set_threads(max(old, 1))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2].rel_residual == b[2].rel_residual


# ---- boundary modes -------------------------------------------------------------------------

from golden_util import clamp_cases  # noqa: E402


def _run_oracle(oracle_mod, meta, arr, boundary):
    vp, tmp = arr["in_vp"].copy(), arr["in_tmp"].copy()
    img, itmp = arr["in_img"].copy(), arr["in_itmp"].copy()
    out = {}
    for s in range(1, meta["steps"] + 1):
        vp, tmp, _ = oracle_mod.step(vp, tmp, meta["dt"], meta["viscosity"], diffuse_iters=meta["iters"],
                                     max_iters=meta["iters"], boundary=boundary)
        img, itmp = oracle_mod.advect_color_step(img, itmp, vp, meta["dt"], boundary=boundary)
        out[s] = (vp.copy(), tmp.copy(), img.copy(), itmp.copy())
    return out


@pytest.mark.parametrize("name", clamp_cases())
def test_oracle_clamp_matches_reference_clamp_golden(oracle_mod, name):
    """The restated clamp mode against the reference's own commented clamp
    lines, enabled (golden/clamp, made from that build)."""
    meta, arr = load(name)
    assert meta["variant"] == "_clamp"
    got = _run_oracle(oracle_mod, meta, arr, boundary=1)
    for s in meta["snaps"]:
        for k, a in zip(("vp", "tmp", "img", "itmp"), got[s]):
            assert np.array_equal(a, arr[f"{k}_s{s}"]), (name, s, k)


def test_clamp_cases_exist_and_differ_from_periodic(oracle_mod):
    assert len(clamp_cases()) >= 2
    meta, arr = load(clamp_cases()[0])
    clamp = _run_oracle(oracle_mod, meta, arr, boundary=1)[meta["steps"]]
    per = _run_oracle(oracle_mod, meta, arr, boundary=0)[meta["steps"]]
    assert not np.array_equal(clamp[0], per[0])


@pytest.mark.parametrize("iters,visc", [(3, 0.05), (30, 0.0)])
def test_oracle_clamp_matches_reference_clamp_build(oracle_mod, iters, visc):
    if not oracle_mod.ref_available(iters, "_clamp"):
        pytest.skip("reference clamp build oracle/_ref not present on this host")
    vp, tmp, img, itmp = S.initial_state(40, 28, 3, seed=iters)
    vp[..., 0:2] *= 500.0  # backtraces that leave the grid by several cells
    a = [vp.copy(), tmp.copy(), img.copy(), itmp.copy()]
    b = [vp.copy(), tmp.copy(), img.copy(), itmp.copy()]
    for _ in range(3):
        a[0], a[1] = oracle_mod.ref_step(iters, a[0], a[1], 0.1, visc, "_clamp")
        a[2], a[3] = oracle_mod.ref_advect_color_step(iters, a[2], a[3], a[0], 0.1, "_clamp")
        b[0], b[1], _ = oracle_mod.step(b[0], b[1], 0.1, visc, diffuse_iters=iters, max_iters=iters, boundary=1)
        b[2], b[3] = oracle_mod.advect_color_step(b[2], b[3], b[0], 0.1, boundary=1)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_oracle_walls_hold_zero_velocity_on_the_boundary(oracle_mod):
    vp, tmp, img, itmp = S.initial_state(36, 30, 3, seed=4)
    for _ in range(3):
        vp, tmp, _ = oracle_mod.step(vp, tmp, 0.1, 0.0, diffuse_iters=2, max_iters=40, boundary=2)
        img, itmp = oracle_mod.advect_color_step(img, itmp, vp, 0.1, boundary=2)
        for ch in (0, 1):
            u = vp[..., ch]
            assert not u[0].any() and not u[-1].any() and not u[:, 0].any() and not u[:, -1].any()
            assert u[1:-1, 1:-1].any()
    with pytest.raises(RuntimeError):
        oracle_mod.step(np.zeros((1, 5, 4), np.float32), np.zeros((1, 5, 4), np.float32), 0.1, 0.0,
                        diffuse_iters=1, max_iters=1, boundary=1)  # clamp needs sides >= 2
