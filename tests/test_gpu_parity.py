"""Parity of the CUDA path (called through the C ABI) with the reference.

Tolerance: the bar is max|x - y| / max|y| <= 1e-5 per field (FP32), but the
kernels reproduce the reference's per-operation rounding, so every check
here is exact equality (np.array_equal, which treats +0 and -0 as equal:
with viscosity 0 the reference's identity diffusion sweeps can flip the
sign of a zero, which the GPU path does not replay).
"""
import ctypes
import hashlib

import numpy as np
import pytest

from golden_util import c0_digests, cases, load
from probabilistic_fluid_simulation_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5  # the parity bar; exact equality is asserted below


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def assert_same(got, want, what=""):
    assert got.shape == want.shape, what
    if not np.array_equal(got, want):
        d = np.abs(got.astype(np.float64) - want).max()
        scale = max(np.abs(want).max(), 1e-30)
        raise AssertionError(f"{what}: max|d| = {d} (rel {d / scale}, bar {REL_TOL})")


# ---------------------------------------------------------------------------------------------
# Drop-in calls vs golden vectors from the reference's own src/fluid.cpp

@pytest.mark.parametrize("name", cases())
def test_dropin_device_matches_reference(cuda_device, pfs_lib, name):
    meta, arrays = load(name)
    pfs_lib.set_jacobi_iters(meta["iters"])
    try:
        vp, tmp = dev(arrays["in_vp"]), dev(arrays["in_tmp"])
        img, itmp = dev(arrays["in_img"]), dev(arrays["in_itmp"])
        vp_id, tmp_id = vp.data_ptr(), tmp.data_ptr()
        for s in range(1, meta["steps"] + 1):
            vp, tmp = pfs_lib.simulate_fluid_step(vp, tmp, meta["dt"], meta["viscosity"])
            # with equal diffusion / pressure counts the reference's swaps cancel out
            assert vp.data_ptr() == vp_id and tmp.data_ptr() == tmp_id
            img2, itmp2 = pfs_lib.advect_color_step(img, itmp, vp, meta["dt"])
            assert img2 is itmp and itmp2 is img  # src/fluid.cpp:317-319 swap
            img, itmp = img2, itmp2
            if s in meta["snaps"]:
                for k, t in (("vp", vp), ("tmp", tmp), ("img", img), ("itmp", itmp)):
                    assert_same(host(t), arrays[f"{k}_s{s}"], f"{name} step {s} {k}")
    finally:
        pfs_lib.set_jacobi_iters(30)


@pytest.mark.parametrize("name", ["vortex32x24_it40", "vortex20x14_it3_visc", "ones3x3_it30"])
def test_dropin_host_matches_reference(cuda_device, pfs_lib, name):
    meta, arrays = load(name)
    pfs_lib.set_jacobi_iters(meta["iters"])
    try:
        vp, tmp = arrays["in_vp"].copy(), arrays["in_tmp"].copy()
        img, itmp = arrays["in_img"].copy(), arrays["in_itmp"].copy()
        for s in range(1, meta["steps"] + 1):
            vp, tmp = pfs_lib.simulate_fluid_step(vp, tmp, meta["dt"], meta["viscosity"])
            img, itmp = pfs_lib.advect_color_step(img, itmp, vp, meta["dt"])
            if s in meta["snaps"]:
                for k, a in (("vp", vp), ("tmp", tmp), ("img", img), ("itmp", itmp)):
                    assert_same(a, arrays[f"{k}_s{s}"], f"{name} step {s} {k}")
    finally:
        pfs_lib.set_jacobi_iters(30)


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_c0_256_100_steps_session_digests(cuda_device, pfs_lib):
    """256x256, 40 sweeps, dt 0.1, 100 steps through a session: all buffers
    after steps 1 and 100 equal the reference's (SHA-256 of the bytes)."""
    rec = c0_digests()
    vp, tmp, img, itmp = S.initial_state(rec["w"], rec["h"], rec["channels"], rec["seed"])
    assert _digest(vp) == rec["input_digests"]["vp"]
    n = rec["iters"]
    with pfs_lib.Session(rec["w"], rec["h"], image_shape=img.shape, dt=rec["dt"], viscosity=rec["viscosity"],
                         diffuse_iters=n, max_iters=n) as s:
        s.upload(vp, tmp, img)
        done = 0
        for target in (1, rec["steps"]):
            s.step(target - done)
            done = target
            a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
            s.download(a, b, c)
            want = rec["digests"][str(target)]
            assert _digest(a) == want["vp"] and _digest(b) == want["tmp"] and _digest(c) == want["img"], target


def test_c0_256_100_steps_dropin_digests(cuda_device, pfs_lib):
    rec = c0_digests()
    vp, tmp, img, itmp = (dev(a) for a in S.initial_state(rec["w"], rec["h"], rec["channels"], rec["seed"]))
    pfs_lib.set_jacobi_iters(rec["iters"])
    try:
        for _ in range(rec["steps"]):
            vp, tmp = pfs_lib.simulate_fluid_step(vp, tmp, rec["dt"], rec["viscosity"])
            img, itmp = pfs_lib.advect_color_step(img, itmp, vp, rec["dt"])
    finally:
        pfs_lib.set_jacobi_iters(30)
    want = rec["digests"][str(rec["steps"])]
    got = {k: _digest(host(t)) for k, t in (("vp", vp), ("tmp", tmp), ("img", img), ("itmp", itmp))}
    assert got == want


# ---------------------------------------------------------------------------------------------
# Sessions vs the oracle (generalised counts, residual stop, sizes)

def oracle_run(O, vp, tmp, img, itmp, steps, dt, visc, D, S_, tol=0.0, check_every=0):
    stats = []
    for _ in range(steps):
        vp, tmp, st = O.step(vp, tmp, dt, visc, diffuse_iters=D, max_iters=S_, tol=tol, check_every=check_every)
        if img is not None:
            img, itmp = O.advect_color_step(img, itmp, vp, dt)
        stats.append(st)
    return vp, tmp, img, stats


SESSION_CASES = [
    # w, h, image (w, h, c) or None, D, S, visc, steps
    (64, 64, (64, 64, 3), 40, 40, 0.0, 3),
    (96, 40, (96, 40, 3), 3, 17, 0.0, 3),       # odd/even mixes: roles swap between steps
    (100, 36, (50, 72, 4), 2, 9, 0.05, 2),      # w % 4 == 0, image grid differs, viscosity
    (37, 29, (37, 29, 3), 5, 6, 0.02, 2),       # w % 4 != 0: single-sweep path
    (8, 4, None, 1, 1, 0.0, 3),
    (2, 2, (2, 2, 4), 30, 30, 0.0, 2),
    (260, 132, (260, 132, 3), 0, 25, 0.0, 2),   # no diffusion sweeps
    (256, 256, (256, 256, 3), 4, 0, 0.0, 2),    # no pressure sweeps
    (1024, 768, (1024, 768, 3), 2, 43, 0.0, 1),
]


@pytest.mark.parametrize("w,h,imgs,D,S_,visc,steps", SESSION_CASES)
def test_session_matches_oracle(cuda_device, pfs_lib, oracle_mod, w, h, imgs, D, S_, visc, steps):
    vp = S.vortex_field(w, h, seed=w + h)
    vp[..., 2] = 0.25 * S.vortex_field(w, h, seed=1)[..., 0]   # non-zero initial pressure in both buffers
    tmp = np.zeros_like(vp)
    tmp[..., 2] = -0.5 * vp[..., 1]
    img = S.blob_image(imgs[0], imgs[1], imgs[2], seed=4) if imgs else None
    itmp = np.zeros_like(img) if imgs else None
    ov, ot, oi, _ = oracle_run(oracle_mod, vp.copy(), tmp.copy(), None if img is None else img.copy(),
                               None if img is None else itmp.copy(), steps, 0.1, visc, D, S_)
    shape = (imgs[1], imgs[0], imgs[2]) if imgs else None
    with pfs_lib.Session(w, h, image_shape=shape, dt=0.1, viscosity=visc, diffuse_iters=D, max_iters=S_) as s:
        s.upload(vp, tmp, img)
        s.step(steps)
        a, b = np.empty_like(vp), np.empty_like(tmp)
        c = np.empty_like(img) if img is not None else None
        s.download(a, b, c)
        st = s.stats()
    assert st["steps"] == steps and st["sweeps"] == S_
    assert_same(a, ov, "vp")
    assert_same(b, ot, "tmp")
    if img is not None:
        assert_same(c, oi, "image")


@pytest.mark.parametrize("fuse", [1, 3, 8])
def test_session_residual_mode_matches_oracle(cuda_device, pfs_lib, oracle_mod, fuse):
    w, h = 64, 48
    vp, tmp, img, itmp = S.initial_state(w, h, 3, seed=21)
    tol, cap, every = 1e-4, 3000, 50  # converges in 950-1000 sweeps per step
    ov, ot, oi, ost = oracle_run(oracle_mod, vp.copy(), tmp.copy(), img.copy(), itmp.copy(), 3, 0.1, 0.0, 40,
                                 cap, tol=tol, check_every=every)
    with pfs_lib.Session(w, h, image_shape=img.shape, dt=0.1, diffuse_iters=40, max_iters=cap, tol=tol,
                         check_every=every, fuse_depth=fuse) as s:
        s.upload(vp, tmp, img)
        sweeps = []
        for _ in range(3):
            s.step(1)
            st = s.stats()
            sweeps.append(st["sweeps"])
            assert st["rel_residual"] == pytest.approx(ost[len(sweeps) - 1].rel_residual, rel=1e-9)
        a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
        s.download(a, b, c)
    assert sweeps == [x.sweeps for x in ost]
    assert all(x.sweeps < cap for x in ost)
    assert_same(a, ov, "vp")
    assert_same(b, ot, "tmp")
    assert_same(c, oi, "image")


def test_session_residual_cap_hits(cuda_device, pfs_lib, oracle_mod):
    w, h = 256, 256
    vp, tmp, img, itmp = S.initial_state(w, h, 3, seed=3)
    ov, ot, _, ost = oracle_run(oracle_mod, vp.copy(), tmp.copy(), None, None, 2, 0.05, 0.0, 40, 400,
                                tol=1e-9, check_every=100)
    with pfs_lib.Session(w, h, dt=0.05, diffuse_iters=40, max_iters=400, tol=1e-9, check_every=100) as s:
        s.upload(vp, tmp)
        s.step(2)
        st = s.stats()
        a, b = np.empty_like(vp), np.empty_like(tmp)
        s.download(a, b)
    assert st["cap_hits"] == 2 and st["capped"] == 1 and st["sweeps"] == 400 and st["checks"] == 4
    assert st["rel_residual"] == pytest.approx(ost[-1].rel_residual, rel=1e-9)
    assert_same(a, ov, "vp")
    assert_same(b, ot, "tmp")


def test_full_size_2048_one_step_to_residual(cuda_device, pfs_lib, oracle_mod):
    """The 2048x2048 workload (dt 0.05, residual 1e-5, cap 2000, checks every
    100 sweeps): one full step, every buffer bit-equal to the oracle."""
    w = h = 2048
    vp, tmp, img, itmp = S.initial_state(w, h, 3, seed=1)
    ov, ot, oi, ost = oracle_run(oracle_mod, vp.copy(), tmp.copy(), img.copy(), itmp.copy(), 1, 0.05, 0.0, 40,
                                 2000, tol=1e-5, check_every=100)
    with pfs_lib.Session(w, h, image_shape=img.shape, dt=0.05, diffuse_iters=40, max_iters=2000, tol=1e-5,
                         check_every=100) as s:
        s.upload(vp, tmp, img)
        s.step(1)
        st = s.stats()
        a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
        s.download(a, b, c)
    assert st["sweeps"] == ost[0].sweeps
    assert st["rel_residual"] == pytest.approx(ost[0].rel_residual, rel=1e-9)
    assert_same(a, ov, "vp")
    assert_same(b, ot, "tmp")
    assert_same(c, oi, "image")


# ---------------------------------------------------------------------------------------------
# Kernel-level: the fused (temporally blocked) sweep equals repeated single sweeps

# default chunk heights from 4 rows (1024x200, 128x128) to 18 (1536^2), 32 (2048^2) and 128 (4096^2)
@pytest.mark.parametrize("w,h", [(4096, 4096), (2048, 2048), (1536, 1536), (1024, 200), (260, 132), (128, 128),
                                 (64, 64), (12, 8), (4, 3)])
@pytest.mark.parametrize("levels", [1, 2, 5, 8])
def test_fused_sweeps_equal_single_sweeps(cuda_device, pfs_lib, w, h, levels):
    import torch
    g = torch.Generator(device="cpu").manual_seed(w * 31 + h + levels)
    ld = (w + 31) // 32 * 32
    p = torch.randn(h, ld, generator=g).cuda()
    b = torch.randn(h, ld, generator=g).cuda()
    out = torch.zeros_like(p)
    prev = torch.zeros_like(p)
    pfs_lib.pressure_sweeps(p, b, out, prev, levels, fused=True, w=w)
    ref_out = torch.zeros_like(p)
    ref_prev = torch.zeros_like(p)
    pfs_lib.pressure_sweeps(p, b, ref_out, ref_prev if levels > 1 else None, levels, fused=False, w=w)
    torch.cuda.synchronize()
    assert torch.equal(out[:, :w], ref_out[:, :w])
    if levels > 1:
        assert torch.equal(prev[:, :w], ref_prev[:, :w])
    else:
        assert torch.equal(prev[:, :w], p[:, :w])


@pytest.mark.parametrize("chunk", [4, 8, 9, 17, 18, 32, 64, 200])
def test_fused_sweep_chunking(cuda_device, pfs_lib, chunk):
    import torch
    g = torch.Generator(device="cpu").manual_seed(chunk)
    w, h = 512, 300
    p = torch.randn(h, w, generator=g).cuda()
    b = torch.randn(h, w, generator=g).cuda()
    out, prev = torch.zeros_like(p), torch.zeros_like(p)
    pfs_lib.pressure_sweeps(p, b, out, None, 8, fused=True, chunk_rows=chunk)
    pfs_lib.pressure_sweeps(p, b, prev, None, 8, fused=True, chunk_rows=32)
    torch.cuda.synchronize()
    assert torch.equal(out, prev)


def test_single_sweep_matches_oracle(cuda_device, pfs_lib, oracle_mod):
    import torch
    vp = S.vortex_field(40, 24, seed=8)
    vp[..., 2] = np.random.default_rng(0).standard_normal((24, 40)).astype(np.float32)
    vp[..., 3] = np.random.default_rng(1).standard_normal((24, 40)).astype(np.float32)
    out = np.zeros_like(vp)
    oracle_mod.pressure_sweep(vp, out)
    p = dev(vp[..., 2].copy())
    b = dev(vp[..., 3].copy())
    q = torch.zeros_like(p)
    pfs_lib.pressure_sweeps(p, b, q, None, 1, fused=False)
    assert_same(host(q), out[..., 2], "sweep")


def test_residual_norms_match_oracle(cuda_device, pfs_lib, oracle_mod):
    vp = np.zeros((96, 128, 4), np.float32)
    rng = np.random.default_rng(3)
    vp[..., 2] = rng.standard_normal((96, 128)).astype(np.float32)
    vp[..., 3] = rng.standard_normal((96, 128)).astype(np.float32)
    rel, bn = oracle_mod.residual(vp)
    rr, bb = pfs_lib.residual_norms(dev(vp[..., 2].copy()), dev(vp[..., 3].copy()))
    assert np.sqrt(bb) == pytest.approx(bn, rel=1e-12)
    assert np.sqrt(rr) / np.sqrt(bb) == pytest.approx(rel, rel=1e-12)


@pytest.mark.parametrize("static", [False, True])
def test_residual_norms_of_unaligned_views(cuda_device, pfs_lib, oracle_mod, static):
    # Views that start one float into their planes (4-byte, not 16-byte
    # aligned) with a width divisible by 4: the vector-load kernel must not be
    # chosen for them (its 16-byte loads would be misaligned); the host picks
    # the scalar kernel before any launch, and the norms are the oracle's.
    import torch
    w, h = 128, 40
    rng = np.random.default_rng(11)
    vp = np.zeros((h, w, 4), np.float32)
    vp[..., 2] = rng.standard_normal((h, w)).astype(np.float32)
    vp[..., 3] = rng.standard_normal((h, w)).astype(np.float32)
    rel, bn = oracle_mod.residual(vp)
    ld = 160
    pbase = torch.zeros(h, ld, device="cuda")
    bbase = torch.zeros(h, ld, device="cuda")
    pbase[:, 1:w + 1] = torch.from_numpy(vp[..., 2]).cuda()
    bbase[:, 1:w + 1] = torch.from_numpy(vp[..., 3]).cuda()
    pv, bv = pbase.data_ptr() + 4, bbase.data_ptr() + 4  # column 1 of each plane, row pitch ld
    assert pv % 16 == 4 and bv % 16 == 4
    lib = pfs_lib.lib()
    fn = lib.pfs_residual_norms_static if static else lib.pfs_residual_norms
    rrc, bbc = ctypes.c_double(), ctypes.c_double()
    st = fn(ctypes.c_void_p(pv), ctypes.c_void_p(bv), w, h, ld, ctypes.byref(rrc), ctypes.byref(bbc), None)
    assert st == 0, lib.pfs_last_error()
    rr, bb = rrc.value, bbc.value
    assert np.sqrt(bb) == pytest.approx(bn, rel=1e-12)
    assert np.sqrt(rr) / np.sqrt(bb) == pytest.approx(rel, rel=1e-12)


def test_dropin_rejects_bad_input_on_gpu(cuda_device, pfs_lib):
    import torch
    vp = torch.zeros(8, 8, 4, device="cuda")
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.simulate_fluid_step(vp, vp, 0.1, 0.0)
    img = torch.zeros(8, 8, 3, device="cuda")
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.advect_color_step(img, img, vp, 0.1)


# The last fused launch of each check interval evaluates the residual itself
# (launch_sweep_stream_check). Check intervals that are multiples of 8 split
# their last 8-level launch in two (64); chunks of 32 and 8 rows give the check
# launch different geometries. Each must give the oracle's sweeps, residuals
# and bits.
@pytest.mark.parametrize("every", [64, 100, 24])
def test_fused_check_matches_separate_residual_and_oracle(cuda_device, pfs_lib, oracle_mod, every):
    w, h = 256, 192
    vp, tmp, img, itmp = S.initial_state(w, h, 3, seed=31)
    tol, cap = 3e-3, 6000  # converges in 3984-4700 sweeps per step
    ov, ot, oi, ost = oracle_run(oracle_mod, vp.copy(), tmp.copy(), img.copy(), itmp.copy(), 2, 0.1, 0.0, 40,
                                 cap, tol=tol, check_every=every)
    runs = []
    for chunk in (32, 8):
        with pfs_lib.Session(w, h, image_shape=img.shape, dt=0.1, diffuse_iters=40, max_iters=cap, tol=tol,
                             check_every=every, chunk_rows=chunk) as s:
            s.upload(vp, tmp, img)
            stats = []
            for _ in range(2):
                s.step(1)
                stats.append(s.stats())
            a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
            s.download(a, b, c)
        runs.append((stats, a, b, c))
    for stats, a, b, c in runs:
        assert [x["sweeps"] for x in stats] == [x.sweeps for x in ost]
        assert [x["checks"] for x in stats] == [x.sweeps // every + (x.sweeps % every != 0) for x in ost]
        for x, o in zip(stats, ost):
            assert x["rel_residual"] == pytest.approx(o.rel_residual, rel=1e-9)
        assert_same(a, ov, "vp")
        assert_same(b, ot, "tmp")
        assert_same(c, oi, "image")
    assert all(x.sweeps < cap for x in ost)


def test_fused_check_on_a_large_grid(cuda_device, pfs_lib):
    """4096x4096, checks every 16 sweeps, cap 48: with 32-row chunks the check
    launch has 1184 blocks (more than the 608 of the separate residual
    kernel); with 8-row chunks it would need more partials than the field
    holds, so the separate residual kernel runs. Both give the same bits and
    residuals."""
    w = h = 4096
    vp, tmp, img, _ = S.initial_state(w, h, 3, seed=2)
    out = []
    for chunk in (32, 8):
        with pfs_lib.Session(w, h, dt=0.05, diffuse_iters=2, max_iters=48, tol=1e-12, check_every=16,
                             chunk_rows=chunk) as s:
            s.upload(vp, tmp)
            s.step(1)
            st = s.stats()
            a = np.empty_like(vp)
            s.download(a)
        out.append((st, a))
    (s1, a1), (s2, a2) = out
    assert s1["sweeps"] == s2["sweeps"] == 48 and s1["checks"] == s2["checks"] == 3 and s1["capped"]
    assert s1["rel_residual"] == pytest.approx(s2["rel_residual"], rel=1e-12)
    assert np.array_equal(a1, a2)


@pytest.mark.parametrize("w,h", [(8, 2), (4, 3), (12, 1), (16, 5)])
@pytest.mark.parametrize("every", [3, 8])
def test_fused_check_tiny_grids(cuda_device, pfs_lib, oracle_mod, w, h, every):
    """Grids of 1-5 rows: the check launch's extra halo rows wrap around the
    grid several times; intervals of 3 (3-level check launches) and 8 (split
    4 + 4). Sweeps, residuals and every buffer as the oracle."""
    vp, tmp, _, _ = S.initial_state(w, h, 3, seed=5)
    ov, ot, _, ost = oracle_run(oracle_mod, vp.copy(), tmp.copy(), None, None, 2, 0.1, 0.0, 4, 200, tol=1e-3,
                                check_every=every)
    with pfs_lib.Session(w, h, dt=0.1, diffuse_iters=4, max_iters=200, tol=1e-3, check_every=every) as s:
        s.upload(vp, tmp)
        stats = []
        for _ in range(2):
            s.step(1)
            stats.append(s.stats())
        a, b = np.empty_like(vp), np.empty_like(tmp)
        s.download(a, b)
    assert [x["sweeps"] for x in stats] == [x.sweeps for x in ost]
    for x, o in zip(stats, ost):
        assert x["rel_residual"] == pytest.approx(o.rel_residual, rel=1e-9)
    assert_same(a, ov, "vp")
    assert_same(b, ot, "tmp")


def test_capped_step_then_converging_step(cuda_device, pfs_lib, oracle_mod):
    """After a step that runs to the cap (8 checks) the next solve enqueues 8
    check intervals before reading the state, then 16 more; it converges at
    the 10th, the 14 intervals after it return at once, and the step still
    ends at the oracle's sweep count with its buffers; the step after a
    converged one starts from a batch of 1 again."""
    w, h = 64, 48
    vp, tmp, img, itmp = S.initial_state(w, h, 3, seed=21)
    tol, every = 1e-4, 100
    v1, t1, i1, s1 = oracle_run(oracle_mod, vp.copy(), tmp.copy(), img.copy(), itmp.copy(), 1, 0.1, 0.0, 40, 800,
                                tol=tol, check_every=every)
    v2, t2, i2, s2 = oracle_run(oracle_mod, v1, t1, i1, np.zeros_like(img), 2, 0.1, 0.0, 40, 3000, tol=tol,
                                check_every=every)
    assert s1[0].sweeps == 800 and all(800 < x.sweeps < 3000 for x in s2)
    with pfs_lib.Session(w, h, image_shape=img.shape, dt=0.1, diffuse_iters=40, max_iters=800, tol=tol,
                         check_every=every) as s:
        s.upload(vp, tmp, img)
        s.step(1)
        assert s.stats()["capped"] == 1
        s.set_params(max_iters=3000)
        got = []
        for _ in range(2):
            s.step(1)
            got.append(s.stats())
        a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
        s.download(a, b, c)
    assert [x["sweeps"] for x in got] == [x.sweeps for x in s2]
    for x, o in zip(got, s2):
        assert x["rel_residual"] == pytest.approx(o.rel_residual, rel=1e-9) and not x["capped"]
    assert_same(a, v2, "vp")
    assert_same(b, t2, "tmp")
    assert_same(c, i2, "image")
