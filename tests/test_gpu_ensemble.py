"""Batched form: members of an ensemble (one persistent cooperative kernel per
timestep for all of them) against plain sessions with the same parameters,
bit for bit."""
import numpy as np
import pytest

from probabilistic_fluid_simulation_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (128, 64), (64, 256), (256, 128), (96, 40), (128, 128), (192, 96), (64, 128), (256, 256),
         (32, 48), (8, 8), (520, 64)]


def member_state(w, h, k):
    base = S.draw_vortices(256, 256, seed=99)
    vort = [S.Vortex(v.cx * w / 256, v.cy * h / 256, v.radius * (w * h) ** 0.5 / 256, v.circulation)
            for v in S.perturb_vortices(base, seed=99, member=k)]
    vp = S.velocity_from_vortices(w, h, vort)
    tmp = np.zeros_like(vp)
    img = S.blob_image(w, h, 3, seed=k)
    return vp, tmp, img


def session_run(pfs_lib, vp, tmp, img, steps, **kw):
    h, w, _ = vp.shape
    with pfs_lib.Session(w, h, image_shape=img.shape, **kw) as s:
        s.upload(vp, tmp, img)
        stats = []
        for _ in range(steps):
            s.step(1)
            stats.append(s.stats())
        a, b, c = np.empty_like(vp), np.empty_like(vp), np.empty_like(img)
        s.download(a, b, c)
    return a, b, c, stats


@pytest.mark.parametrize("fuse,chunk,tol,every,cap", [(8, 32, 0.0, 0, 96), (8, 24, 1e-3, 32, 2400),
                                                      (4, 16, 1e-3, 48, 2400)])
def test_ensemble_members_equal_sessions(cuda_device, pfs_lib, fuse, chunk, tol, every, cap):
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=cap, tol=tol, check_every=every, fuse_depth=fuse, chunk_rows=chunk)
    states = [member_state(w, h, k) for k, (w, h) in enumerate(SIZES)]
    steps = 3
    with pfs_lib.Ensemble(SIZES, 3, **kw) as ens:
        for k, (vp, tmp, img) in enumerate(states):
            ens.upload(k, vp, tmp, img)
        per_step = []
        for _ in range(steps):
            ens.step(1)
            per_step.append([ens.stats(k) for k in range(len(SIZES))])
        info = ens.info()
        outs = []
        for k, (vp, tmp, img) in enumerate(states):
            a, c = np.empty_like(vp), np.empty_like(img)
            ens.download(k, a, c)
            outs.append((a, c))
    print("ensemble info", info)
    assert info["fuse_depth"] == fuse and info["chunk_rows"] == chunk
    sweeps_seen = set()
    for k, (vp, tmp, img) in enumerate(states):
        sa, sb, sc, sst = session_run(pfs_lib, vp, tmp, img, steps, **kw)
        a, c = outs[k]
        assert np.array_equal(a[..., 0:2], sa[..., 0:2]), (k, SIZES[k])
        assert np.array_equal(a[..., 2], sb[..., 2]), (k, SIZES[k])  # final pressure
        assert np.array_equal(a[..., 3], sa[..., 3]), (k, SIZES[k])
        assert np.array_equal(c, sc), (k, SIZES[k])
        for step in range(steps):
            e, s = per_step[step][k], sst[step]
            assert e["sweeps"] == s["sweeps"], (k, step, e, s)
            assert e["capped"] == s["capped"]
            if tol > 0:
                assert e["rel_residual"] == pytest.approx(s["rel_residual"], rel=1e-9)
            sweeps_seen.add(e["sweeps"])
    if tol > 0:
        assert len(sweeps_seen) > 2  # members converge at different sweep counts


def test_ensemble_autotuner_keeps_results(cuda_device, pfs_lib):
    from probabilistic_fluid_simulation_gb300 import tune
    sizes = SIZES[:6]
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=96, tol=0.0, check_every=0)
    states = [member_state(w, h, k) for k, (w, h) in enumerate(sizes)]
    with pfs_lib.Ensemble(sizes, 3, **kw) as ens:
        for k, st in enumerate(states):
            ens.upload(k, *st)
        best, timings = tune.tune_ensemble(ens, steps=1)
        assert len(timings) >= 4 and best in timings
        ens.step(2)
        a, c = np.empty_like(states[3][0]), np.empty_like(states[3][2])
        ens.download(3, a, c)
    sa, sb, sc, _ = session_run(pfs_lib, *states[3], 2, **kw)
    assert np.array_equal(a[..., 0:2], sa[..., 0:2]) and np.array_equal(c, sc)


def test_ensemble_rejects_unsupported(cuda_device, pfs_lib):
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.Ensemble([(64, 64)], 3, dt=0.1, diffuse_iters=2, max_iters=100)  # cap not a multiple of 8
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.Ensemble([(66, 64)], 3, dt=0.1, diffuse_iters=2, max_iters=96)  # width not a multiple of 4


def test_ensemble_image_statistics_match_sessions(cuda_device, pfs_lib):
    """Pointwise mean and population variance of the image over the members of
    one grid size, against the same members run as plain sessions (whose
    images equal the members' bit for bit) reduced with numpy in float64."""
    sizes = [(128, 96)] * 6 + [(64, 64), (128, 96), (96, 128)]
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=64, tol=1e-3, check_every=32)
    states = [member_state(w, h, k) for k, (w, h) in enumerate(sizes)]
    group = [k for k, s in enumerate(sizes) if s == (128, 96)]
    with pfs_lib.Ensemble(sizes, 3, **kw) as ens:
        for k, st in enumerate(states):
            ens.upload(k, *st)
        ens.step(3)
        mean, var = ens.image_stats(group)
        with pytest.raises(pfs_lib.PFSError):
            ens.image_stats([0, 6])  # different grid sizes
        sub_mean, _ = ens.image_stats(group[:1])
    imgs = np.stack([session_run(pfs_lib, *states[k], 3, **kw)[2] for k in group]).astype(np.float64)
    ref_mean, ref_var = imgs.mean(axis=0), imgs.var(axis=0)
    assert mean.shape == (96, 128, 3)
    assert np.abs(mean - ref_mean).max() <= 1e-6 * max(1.0, np.abs(ref_mean).max())
    assert np.abs(var - ref_var).max() <= 1e-6 * max(ref_var.max(), 1e-12) + 1e-9
    assert np.array_equal(sub_mean, imgs[0].astype(np.float32))
    assert var.max() > 0.0


def test_grid_barrier_timeout_is_reported(cuda_device, pfs_lib):
    """Failure detection without a GPU fault: one block of the step kernel
    leaves before the first grid barrier, the others' bounded wait runs out
    (~1-2 s), every block returns, and the step reports PFS_ERR_DEVICE_TIMEOUT.
    The failed ensemble stays failed; the device stays usable."""
    import time
    sizes = [(64, 64), (96, 40)]
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=64, tol=1e-3, check_every=32)
    states = [member_state(w, h, k) for k, (w, h) in enumerate(sizes)]
    with pfs_lib.Ensemble(sizes, 3, **kw) as ens:
        for k, st in enumerate(states):
            ens.upload(k, *st)
        ens.step(1)  # a normal step first (graphs built)
        ens.debug_stall_block(0)
        t0 = time.time()
        with pytest.raises(pfs_lib.PFSError) as ei:
            ens.step(1)
        assert ei.value.status == 6  # PFS_ERR_DEVICE_TIMEOUT
        assert time.time() - t0 < 60
        with pytest.raises(pfs_lib.PFSError):
            ens.step(1)  # sticky
    # the device is fine: a new ensemble steps and matches a session
    with pfs_lib.Ensemble(sizes, 3, **kw) as ens:
        for k, st in enumerate(states):
            ens.upload(k, *st)
        ens.step(2)
        a, c = np.empty_like(states[1][0]), np.empty_like(states[1][2])
        ens.download(1, a, c)
    ref = session_run(pfs_lib, *states[1], 2, **kw)
    assert np.array_equal(a[..., :2], ref[0][..., :2]) and np.array_equal(c, ref[2])


def test_ensemble_64_members_up_to_1024_equal_sessions(cuda_device, pfs_lib):
    """64 members with sides drawn from {64, 128, 256, 512, 1024} (w and h
    independently, as the ensemble workload draws them), residual stop, the
    default tile: every member bit-equal to a plain session."""
    rng = np.random.default_rng(2024)
    sides = (64, 128, 256, 512, 1024)
    sizes = [(int(sides[rng.integers(5)]), int(sides[rng.integers(5)])) for _ in range(64)]
    assert max(max(s) for s in sizes) == 1024
    kw = dict(dt=0.05, diffuse_iters=2, max_iters=400, tol=2e-2, check_every=40)
    states = [member_state(w, h, k) for k, (w, h) in enumerate(sizes)]
    with pfs_lib.Ensemble(sizes, 3, **kw) as ens:
        for k, (vp, tmp, img) in enumerate(states):
            ens.upload(k, vp, tmp, img)
        ens.step(2)
        stats = [ens.stats(k) for k in range(len(sizes))]
        outs = []
        for k, (vp, tmp, img) in enumerate(states):
            a, c = np.empty_like(vp), np.empty_like(img)
            ens.download(k, a, c)
            outs.append((a, c))
    for k, (vp, tmp, img) in enumerate(states):
        sa, sb, sc, sst = session_run(pfs_lib, vp, tmp, img, 2, **kw)
        a, c = outs[k]
        assert np.array_equal(a[..., 0:2], sa[..., 0:2]), (k, sizes[k])
        assert np.array_equal(a[..., 2], sb[..., 2]), (k, sizes[k])
        assert np.array_equal(c, sc), (k, sizes[k])
        assert stats[k]["sweeps"] == sst[-1]["sweeps"], (k, stats[k], sst[-1])
    assert len({s["sweeps"] for s in stats}) >= 2  # members stop at different check points


def test_refined_ensemble_members_match_refined_sessions(cuda_device, pfs_lib):
    """PFS_PREC_F32R members (float32 sweeps on a correction, FP64 pressure and
    refinement) reach the tolerance the float32 form cannot, and match
    PFS_PREC_F32R sessions: the same sweeps per step (the same check points,
    refinement intervals and decisions), and fields within 1e-5 of the
    session's (the ensemble does not scale the correction's right-hand side,
    so its float32 rounding differs)."""
    sizes = [(64, 64), (128, 64), (64, 128), (128, 128), (96, 40), (256, 128)]
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=200_000, tol=1e-5, check_every=200, precision=pfs_lib.PREC_F32R)
    states = [member_state(w, h, k) for k, (w, h) in enumerate(sizes)]
    steps = 2
    with pfs_lib.Ensemble(sizes, 3, **kw) as ens:
        for k, (vp, tmp, img) in enumerate(states):
            ens.upload(k, vp, tmp, img)
        per_step = []
        for _ in range(steps):
            ens.step(1)
            per_step.append([ens.stats(k) for k in range(len(sizes))])
        outs = []
        for k, (vp, tmp, img) in enumerate(states):
            a, c = np.empty_like(vp), np.empty_like(img)
            ens.download(k, a, c)
            outs.append((a, c))
    for k, (vp, tmp, img) in enumerate(states):
        h, w, _ = vp.shape
        with pfs_lib.Session(w, h, image_shape=img.shape, **kw) as s:
            s.upload(vp, tmp, img)
            sst = []
            for _ in range(steps):
                s.step(1)
                sst.append(s.stats())
            sa, sc = np.empty_like(vp), np.empty_like(img)
            s.download(sa, None, sc)
        a, c = outs[k]
        for step in range(steps):
            e, q = per_step[step][k], sst[step]
            assert e["rel_residual"] <= 1e-5 and not e["capped"] and not e["stalled"], (k, step, e)
            assert abs(e["sweeps"] - q["sweeps"]) <= 200, (k, step, e, q)
        for ch in (0, 1):
            d = np.abs(a[..., ch] - sa[..., ch]).max() / np.abs(sa[..., ch]).max()
            assert d < 1e-5, (k, ch, d)
        assert np.abs(c - sc).max() < 1e-5, k
