"""Session upload / download with host buffers: pinned (page-locked, also at
an offset that breaks 16-byte alignment) and pageable buffers give the same
bits."""
import numpy as np
import pytest

from probabilistic_fluid_simulation_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def pinned_like(a, offset_floats=0):
    import torch
    buf = torch.empty(a.size + offset_floats, dtype=torch.float32).pin_memory().numpy()
    view = buf[offset_floats:offset_floats + a.size].reshape(a.shape)
    view[...] = a
    return view


@pytest.mark.parametrize("offset", [0, 1])
def test_pinned_host_io_matches_pageable(cuda_device, pfs_lib, offset):
    vp, tmp, img, _ = S.initial_state(96, 64, 3, seed=13)
    tmp[..., 2] = 0.5 * vp[..., 0]
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=300, tol=1e-4, check_every=50)
    outs = []
    for pinned in (False, True):
        with pfs_lib.Session(96, 64, image_shape=img.shape, **kw) as s:
            if pinned:
                s.upload(pinned_like(vp, offset), pinned_like(tmp, offset), pinned_like(img, offset))
            else:
                s.upload(vp, tmp, img)
            s.step(3)
            if pinned:
                a, b, c = (pinned_like(np.zeros_like(x), offset) for x in (vp, tmp, img))
            else:
                a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
            s.download(a, b, c)
            outs.append((a.copy(), b.copy(), c.copy()))
    for x, y in zip(*outs):
        assert np.array_equal(x, y)


def _states(w, h, n, seed):
    out = []
    for k in range(n):
        vp, tmp, img, _ = S.initial_state(w, h, 3, seed=seed + k)
        tmp[..., 2] = 0.25 * vp[..., 1]
        out.append((vp, tmp, img))
    return out


@pytest.mark.parametrize("precision", ["f32", "bf16"])
def test_async_stream_of_states_matches_sync(cuda_device, pfs_lib, precision):
    """A stream of independent states through upload_async / step /
    download_async, the next upload queued before each step (the copies then
    overlap the steps), gives for each state the bits of upload / step /
    download."""
    w, h = 128, 96
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=300, tol=1e-4, check_every=50,
              precision=pfs_lib.PRECISIONS[precision])
    states = _states(w, h, 5, seed=40)
    pinned = [tuple(pinned_like(x) for x in st) for st in states]
    want = []
    with pfs_lib.Session(w, h, image_shape=states[0][2].shape, **kw) as s:
        for vp, tmp, img in states:
            s.upload(vp, tmp, img)
            s.step(2)
            a, b, c = np.empty_like(vp), np.empty_like(tmp), np.empty_like(img)
            s.download(a, b, c)
            want.append((a, b, c))
    got = [tuple(pinned_like(np.zeros_like(x)) for x in st) for st in states]
    with pfs_lib.Session(w, h, image_shape=states[0][2].shape, **kw) as s:
        s.upload_async(*pinned[0])
        for k in range(len(states)):
            if k + 1 < len(states):
                s.upload_async(*pinned[k + 1])
            s.step(2)
            s.download_async(*got[k])
        s.sync()
    for k in range(len(states)):
        for x, y in zip(got[k], want[k]):
            assert np.array_equal(x, y), k


def test_async_download_snapshots_a_running_simulation(cuda_device, pfs_lib):
    """Snapshots of a simulation that keeps its own state (no uploads): each
    download_async holds the state after the steps queued before it, while
    later steps are already queued; more downloads than slots reuse them."""
    w, h = 96, 64
    kw = dict(dt=0.1, diffuse_iters=2, max_iters=40)
    vp, tmp, img = _states(w, h, 1, seed=7)[0]
    want = []
    with pfs_lib.Session(w, h, image_shape=img.shape, **kw) as s:
        s.upload(vp, tmp, img)
        for _ in range(4):
            s.step(1)
            a, c = np.empty_like(vp), np.empty_like(img)
            s.download(a, None, c)
            want.append((a, c))
    got = [(pinned_like(np.zeros_like(vp)), pinned_like(np.zeros_like(img))) for _ in range(4)]
    with pfs_lib.Session(w, h, image_shape=img.shape, **kw) as s:
        s.upload(vp, tmp, img)
        for k in range(4):
            s.step(1)
            s.download_async(got[k][0], None, got[k][1])
        s.wait_io()
        s.sync()
    for (a, c), (x, y) in zip(want, got):
        assert np.array_equal(a, x) and np.array_equal(c, y)


def test_async_queue_rules(cuda_device, pfs_lib):
    w, h = 64, 64
    vp, tmp, img = _states(w, h, 1, seed=3)[0]
    with pfs_lib.Session(w, h, image_shape=img.shape, dt=0.1) as s:
        s.upload_async(vp, tmp, img)
        s.upload_async(vp, tmp, img)
        with pytest.raises(pfs_lib.PFSError):
            s.upload_async(vp, tmp, img)  # two slots
        with pytest.raises(pfs_lib.PFSError):
            s.upload(vp, tmp, img)  # a queued upload would replace it at the next step
        with pytest.raises(ValueError):
            s.download_async(np.empty(5, np.float32))
        s.step(1)
        s.step(1)
        s.upload(vp, tmp, img)  # queue empty again
        s.sync()
