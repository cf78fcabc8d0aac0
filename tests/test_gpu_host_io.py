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
