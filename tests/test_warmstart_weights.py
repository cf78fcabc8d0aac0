"""The shipped warm-start weights: layout and training record (no GPU)."""
import numpy as np

from oracle import unet_ref as R
from probabilistic_fluid_simulation_gb300 import warmstart as WS


def test_shipped_weights_layout_and_record():
    params, meta = WS.load_default()
    n = sum(co * 9 * R.cinp(ci) + co for ci, co in R.CONVS) + 17
    assert params.dtype == np.float32 and params.shape == (n,)
    assert np.isfinite(params).all()
    assert meta["pairs"] == 40000 and meta["size"] == 256
    assert meta["training"]["val_loss"][-1] < 0.01
    assert WS.init_params(n).shape == params.shape


def test_starts_parser():
    assert WS._starts("1x2,4x1") == ((1, 2), (4, 1))


def test_augmentation_keeps_pairs_solutions():
    """Every augmented (b, p) pair still satisfies the pressure equation
    4p - (pL + pR + pT + pB) = b on the periodic grid (the symmetries commute
    with the operator): checked for many draws on pairs made exact by
    construction (b = A p for a random p)."""
    import numpy as np
    import torch

    from probabilistic_fluid_simulation_gb300 import warmstart as W

    def apply_a(p):
        return 4 * p - (torch.roll(p, 1, -1) + torch.roll(p, -1, -1) + torch.roll(p, 1, -2) + torch.roll(p, -1, -2))

    g = torch.Generator().manual_seed(3)
    for h, w in ((16, 16), (12, 20)):
        p = torch.randn(4, h, w, generator=g, dtype=torch.float64)
        b = apply_a(p)
        for _ in range(24):
            bb, pp = W.augment(b, p, g)
            assert bb.shape == b.shape and pp.shape == p.shape
            assert torch.allclose(apply_a(pp), bb, atol=1e-12)
        # the draws include non-trivial transforms
        assert not np.allclose(W.augment(b, p, torch.Generator().manual_seed(7))[0].numpy(), b.numpy())
