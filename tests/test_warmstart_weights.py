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
