"""The warm-start network's GPU kernels against the FP64 CPU reference
(oracle/unet_ref.py): forward loss, every parameter gradient, and training.

Tolerances: the GPU stores activations in bf16 (8 significant bits), so
values agree to about 1e-2 relative; gradients per layer are compared by
relative L2 error and by direction (cosine)."""
import numpy as np
import pytest

from oracle import unet_ref as R

pytestmark = pytest.mark.gpu


def smooth_batch(n, h, w, seed):
    rng = np.random.default_rng(seed)
    b = rng.standard_normal((n, h, w))
    # low-pass so the pairs resemble divergence fields
    k = np.fft.fftfreq(h)[:, None] ** 2 + np.fft.fftfreq(w)[None, :] ** 2
    b = np.real(np.fft.ifft2(np.fft.fft2(b) * np.exp(-k * 400.0)))
    b /= np.sqrt((b ** 2).mean(axis=(1, 2), keepdims=True))
    p = R.poisson_solution(b)
    return b.astype(np.float32), p.astype(np.float32)


def layer_slices():
    out, off = [], 0
    for ci, co in R.CONVS:
        n = co * 9 * R.cinp(ci)
        out.append((f"conv{len(out)}.w", slice(off, off + n)))
        off += n
        out.append((f"conv{len(out) - 1}.b", slice(off, off + co)))
        off += co
    out.append(("head.w", slice(off, off + 16)))
    out.append(("head.b", slice(off + 16, off + 17)))
    return out


def test_unet_param_count(pfs_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    net = pfs_lib.UNet(2 * 128 * 128)
    assert net.n_params == R.n_params()


def test_unet_forward_and_gradients_match_fp64_reference(cuda_device, pfs_lib):
    import torch
    params = R.init_params(seed=3)
    b, p = smooth_batch(2, 128, 128, seed=1)
    net = pfs_lib.UNet(2 * 128 * 128)
    net.set_params(params)
    loss = net.forward_backward(torch.from_numpy(b).cuda(), torch.from_numpy(p).cuda())
    g = net.grads()
    ref_loss, ref_g, _ = R.loss_and_grads(params, b, p)
    assert loss == pytest.approx(ref_loss, rel=2e-2)
    worst = []
    for name, sl in layer_slices():
        gg, rg = g[sl].astype(np.float64), ref_g[sl]
        rn = np.linalg.norm(rg)
        rel = np.linalg.norm(gg - rg) / max(rn, 1e-30)
        cos = float(gg @ rg / max(np.linalg.norm(gg) * rn, 1e-30))
        worst.append((rel, cos, name))
        assert rel < 6e-2 and cos > 0.998, (name, rel, cos)
    print("worst gradient errors", sorted(worst)[-3:])


def test_unet_prediction_matches_reference(cuda_device, pfs_lib):
    import torch
    params = R.init_params(seed=4)
    b, _ = smooth_batch(1, 128, 256, seed=2)
    net = pfs_lib.UNet(128 * 256)
    net.set_params(params)
    out = torch.empty(128, 256, device="cuda")
    scale = 3.5
    net.predict(torch.from_numpy(b[0] * scale).cuda(), out)
    layers, head = R.unpack(params)
    ref = R.forward(layers, head, torch.from_numpy(b.astype(np.float64))[:, None]).detach().numpy()[0] * scale
    err = np.abs(out.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 3e-2, err


def test_unet_training_reduces_loss(cuda_device, pfs_lib):
    import torch
    b, p = smooth_batch(8, 128, 128, seed=5)
    net = pfs_lib.UNet(8 * 128 * 128)
    net.set_params(R.init_params(seed=6))
    bt, pt = torch.from_numpy(b).cuda(), torch.from_numpy(p).cuda()
    first = net.forward_backward(bt, pt)
    for _ in range(150):
        net.forward_backward(bt, pt)
        net.adam_step(1e-3)
    last = net.forward_backward(bt, pt)
    assert last < 0.2 * first, (first, last)


def test_unet_trains_on_wide_grids(cuda_device, pfs_lib):
    """The weight gradient streams row segments of at most 128 pixels, so
    training takes any width (here 1024) and gives finite gradients."""
    import torch
    net = pfs_lib.UNet(128 * 1024)
    rng = np.random.default_rng(1)
    net.set_params((rng.standard_normal(net.n_params) * 0.05).astype(np.float32))
    b, p = smooth_batch(1, 128, 1024, seed=3)
    loss = net.forward_backward(torch.from_numpy(b).cuda(), torch.from_numpy(p).cuda())
    g = net.grads()
    assert np.isfinite(loss) and loss > 0 and np.isfinite(g).all() and np.abs(g).max() > 0
