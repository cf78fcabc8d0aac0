"""FP64 CPU reference of the warm-start U-Net (the network of
probabilistic_fluid_simulation_gb300/csrc/unet.cu), written with torch on the
CPU in float64 with autograd.

TEST INFRASTRUCTURE ONLY: used by tests/ to check the GPU network's forward
pass and gradients. The product never imports it.

Parameter layout (flat float32 vector, as the library's): for each of the 14
3x3 convolutions w[cout][9][cinp] (tap = 3*ky + kx, cinp = max(cin, 16),
channels beyond cin are zero) then b[cout]; then the 1x1 head w[16], b[1].
"""
import numpy as np
import torch
import torch.nn.functional as F

CONVS = [(1, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 64), (64, 64), (128, 64), (64, 64),
         (96, 32), (32, 32), (48, 16), (16, 16)]


def cinp(c):
    return max(c, 16)


def n_params():
    return sum(co * 9 * cinp(ci) + co for ci, co in CONVS) + 17


def unpack(params, bf16_weights=True):
    """Flat vector -> list of (w [cout, cin, 3, 3] float64 tensor, b [cout]) and (head_w, head_b)."""
    p = np.asarray(params, np.float32)
    out, off = [], 0
    for ci, co in CONVS:
        cp = cinp(ci)
        w = p[off:off + co * 9 * cp].reshape(co, 9, cp)[:, :, :ci]
        off += co * 9 * cp
        b = p[off:off + co]
        off += co
        wt = torch.from_numpy(np.ascontiguousarray(w))
        if bf16_weights:
            wt = wt.to(torch.bfloat16)
        wt = wt.to(torch.float64).reshape(co, 3, 3, ci).permute(0, 3, 1, 2).contiguous()
        out.append((wt.requires_grad_(True), torch.from_numpy(b.astype(np.float64)).requires_grad_(True)))
    hw = torch.from_numpy(p[off:off + 16].astype(np.float64)).requires_grad_(True)
    hb = torch.from_numpy(p[off + 16:off + 17].astype(np.float64)).requires_grad_(True)
    return out, (hw, hb)


def conv(x, wb):
    w, b = wb
    return F.relu(F.conv2d(F.pad(x, (1, 1, 1, 1), mode="circular"), w, b))


def forward(layers, head, x):
    """x: (n, 1, h, w) float64 -> (n, h, w)."""
    e1 = conv(conv(x, layers[0]), layers[1])
    e2 = conv(conv(F.avg_pool2d(e1, 2), layers[2]), layers[3])
    e3 = conv(conv(F.avg_pool2d(e2, 2), layers[4]), layers[5])
    e4 = conv(conv(F.avg_pool2d(e3, 2), layers[6]), layers[7])
    d3 = conv(conv(torch.cat([F.interpolate(e4, scale_factor=2, mode="nearest"), e3], 1), layers[8]), layers[9])
    d2 = conv(conv(torch.cat([F.interpolate(d3, scale_factor=2, mode="nearest"), e2], 1), layers[10]), layers[11])
    d1 = conv(conv(torch.cat([F.interpolate(d2, scale_factor=2, mode="nearest"), e1], 1), layers[12]), layers[13])
    hw, hb = head
    return torch.einsum("nchw,c->nhw", d1, hw) + hb


def loss_and_grads(params, b, p):
    """MSE loss and gradients in the flat layout (float64 numpy)."""
    layers, head = unpack(params)
    x = torch.from_numpy(np.asarray(b, np.float64))[:, None]
    y = forward(layers, head, x)
    loss = ((y - torch.from_numpy(np.asarray(p, np.float64))) ** 2).mean()
    loss.backward()
    g = []
    for (ci, co), (w, bb) in zip(CONVS, layers):
        gw = np.zeros((co, 9, cinp(ci)))
        gw[:, :, :ci] = w.grad.permute(0, 2, 3, 1).reshape(co, 9, ci).numpy()
        g += [gw.ravel(), bb.grad.numpy()]
    g += [head[0].grad.numpy(), head[1].grad.numpy()]
    return float(loss.detach()), np.concatenate(g), y.detach().numpy()


def init_params(seed=0):
    """He-normal convolution weights, zero biases (padding channels zero)."""
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co in CONVS:
        w = np.zeros((co, 9, cinp(ci)), np.float32)
        w[:, :, :ci] = rng.standard_normal((co, 9, ci)) * np.sqrt(2.0 / (9 * ci))
        parts += [w.ravel(), np.zeros(co, np.float32)]
    parts += [(rng.standard_normal(16) * np.sqrt(1.0 / 16)).astype(np.float32), np.zeros(1, np.float32)]
    return np.concatenate(parts).astype(np.float32)


def poisson_solution(b):
    """Exact solution (zero mean) of 4p - sum(neighbours) = b on the periodic grid, by FFT."""
    h, w = b.shape[-2:]
    ky = np.fft.fftfreq(h)[:, None]
    kx = np.fft.fftfreq(w)[None, :]
    lam = 4.0 - 2.0 * np.cos(2 * np.pi * kx) - 2.0 * np.cos(2 * np.pi * ky)
    lam[0, 0] = 1.0
    bh = np.fft.fft2(b)
    ph = bh / lam
    ph[..., 0, 0] = 0.0
    return np.real(np.fft.ifft2(ph))
