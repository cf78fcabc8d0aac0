"""The command-line driver (fluidsim_gb300) against the reference's program
flow (src/main.cpp) restated with the oracle: PNG inputs made by an
independent writer, outputs decoded by an independent reader, every step's
image compared byte for byte."""
import os
import subprocess

import numpy as np
import pytest

import png_util as P

pytestmark = pytest.mark.gpu


def smooth_rgba(w, h, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    out = np.empty((h, w, 4))
    for c in range(4):
        kx, ky, ph = rng.uniform(1, 3), rng.uniform(1, 3), rng.uniform(0, 6.3)
        out[..., c] = 0.5 + 0.45 * np.sin(2 * np.pi * kx * xx / w + ph) * np.cos(2 * np.pi * ky * yy / h)
    return np.clip(np.round(out * 255), 0, 255).astype(np.uint8)


def to_float(b):
    return (b.astype(np.float32).astype(np.float64) / 255.0).astype(np.float32)  # includes/utils.hpp:81-83


@pytest.mark.parametrize("vel,img,steps,visc", [((64, 48), (64, 48), 3, 0.0), ((48, 40), (72, 56), 2, 0.05)])
def test_cli_matches_reference_flow(cuda_device, oracle_mod, tmp_path, vel, img, steps, visc):
    vb, ib = smooth_rgba(*vel, seed=1), smooth_rgba(*img, seed=2)
    (tmp_path / "v.png").write_bytes(P.encode(vb, 6))
    (tmp_path / "i.png").write_bytes(P.encode(ib, 6))
    out = tmp_path / "out"
    env = dict(os.environ, PFS_JACOBI_ITERS="30")
    r = subprocess.run([P.CLI, str(steps), "0.1", str(visc), str(tmp_path / "i.png"), str(tmp_path / "v.png"),
                        str(out)], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert f"Simulating [{vel[1]} x {vel[0]}] domain for {steps} timesteps at dt=0.1..." in r.stdout
    assert f"{steps} timesteps took" in r.stdout

    # src/main.cpp:171-195: rescale all four channels, tmp = (-1, -1, -1, 1)
    vp = (to_float(vb).astype(np.float64) * 2.0 - 1.0).astype(np.float32)
    tmp = np.tile(np.array([-1, -1, -1, 1], np.float32), vp.shape[:2] + (1,))
    image, itmp = to_float(ib), np.zeros(ib.shape, np.float32)
    dt = float(np.float32(0.1))
    for i in range(steps):
        vp, tmp, _ = oracle_mod.step(vp, tmp, dt, float(np.float32(visc)), diffuse_iters=30, max_iters=30)
        image, itmp = oracle_mod.advect_color_step(image, itmp, vp, dt)
        want = np.clip(np.trunc(image.astype(np.float64) * 255.0), 0, 255).astype(np.uint8)
        got = P.decode_rgba8((out / f"{i}.png").read_bytes())
        assert np.array_equal(got, want), (i, np.abs(got.astype(int) - want).max())
