"""The command-line driver's argument checks (src/main.cpp:40-42,110-126):
every one of them ends the run before any CUDA call, so they run without a
GPU. The messages and exit status are the reference program's."""
import os
import subprocess

import numpy as np
import pytest

import png_util as P

pytestmark = pytest.mark.skipif(not os.path.exists(P.CLI), reason="driver not built")


def run(args, env=None):
    e = dict(os.environ)
    if env:
        e.update(env)
    return subprocess.run([P.CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=60, env=e)


@pytest.fixture
def pngs(tmp_path):
    rgba = np.full((8, 8, 4), 128, np.uint8)
    for name in ("i.png", "v.png"):
        (tmp_path / name).write_bytes(P.encode(rgba, 6))  # colour type 6: RGBA
    return str(tmp_path / "i.png"), str(tmp_path / "v.png")


@pytest.mark.parametrize("args", [[], [1, 0.1, 0.0, "a.png"], [1, 0.1, 0.0, "a", "b", "c", "d"]])
def test_wrong_argument_count_prints_usage(args):
    r = run(args)
    assert r.returncode == 1
    assert "Usage:" in r.stderr and "<n_timesteps> <delta_t> <viscosity>" in r.stderr


def test_nonpositive_timesteps(pngs):
    r = run([0, 0.1, 0.0, *pngs])
    assert r.returncode == 1 and "Timesteps must be greater than 0." in r.stderr


def test_nonpositive_delta_t(pngs):
    r = run([3, 0.0, 0.0, *pngs])
    assert r.returncode == 1 and "Delta T must be greater than 0." in r.stderr


def test_missing_input_image(tmp_path, pngs):
    r = run([3, 0.1, 0.0, str(tmp_path / "missing.png"), pngs[1]])
    assert r.returncode == 1 and "Something went wrong reading the input image" in r.stderr


def test_unreadable_velocity_field(tmp_path, pngs):
    bad = tmp_path / "bad.png"
    bad.write_bytes(b"not a png at all")
    r = run([3, 0.1, 0.0, pngs[0], str(bad)])
    assert r.returncode == 1 and "Something went wrong reading the initial velocity field" in r.stderr


def test_jacobi_iterations_setting_checked(pngs):
    r = run([3, 0.1, 0.0, *pngs], env={"PFS_JACOBI_ITERS": "0"})
    assert r.returncode == 1 and "PFS_JACOBI_ITERS must be at least 1." in r.stderr
