"""The C++ drop-in header include/fluid.hpp: it compiles with a plain C++
compiler against the C ABI (no CUDA headers needed) and, on a GPU, a program
using it the way the reference's src/main.cpp does matches the reference."""
import os
import subprocess

import numpy as np
import pytest

from golden_util import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp")
PKG = os.path.join(ROOT, "probabilistic_fluid_simulation_gb300")


def build_dropin(tmp_path):
    exe = str(tmp_path / "dropin_main")
    cmd = ["g++", "-std=c++11", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", PKG, "-lpfs_gb300", f"-Wl,-rpath,{PKG}"]
    subprocess.run(cmd, check=True)
    return exe


def test_fluid_hpp_compiles_without_cuda(pfs_lib, tmp_path):
    exe = build_dropin(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["vortex32x24_it40", "vortex20x14_it3_visc"])
def test_cpp_dropin_matches_reference(cuda_device, pfs_lib, tmp_path, name):
    meta, arrs = load(name)
    exe = build_dropin(tmp_path)
    h, w, _ = arrs["in_vp"].shape
    ih, iw, ic = arrs["in_img"].shape
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([w, h, iw, ih, ic], np.int32).tofile(f)
        for k in ("in_vp", "in_tmp", "in_img"):
            arrs[k].astype(np.float32).tofile(f)
    steps = meta["steps"]
    subprocess.run([exe, str(inp), str(out), str(steps), str(meta["dt"]), str(meta["viscosity"]),
                    str(meta["iters"])], check=True)
    raw = np.fromfile(out, np.float32)[5:]
    nv, ni = h * w * 4, ih * iw * ic
    got = {"vp": raw[:nv].reshape(h, w, 4), "tmp": raw[nv:2 * nv].reshape(h, w, 4),
           "img": raw[2 * nv:2 * nv + ni].reshape(ih, iw, ic), "itmp": raw[2 * nv + ni:].reshape(ih, iw, ic)}
    for k, v in got.items():
        assert np.array_equal(v, arrs[f"{k}_s{steps}"]), k
