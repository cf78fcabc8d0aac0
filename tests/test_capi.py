"""The C-ABI library without a GPU: it loads, exports every entry point that
include/*.h declares, and rejects bad arguments before touching the device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(pfs_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(pfs_lib):
    lib = pfs_lib.lib()
    declared = declared_functions()
    assert len(declared) >= 20
    for name in sorted(declared):
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    bound = {n for n, _, _ in pfs_lib.SIGNATURES}
    assert declared <= bound, f"Python binding misses {declared - bound}"


def test_status_strings(pfs_lib):
    lib = pfs_lib.lib()
    assert lib.pfs_status_string(0) == b"ok"
    assert lib.pfs_status_string(1) == b"invalid argument"
    assert lib.pfs_status_string(99) == b"unknown status"
    assert lib.pfs_version() >= 100


def test_jacobi_iters_setting(pfs_lib):
    old = pfs_lib.get_jacobi_iters()
    assert old == 30  # includes/fluid.hpp:11
    pfs_lib.set_jacobi_iters(40)
    assert pfs_lib.get_jacobi_iters() == 40
    with pytest.raises(pfs_lib.PFSError) as e:
        pfs_lib.set_jacobi_iters(-1)
    assert e.value.status == 1
    pfs_lib.set_jacobi_iters(old)


def test_invalid_arguments_rejected_on_host(pfs_lib):
    lib = pfs_lib.lib()
    a = C.c_void_p(0)
    assert lib.pfs_simulate_fluid_step(C.byref(a), C.byref(a), 0.1, 0.0, 8, 8, 4) == 1
    x, y = C.c_void_p(16), C.c_void_p(32)
    assert lib.pfs_simulate_fluid_step(C.byref(x), C.byref(y), 0.1, 0.0, 8, 8, 3) == 1  # vz must be 4
    assert b"4 channels" in lib.pfs_last_error()
    assert lib.pfs_simulate_fluid_step(C.byref(x), C.byref(y), -0.1, 0.0, 8, 8, 4) == 1  # dt <= 0
    assert lib.pfs_simulate_fluid_step(C.byref(x), C.byref(y), 0.1, float("nan"), 8, 8, 4) == 3
    assert lib.pfs_simulate_fluid_step(C.byref(x), C.byref(x), 0.1, 0.0, 8, 8, 4) == 1  # aliased buffers
    assert lib.pfs_advect_color_step(C.byref(x), C.byref(x), C.byref(y), 0.1, 8, 8, 3, 8, 8, 4) == 1
    assert lib.pfs_pressure_sweeps(None, None, None, None, 8, 8, 8, 1, 1, 0, None) == 1
    p = pfs_lib.default_params(dt=0.0)
    s = C.c_void_p()
    assert lib.pfs_session_create(C.byref(s), 8, 8, 0, 0, 0, C.byref(p), None) == 1
    p = pfs_lib.default_params(fuse_depth=9)
    assert lib.pfs_session_create(C.byref(s), 8, 8, 0, 0, 0, C.byref(p), None) == 1


def test_host_call_shape_checks(pfs_lib):
    vp = np.zeros((4, 4, 4), np.float32)
    tmp = np.zeros((4, 5, 4), np.float32)
    with pytest.raises(pfs_lib.PFSError):
        pfs_lib.simulate_fluid_step(vp, tmp, 0.1, 0.0)


def test_params_default(pfs_lib):
    p = pfs_lib.default_params()
    assert p.dt == pytest.approx(0.1) and p.max_iters == 30 and p.diffuse_iters == 30 and p.tol == 0.0


def test_headers_compile_as_c_and_cxx():
    """include/pfs.h is plain C (a cgo / JNI / FFI binding includes it as
    such) and also valid C++."""
    import shutil
    import subprocess
    if not shutil.which("gcc") or not shutil.which("g++"):
        pytest.skip("no host compiler")
    hdr = os.path.join(ROOT, "include", "pfs.h")
    for cmd in (["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c", hdr],
                ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c++", hdr]):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
