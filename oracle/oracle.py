"""ctypes binding of the CPU oracle (oracle/liboracle.so) and of the reference
build (oracle/_ref/libfluidref_it<N>.so, present only where the reference
sources were available to compile).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg. The product never imports this module.

Arrays are numpy, interleaved HWC exactly as the reference stores them
(src/fluid.cpp:15-17): velocity (h, w, 4), image (h, w, C). The step calls
swap the caller's buffers like the reference does (src/fluid.cpp:188-194,
260-266, 317-319); the Python functions return the arrays in their new roles.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


class _Stats(C.Structure):
    _fields_ = [("sweeps", C.c_int), ("checks", C.c_int), ("rel_residual", C.c_double),
                ("bnorm", C.c_double), ("capped", C.c_int)]


@dataclass
class StepStats:
    sweeps: int
    checks: int
    rel_residual: float
    bnorm: float
    capped: bool


_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with oracle/Makefile (no reference needed)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f))
                                             for f in ("fluid_oracle.c", "fluid_oracle_body.h")):
        subprocess.run(["make", "-C", HERE, "oracle"], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        for sfx, real in (("_f32", C.c_float), ("_f64", C.c_double)):
            f = getattr(L, "pfso_step" + sfx)
            f.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int, real, real,
                          C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(_Stats)]
            f.restype = C.c_int
            f = getattr(L, "pfso_step_bc" + sfx)
            f.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int, real, real,
                          C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(_Stats)]
            f.restype = C.c_int
            f = getattr(L, "pfso_advect_color_step" + sfx)
            f.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int,
                          C.c_void_p, C.c_int, C.c_int, real]
            f.restype = C.c_int
            f = getattr(L, "pfso_advect_color_step_bc" + sfx)
            f.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int,
                          C.c_void_p, C.c_int, C.c_int, real, C.c_int]
            f.restype = C.c_int
            getattr(L, "pfso_advect" + sfx).argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, real]
            getattr(L, "pfso_pressure_sweep" + sfx).argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
            getattr(L, "pfso_divergence" + sfx).argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, real]
            f = getattr(L, "pfso_residual" + sfx)
            f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
            f.restype = C.c_double
        L.pfso_num_threads.restype = C.c_int
        L.pfso_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    lib().pfso_set_num_threads(int(n))
    return lib().pfso_num_threads()


def _sfx(a: np.ndarray) -> str:
    if a.dtype == np.float32:
        return "_f32"
    if a.dtype == np.float64:
        return "_f64"
    raise TypeError(f"oracle supports float32/float64, got {a.dtype}")


def _check(a: np.ndarray, ch: Optional[int] = None):
    if not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous")
    if a.ndim != 3 or (ch is not None and a.shape[2] != ch):
        raise ValueError(f"expected (h, w, {ch or 'C'}) array, got {a.shape}")


def _pick(ptr: int, arrays):
    for a in arrays:
        if a.ctypes.data == ptr:
            return a
    raise RuntimeError("oracle returned an unknown buffer")


def step(vp: np.ndarray, tmp: np.ndarray, dt: float, viscosity: float, *, diffuse_iters: int,
         max_iters: int, tol: float = 0.0, check_every: int = 0,
         want_residual: bool = False, boundary: int = 0) -> Tuple[np.ndarray, np.ndarray, StepStats]:
    """One timestep (src/fluid.cpp:298-310 generalised; see fluid_oracle_body.h).

    Mutates both arrays; returns (vp_after, tmp_after, stats) where the
    first two are the input arrays in the roles the pointer swaps left them.
    boundary: 0 periodic (the reference), 1 clamp (the reference's commented
    clamp mode, src/fluid.cpp:43-45), 2 walls (clamp + zero velocity on the
    boundary cells after advection and projection).
    """
    _check(vp, 4)
    _check(tmp, 4)
    if vp.shape != tmp.shape or vp.dtype != tmp.dtype:
        raise ValueError("vp and tmp must match")
    h, w, _ = vp.shape
    real = C.c_float if vp.dtype == np.float32 else C.c_double
    p_vp = C.c_void_p(vp.ctypes.data)
    p_tmp = C.c_void_p(tmp.ctypes.data)
    st = _Stats()
    rc = getattr(lib(), "pfso_step_bc" + _sfx(vp))(C.byref(p_vp), C.byref(p_tmp), w, h, real(dt),
                                                    real(viscosity), int(diffuse_iters), int(max_iters),
                                                    float(tol), int(check_every), int(want_residual),
                                                    int(boundary), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"pfso_step failed: {rc}")
    a = _pick(p_vp.value, (vp, tmp))
    b = _pick(p_tmp.value, (vp, tmp))
    return a, b, StepStats(st.sweeps, st.checks, st.rel_residual, st.bnorm, bool(st.capped))


def advect_color_step(image: np.ndarray, itmp: np.ndarray, vel: np.ndarray, dt: float, boundary: int = 0):
    """src/fluid.cpp:312-320: returns (image_after, itmp_after); boundary as in step()."""
    _check(image)
    _check(itmp)
    _check(vel, 4)
    ih, iw, ic = image.shape
    vh, vw, _ = vel.shape
    real = C.c_float if image.dtype == np.float32 else C.c_double
    p_i = C.c_void_p(image.ctypes.data)
    p_t = C.c_void_p(itmp.ctypes.data)
    rc = getattr(lib(), "pfso_advect_color_step_bc" + _sfx(image))(C.byref(p_i), C.byref(p_t), iw, ih, ic,
                                                                    C.c_void_p(vel.ctypes.data), vw, vh, real(dt),
                                                                    int(boundary))
    if rc != 0:
        raise RuntimeError(f"pfso_advect_color_step failed: {rc}")
    return _pick(p_i.value, (image, itmp)), _pick(p_t.value, (image, itmp))


def residual(vp: np.ndarray) -> Tuple[float, float]:
    """(||b - A p||_2 / ||b||_2, ||b||_2) for channels 2 (p) and 3 (b) of vp."""
    _check(vp, 4)
    h, w, _ = vp.shape
    bn = C.c_double()
    r = getattr(lib(), "pfso_residual" + _sfx(vp))(C.c_void_p(vp.ctypes.data), w, h, C.byref(bn))
    return float(r), float(bn.value)


def pressure_sweep(src: np.ndarray, dst: np.ndarray):
    h, w, _ = src.shape
    getattr(lib(), "pfso_pressure_sweep" + _sfx(src))(C.c_void_p(src.ctypes.data), C.c_void_p(dst.ctypes.data), w, h)


# ----------------------------------------------------------------------------------------------
# The reference's own src/fluid.cpp (oracle/_ref), where it could be compiled.

def ref_available(iters: int, variant: str = "") -> bool:
    """variant "" is src/fluid.cpp as it is; "_clamp" its commented clamp mode enabled."""
    return os.path.exists(os.path.join(REF_DIR, f"libfluidref{variant}_it{iters}.so"))


_refs = {}


def ref_lib(iters: int, variant: str = ""):
    key = (iters, variant)
    if key not in _refs:
        path = os.path.join(REF_DIR, f"libfluidref{variant}_it{iters}.so")
        L = C.CDLL(path)
        L.pfsref_simulate_fluid_step.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                                 C.c_float, C.c_float]
        L.pfsref_advect_color_step.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                               C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_float]
        L.pfsref_num_jacobi_iters.restype = C.c_int
        assert L.pfsref_num_jacobi_iters() == iters
        _refs[key] = L
    return _refs[key]


def ref_step(iters: int, vp: np.ndarray, tmp: np.ndarray, dt: float, viscosity: float, variant: str = ""):
    """The reference's simulate_fluid_step (includes/fluid.hpp:109) built with
    NUM_JACOBI_ITERS = iters; returns (vp_after, tmp_after)."""
    _check(vp, 4)
    h, w, _ = vp.shape
    p_vp = C.c_void_p(vp.ctypes.data)
    p_tmp = C.c_void_p(tmp.ctypes.data)
    ref_lib(iters, variant).pfsref_simulate_fluid_step(C.byref(p_vp), C.byref(p_tmp), w, h, C.c_float(dt),
                                                       C.c_float(viscosity))
    return _pick(p_vp.value, (vp, tmp)), _pick(p_tmp.value, (vp, tmp))


def ref_advect_color_step(iters: int, image: np.ndarray, itmp: np.ndarray, vel: np.ndarray, dt: float,
                          variant: str = ""):
    ih, iw, ic = image.shape
    vh, vw, _ = vel.shape
    p_i = C.c_void_p(image.ctypes.data)
    p_t = C.c_void_p(itmp.ctypes.data)
    ref_lib(iters, variant).pfsref_advect_color_step(C.byref(p_i), C.byref(p_t), iw, ih, ic,
                                                     C.c_void_p(vel.ctypes.data), vw, vh, C.c_float(dt))
    return _pick(p_i.value, (image, itmp)), _pick(p_t.value, (image, itmp))
