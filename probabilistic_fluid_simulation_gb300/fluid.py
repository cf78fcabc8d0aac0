"""Python mirror of the reference's step API over libpfs_gb300.so (include/pfs.h).

The reference exposes two calls (includes/fluid.hpp:106-119):

    simulate_fluid_step(vp, tmp, dt, viscosity)
    advect_color_step(image, itmp, vp, dt)

Both take the interleaved HWC buffers of src/fluid.cpp:15-17 and swap the
caller's buffers the way the reference swaps its pointers. The functions
here take torch CUDA tensors (device buffers, the CUDA branch of the header)
or numpy arrays (host buffers, the CPU branch, computed on the GPU) and
return the buffers in their new roles.

`Session` keeps one simulation resident on the device in planar layout and
advances it many steps per call (fixed sweep count or residual stop).

There is no CPU fallback: if the CUDA library cannot be loaded every call
raises.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
# PFS_LIBRARY selects another build of the library, e.g. the bounds-checking
# libpfs_gb300_bounds.so (build.build(bounds=True)).
LIB_PATH = os.environ.get("PFS_LIBRARY") or os.path.join(_PKG, "libpfs_gb300.so")

PFS_HOST, PFS_DEVICE = 0, 1
PREC_F32, PREC_BF16, PREC_F16, PREC_F64, PREC_F32R = 0, 1, 2, 3, 4
PRECISIONS = {"f32": PREC_F32, "bf16": PREC_BF16, "f16": PREC_F16, "f64": PREC_F64, "f32r": PREC_F32R}
START_PREVIOUS, START_ZERO, START_NETWORK, START_FALLBACK = 0, 1, 2, 3
START_DAMP_PASSES, START_SLACK = 8, 4
BOUNDARY_PERIODIC, BOUNDARY_CLAMP, BOUNDARY_WALLS = 0, 1, 2


class PFSError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class _VpField(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int), ("data", C.c_void_p)]


class Params(C.Structure):
    """pfs_params (include/pfs.h)."""
    _fields_ = [("dt", C.c_float), ("viscosity", C.c_float), ("diffuse_iters", C.c_int), ("max_iters", C.c_int),
                ("tol", C.c_double), ("check_every", C.c_int), ("fuse_depth", C.c_int), ("chunk_rows", C.c_int),
                ("want_residual", C.c_int), ("precision", C.c_int), ("boundary", C.c_int),
                ("stall_sweeps", C.c_int)]


class Stats(C.Structure):
    """pfs_stats (include/pfs.h)."""
    _fields_ = [("sweeps", C.c_int), ("checks", C.c_int), ("rel_residual", C.c_double), ("bnorm", C.c_double),
                ("capped", C.c_int), ("steps", C.c_longlong), ("total_sweeps", C.c_longlong),
                ("cap_hits", C.c_longlong), ("start_kind", C.c_int), ("rel_start", C.c_double),
                ("start_passes", C.c_int), ("stalled", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None

# (name, restype, argtypes) of every symbol include/pfs.h declares
_PP = C.POINTER(C.c_void_p)
SIGNATURES = [
    ("pfs_status_string", C.c_char_p, [C.c_int]),
    ("pfs_last_error", C.c_char_p, []),
    ("pfs_version", C.c_int, []),
    ("pfs_kernel_launches", C.c_longlong, []),
    ("pfs_bounds_status", C.c_int, [C.POINTER(C.c_longlong)]),
    ("pfs_set_jacobi_iters", C.c_int, [C.c_int]),
    ("pfs_get_jacobi_iters", C.c_int, []),
    ("pfs_set_stream", C.c_int, [C.c_void_p]),
    ("pfs_release_workspace", C.c_int, []),
    ("pfs_simulate_fluid_step", C.c_int, [_PP, _PP, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int]),
    ("pfs_advect_color_step", C.c_int, [_PP, _PP, _PP, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_int]),
    ("pfs_simulate_fluid_step_host", C.c_int, [C.POINTER(_VpField), C.POINTER(_VpField), C.c_float, C.c_float]),
    ("pfs_advect_color_step_host", C.c_int, [C.POINTER(_VpField), C.POINTER(_VpField), C.POINTER(_VpField),
                                             C.c_float]),
    ("pfs_params_default", None, [C.POINTER(Params)]),
    ("pfs_session_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(Params), C.c_void_p]),
    ("pfs_session_set_params", C.c_int, [C.c_void_p, C.POINTER(Params)]),
    ("pfs_session_upload", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("pfs_session_step", C.c_int, [C.c_void_p, C.c_int]),
    ("pfs_session_download", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("pfs_session_download_f64", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("pfs_session_stats", C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    ("pfs_session_sync", C.c_int, [C.c_void_p]),
    ("pfs_session_upload_async", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pfs_session_download_async", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pfs_session_wait_io", C.c_int, [C.c_void_p]),
    ("pfs_session_destroy", C.c_int, [C.c_void_p]),
    ("pfs_unet_create", C.c_int, [C.POINTER(C.c_void_p), C.c_longlong]),
    ("pfs_unet_destroy", C.c_int, [C.c_void_p]),
    ("pfs_unet_num_params", C.c_longlong, [C.c_void_p]),
    ("pfs_unet_set_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pfs_unet_get_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pfs_unet_get_grads", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pfs_unet_forward_backward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                            C.POINTER(C.c_float), C.c_void_p]),
    ("pfs_unet_adam_step", C.c_int, [C.c_void_p, C.c_float, C.c_void_p]),
    ("pfs_unet_predict", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                   C.c_void_p]),
    ("pfs_unet_predict_coarse", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_void_p]),
    ("pfs_session_set_start", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("pfs_session_set_start_network", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    ("pfs_ensemble_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int,
                                      C.POINTER(Params), C.c_void_p]),
    ("pfs_ensemble_upload", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("pfs_ensemble_step", C.c_int, [C.c_void_p, C.c_int]),
    ("pfs_ensemble_download", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    ("pfs_ensemble_member_stats", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Stats)]),
    ("pfs_ensemble_config", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("pfs_ensemble_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]),
    ("pfs_ensemble_snapshot", C.c_int, [C.c_void_p, C.c_int]),
    ("pfs_ensemble_debug_stall_block", C.c_int, [C.c_void_p, C.c_int]),
    ("pfs_ensemble_image_stats", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_int]),
    ("pfs_ensemble_destroy", C.c_int, [C.c_void_p]),
    ("pfs_pressure_sweeps", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                      C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("pfs_residual_norms", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.c_void_p]),
    ("pfs_residual_norms_static", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                            C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p]),
]


def lib():
    """Load libpfs_gb300.so (built by probabilistic_fluid_simulation_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with "
                              "`python -m probabilistic_fluid_simulation_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int):
    if status != 0:
        raise PFSError(status, lib().pfs_last_error().decode())


def set_jacobi_iters(n: int):
    """Runtime replacement of NUM_JACOBI_ITERS (includes/fluid.hpp:11)."""
    _check(lib().pfs_set_jacobi_iters(int(n)))


def get_jacobi_iters() -> int:
    return lib().pfs_get_jacobi_iters()


def kernel_launches() -> int:
    """Kernels the library has launched since it was loaded."""
    return lib().pfs_kernel_launches()


def bounds_status() -> dict:
    """Read and clear the device-side bounds record of the bounds-checking build
    (pfs_bounds_status in include/pfs.h); raises PFSError (unsupported) on the
    normal build."""
    out = (C.c_longlong * 5)()
    _check(lib().pfs_bounds_status(out))
    return {"count": out[0], "site": out[1], "line": out[2], "index": out[3], "extent": out[4]}


def set_stream(stream_handle: int):
    _check(lib().pfs_set_stream(C.c_void_p(stream_handle or None)))


def _ptr(t) -> int:
    """Device or host address of a torch tensor / numpy array (C-contiguous)."""
    if isinstance(t, np.ndarray):
        if not t.flags.c_contiguous or t.dtype != np.float32:
            raise ValueError("numpy buffers must be C-contiguous float32")
        return t.ctypes.data
    if not t.is_contiguous() or str(t.dtype) != "torch.float32":
        raise ValueError("tensors must be contiguous float32")
    return t.data_ptr()


def _pick(addr: int, *bufs):
    for b in bufs:
        if _ptr(b) == addr:
            return b
    raise RuntimeError("library returned an unknown buffer")


def simulate_fluid_step(vp, tmp, dt: float, viscosity: float):
    """One timestep; replaces simulate_fluid_step (includes/fluid.hpp:107/109).

    vp, tmp: (h, w, 4) float32 torch CUDA tensors (device path) or numpy
    arrays (host path). Returns (vp, tmp) in the roles the reference's
    pointer swaps leave them."""
    if isinstance(vp, np.ndarray):
        h, w, z = vp.shape
        a = _VpField(w, h, z, _ptr(vp))
        b = _VpField(w, h, z, _ptr(tmp))
        _check(lib().pfs_simulate_fluid_step_host(C.byref(a), C.byref(b), float(dt), float(viscosity)))
        return _pick(a.data, vp, tmp), _pick(b.data, vp, tmp)
    h, w, z = vp.shape
    pa = C.c_void_p(_ptr(vp))
    pb = C.c_void_p(_ptr(tmp))
    _check(lib().pfs_simulate_fluid_step(C.byref(pa), C.byref(pb), float(dt), float(viscosity), w, h, z))
    return _pick(pa.value, vp, tmp), _pick(pb.value, vp, tmp)


def advect_color_step(image, itmp, vp, dt: float):
    """Image advection then buffer swap; replaces advect_color_step
    (includes/fluid.hpp:116/118). Returns (image, itmp) after the swap."""
    ih, iw, iz = image.shape
    vh, vw, vz = vp.shape
    if isinstance(image, np.ndarray):
        a = _VpField(iw, ih, iz, _ptr(image))
        b = _VpField(iw, ih, iz, _ptr(itmp))
        v = _VpField(vw, vh, vz, _ptr(vp))
        _check(lib().pfs_advect_color_step_host(C.byref(a), C.byref(b), C.byref(v), float(dt)))
        return _pick(a.data, image, itmp), _pick(b.data, image, itmp)
    pi = C.c_void_p(_ptr(image))
    pt = C.c_void_p(_ptr(itmp))
    pv = C.c_void_p(_ptr(vp))
    _check(lib().pfs_advect_color_step(C.byref(pi), C.byref(pt), C.byref(pv), float(dt), iw, ih, iz, vw, vh, vz))
    return _pick(pi.value, image, itmp), _pick(pt.value, image, itmp)


def default_params(**kw) -> Params:
    p = Params()
    lib().pfs_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class Session:
    """One simulation resident on the device (pfs_session_* in include/pfs.h)."""

    def __init__(self, w: int, h: int, image_shape: Optional[Tuple[int, int, int]] = None,
                 params: Optional[Params] = None, stream: int = 0, **kw):
        self._h = C.c_void_p()
        self.w, self.h = w, h
        ih, iw, ic = image_shape if image_shape else (0, 0, 0)
        self.image_shape = (ih, iw, ic)
        self.params = params if params is not None else default_params(**kw)
        _check(lib().pfs_session_create(C.byref(self._h), w, h, iw, ih, ic, C.byref(self.params),
                                        C.c_void_p(stream or None)))

    def set_params(self, **kw):
        for k, v in kw.items():
            setattr(self.params, k, v)
        _check(lib().pfs_session_set_params(self._h, C.byref(self.params)))

    def upload(self, vp, tmp, image=None):
        where = PFS_HOST if isinstance(vp, np.ndarray) else PFS_DEVICE
        _check(lib().pfs_session_upload(self._h, C.c_void_p(_ptr(vp)), C.c_void_p(_ptr(tmp)),
                                        C.c_void_p(_ptr(image) if image is not None else None), where))

    def step(self, n: int = 1):
        _check(lib().pfs_session_step(self._h, int(n)))

    def download(self, vp=None, tmp=None, image=None):
        """Fill the given buffers (numpy -> host, torch -> device); returns them."""
        ref = next(x for x in (vp, tmp, image) if x is not None)
        where = PFS_HOST if isinstance(ref, np.ndarray) else PFS_DEVICE
        _check(lib().pfs_session_download(self._h, C.c_void_p(_ptr(vp) if vp is not None else None),
                                          C.c_void_p(_ptr(tmp) if tmp is not None else None),
                                          C.c_void_p(_ptr(image) if image is not None else None), where))
        return vp, tmp, image

    def download_f64(self, vp=None, image=None):
        """The state in float64 (numpy float64 arrays -> host): vp (u, v, p, b), image."""
        ref = vp if vp is not None else image
        where = PFS_HOST if isinstance(ref, np.ndarray) else PFS_DEVICE

        def addr(a):
            if a is None:
                return None
            if isinstance(a, np.ndarray):
                if a.dtype != np.float64 or not a.flags.c_contiguous:
                    raise ValueError("float64 C-contiguous arrays expected")
                return a.ctypes.data
            return a.data_ptr()
        _check(lib().pfs_session_download_f64(self._h, C.c_void_p(addr(vp)), C.c_void_p(addr(image)), where))
        return vp, image

    def stats(self) -> dict:
        s = Stats()
        _check(lib().pfs_session_stats(self._h, C.byref(s)))
        return s.as_dict()

    def checkpoint(self, path: str):
        """Write the state (both velocity buffers with channels 2-3, the image)
        and the parameters to an .npz file. For the float32 form this is the
        whole state: restoring it into a session with the same parameters and
        stepping on gives the same bits as never stopping. The refined forms
        keep their pressure in FP64, which this float32 snapshot rounds."""
        h, w = self.h, self.w
        vp, tmp = np.empty((h, w, 4), np.float32), np.empty((h, w, 4), np.float32)
        ih, iw, ic = self.image_shape
        img = np.empty((ih, iw, ic), np.float32) if ic else None
        self.download(vp, tmp, img)
        st = self.stats()
        params = {k: getattr(self.params, k) for k, _ in Params._fields_}
        np.savez(path, vp=vp, tmp=tmp, image=img if img is not None else np.zeros(0, np.float32),
                 params=json.dumps(params), steps=st["steps"])

    @classmethod
    def restore(cls, path: str, stream: int = 0) -> "Session":
        """A new session holding a checkpoint's state and parameters."""
        z = np.load(path)
        vp, tmp, img = z["vp"], z["tmp"], z["image"]
        params = default_params(**json.loads(str(z["params"])))
        h, w, _ = vp.shape
        s = cls(w, h, image_shape=img.shape if img.size else None, params=params, stream=stream)
        s.upload(vp, tmp, img if img.size else None)
        return s

    def set_start(self, mode: int, net: "UNet" = None, coarsen: int = 1, passes: int = 1):
        """Initial pressure of each step: START_PREVIOUS (reference), START_ZERO,
        START_NETWORK (the network run on the grid coarsened `coarsen` times,
        applied `passes` times)."""
        self._net = net  # keep the network alive while the session uses it
        if mode == START_NETWORK:
            _check(lib().pfs_session_set_start_network(self._h, net._h if net is not None else None, int(coarsen),
                                                       int(passes)))
        else:
            _check(lib().pfs_session_set_start(self._h, int(mode), net._h if net is not None else None))

    def upload_async(self, vp: np.ndarray, tmp: np.ndarray, image: Optional[np.ndarray] = None):
        """Queue a state from host arrays (pinned ones overlap the copy with
        the steps); the next step() starts from it. The arrays are kept
        referenced, and must stay unchanged, until wait_io() or sync()."""
        self._check_host(vp, tmp, image, "upload_async")
        _check(lib().pfs_session_upload_async(self._h, C.c_void_p(_ptr(vp)), C.c_void_p(_ptr(tmp)),
                                              C.c_void_p(_ptr(image) if image is not None else None)))
        self._inflight().append((vp, tmp, image))

    def download_async(self, vp: Optional[np.ndarray] = None, tmp: Optional[np.ndarray] = None,
                       image: Optional[np.ndarray] = None):
        """Queue a copy of the state after the steps queued so far into host
        arrays; they hold it once wait_io() or sync() has returned."""
        self._check_host(vp, tmp, image, "download_async")
        _check(lib().pfs_session_download_async(self._h, C.c_void_p(_ptr(vp) if vp is not None else None),
                                                C.c_void_p(_ptr(tmp) if tmp is not None else None),
                                                C.c_void_p(_ptr(image) if image is not None else None)))
        self._inflight().append((vp, tmp, image))

    def _check_host(self, vp, tmp, image, what):
        ih, iw, ic = self.image_shape
        for a, n in ((vp, self.h * self.w * 4), (tmp, self.h * self.w * 4), (image, ih * iw * ic)):
            if a is None:
                continue
            if not isinstance(a, np.ndarray):
                raise TypeError(f"{what} takes host (numpy) arrays")
            if a.size != n:
                raise ValueError(f"{what}: buffer of {a.size} floats, {n} expected")

    def _inflight(self) -> list:
        if not hasattr(self, "_io"):
            self._io = []
        return self._io

    def wait_io(self):
        _check(lib().pfs_session_wait_io(self._h))
        self._inflight().clear()

    def sync(self):
        _check(lib().pfs_session_sync(self._h))
        self._inflight().clear()

    def close(self):
        if self._h:
            lib().pfs_session_destroy(self._h)
            self._h = C.c_void_p()
        self._inflight().clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class UNet:
    """The warm-start network (pfs_unet_* in include/pfs.h)."""

    def __init__(self, max_pixels: int):
        self._h = C.c_void_p()
        _check(lib().pfs_unet_create(C.byref(self._h), int(max_pixels)))
        self.n_params = lib().pfs_unet_num_params(self._h)

    def set_params(self, params: np.ndarray):
        params = np.ascontiguousarray(params, np.float32)
        assert params.size == self.n_params
        _check(lib().pfs_unet_set_params(self._h, C.c_void_p(params.ctypes.data)))

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        _check(lib().pfs_unet_get_params(self._h, C.c_void_p(out.ctypes.data)))
        return out

    def grads(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        _check(lib().pfs_unet_get_grads(self._h, C.c_void_p(out.ctypes.data)))
        return out

    def forward_backward(self, b, p, stream: int = 0) -> float:
        """b, p: (n, h, w) float32 CUDA tensors (normalised pairs)."""
        n, h, w = b.shape
        loss = C.c_float()
        _check(lib().pfs_unet_forward_backward(self._h, C.c_void_p(_ptr(b)), C.c_void_p(_ptr(p)), n, h, w,
                                               C.byref(loss), C.c_void_p(stream or None)))
        return loss.value

    def adam_step(self, lr: float, stream: int = 0):
        _check(lib().pfs_unet_adam_step(self._h, float(lr), C.c_void_p(stream or None)))

    def predict(self, b, out, coarsen: int = 1, stream: int = 0):
        """b, out: (h, w) float32 CUDA tensors: out = rms(b) * net(b / rms(b)),
        the network run on the grid coarsened `coarsen` times."""
        h, w = b.shape
        if coarsen == 1:
            _check(lib().pfs_unet_predict(self._h, C.c_void_p(_ptr(b)), w, C.c_void_p(_ptr(out)), w, h, w,
                                          C.c_void_p(stream or None)))
        else:
            _check(lib().pfs_unet_predict_coarse(self._h, C.c_void_p(_ptr(b)), w, C.c_void_p(_ptr(out)), w, h, w,
                                                 int(coarsen), C.c_void_p(stream or None)))
        return out

    def close(self):
        if self._h:
            lib().pfs_unet_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Many independent simulations in one persistent kernel per timestep
    (pfs_ensemble_* in include/pfs.h). sizes: list of (w, h)."""

    def __init__(self, sizes, channels: int, params: Optional[Params] = None, stream: int = 0, **kw):
        self._h = C.c_void_p()
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        self.channels = channels
        self.params = params if params is not None else default_params(**kw)
        n = len(self.sizes)
        ws = (C.c_int * n)(*[w for w, _ in self.sizes])
        hs = (C.c_int * n)(*[h for _, h in self.sizes])
        _check(lib().pfs_ensemble_create(C.byref(self._h), n, ws, hs, channels, C.byref(self.params),
                                         C.c_void_p(stream or None)))

    def upload(self, k: int, vp, tmp, image=None):
        where = PFS_HOST if isinstance(vp, np.ndarray) else PFS_DEVICE
        _check(lib().pfs_ensemble_upload(self._h, k, C.c_void_p(_ptr(vp)), C.c_void_p(_ptr(tmp)),
                                         C.c_void_p(_ptr(image) if image is not None else None), where))

    def step(self, n: int = 1):
        _check(lib().pfs_ensemble_step(self._h, int(n)))

    def download(self, k: int, vp=None, image=None):
        ref = vp if vp is not None else image
        where = PFS_HOST if isinstance(ref, np.ndarray) else PFS_DEVICE
        _check(lib().pfs_ensemble_download(self._h, k, C.c_void_p(_ptr(vp) if vp is not None else None),
                                           C.c_void_p(_ptr(image) if image is not None else None), where))
        return vp, image

    def debug_stall_block(self, block: int):
        """Test hook: block `block` skips the next step's grid barriers (the step then times out)."""
        _check(lib().pfs_ensemble_debug_stall_block(self._h, int(block)))

    def image_stats(self, members, mean=None, var=None):
        """Pointwise mean and population variance of the image over `members`
        (one grid size): numpy (h, w, channels) float32 arrays by default, or
        the given numpy / torch CUDA buffers."""
        members = [int(m) for m in members]
        w, h = self.sizes[members[0]]
        if mean is None:
            mean = np.empty((h, w, self.channels), np.float32)
        if var is None:
            var = np.empty_like(mean) if isinstance(mean, np.ndarray) else mean.new_empty(mean.shape)
        where = PFS_HOST if isinstance(mean, np.ndarray) else PFS_DEVICE
        sel = (C.c_int * len(members))(*members)
        _check(lib().pfs_ensemble_image_stats(self._h, sel, len(members), C.c_void_p(_ptr(mean)),
                                              C.c_void_p(_ptr(var)), where))
        return mean, var

    def stats(self, k: int) -> dict:
        s = Stats()
        _check(lib().pfs_ensemble_member_stats(self._h, k, C.byref(s)))
        return s.as_dict()

    def config(self, fuse_depth: int, chunk_rows: int):
        _check(lib().pfs_ensemble_config(self._h, int(fuse_depth), int(chunk_rows)))

    def snapshot(self):
        _check(lib().pfs_ensemble_snapshot(self._h, 0))

    def restore(self):
        _check(lib().pfs_ensemble_snapshot(self._h, 1))

    def info(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        _check(lib().pfs_ensemble_info(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("fuse_depth", "chunk_rows", "grid_blocks", "graphs"), [x.value for x in v]))

    def close(self):
        if self._h:
            lib().pfs_ensemble_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def pressure_sweeps(p_in, b, p_out, p_prev, levels: int, fused: bool = True, chunk_rows: int = 0,
                    w: Optional[int] = None, stream: int = 0):
    """`levels` Jacobi sweeps on planar (h, ld) tensors whose first w columns
    are the grid (kernel-level entry point)."""
    h, ldd = p_in.shape
    w = w if w is not None else ldd
    _check(lib().pfs_pressure_sweeps(C.c_void_p(_ptr(p_in)), C.c_void_p(_ptr(b)), C.c_void_p(_ptr(p_out)),
                                     C.c_void_p(_ptr(p_prev) if p_prev is not None else None), w, h, ldd,
                                     int(levels), int(fused), int(chunk_rows), C.c_void_p(stream or None)))


def residual_norms(p, b, w: Optional[int] = None, stream: int = 0) -> Tuple[float, float]:
    """(||b - A p||^2, ||b||^2) in FP64 for planar (h, ld) tensors."""
    h, ld = p.shape
    rr, bb = C.c_double(), C.c_double()
    _check(lib().pfs_residual_norms(C.c_void_p(_ptr(p)), C.c_void_p(_ptr(b)), w or ld, h, ld, C.byref(rr),
                                    C.byref(bb), C.c_void_p(stream or None)))
    return rr.value, bb.value


def residual_norms_static(p, b, w: Optional[int] = None, stream: int = 0) -> Tuple[float, float]:
    """residual_norms for callers that must not allocate device memory: the
    reduction's scratch is a fixed array inside the library
    (pfs_residual_norms_static in include/pfs.h)."""
    h, ld = p.shape
    rr, bb = C.c_double(), C.c_double()
    _check(lib().pfs_residual_norms_static(C.c_void_p(_ptr(p)), C.c_void_p(_ptr(b)), w or ld, h, ld, C.byref(rr),
                                           C.byref(bb), C.c_void_p(stream or None)))
    return rr.value, bb.value
