"""Build libpfs_gb300.so in-tree with nvcc for sm_103a (GB300).

    python -m probabilistic_fluid_simulation_gb300.build [--force] [--verbose]

Each .cu under csrc/ compiles to an object in parallel, then one link step.
No fast-math: the step kernels rely on IEEE division and on explicit
round-to-nearest intrinsics for bit-exact parity with the reference.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpfs_gb300.so")
# the bounds-checking build (device-side bounds checks reported by pfs_bounds_status)
OBJDIR_BOUNDS = os.path.join(PKG, "_build_bounds")
LIB_BOUNDS = os.path.join(PKG, "libpfs_gb300_bounds.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE, "-I", CSRC,
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith((".h", ".hpp"))]
    return hs


def _compile(src: str, force: bool, verbose: bool, bounds: bool = False) -> str:
    obj = os.path.join(OBJDIR_BOUNDS if bounds else OBJDIR, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in headers()])
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-DPFS_BOUNDS_CHECK"] if bounds else []) + \
        (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


CLI_DIR = os.path.join(PKG, "cli")
PNG_LIB = os.path.join(PKG, "libpfs_png.so")
CLI_BIN = os.path.join(PKG, "fluidsim_gb300")


def _stale(target: str, deps) -> bool:
    return not os.path.exists(target) or os.path.getmtime(target) < max(os.path.getmtime(d) for d in deps)


def build_cli(force: bool = False) -> str:
    """The command-line driver (cli/fluidsim.cpp, linked against the library)
    and the PNG codec as a small shared library for the tests."""
    gxx = os.environ.get("CXX", "g++")
    png = [os.path.join(CLI_DIR, "png.cpp")]
    deps = png + [os.path.join(CLI_DIR, "png.h")]
    flags = ["-O2", "-std=c++17", "-Wall"]
    if force or _stale(PNG_LIB, deps):
        r = subprocess.run([gxx] + flags + ["-fPIC", "-shared"] + png + ["-o", PNG_LIB], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for the PNG codec:\n{r.stdout}\n{r.stderr}")
    main = os.path.join(CLI_DIR, "fluidsim.cpp")
    if force or _stale(CLI_BIN, deps + [main, LIB, os.path.join(INCLUDE, "pfs.h")]):
        cmd = [gxx] + flags + ["-pthread", main] + png + ["-I", INCLUDE, "-L", PKG, "-lpfs_gb300",
                                                          "-Wl,-rpath,$ORIGIN", "-o", CLI_BIN]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for the driver:\n{r.stdout}\n{r.stderr}")
    return CLI_BIN


def build(force: bool = False, verbose: bool = False, bounds: bool = False) -> str:
    """Build libpfs_gb300.so (and the CLI), or with bounds=True the
    bounds-checking libpfs_gb300_bounds.so (same sources, PFS_BOUNDS_CHECK)."""
    objdir, lib = (OBJDIR_BOUNDS, LIB_BOUNDS) if bounds else (OBJDIR, LIB)
    os.makedirs(objdir, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose, bounds), srcs))
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if not bounds:
        build_cli(force)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--bounds", action="store_true", help="the bounds-checking library")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose, bounds=a.bounds))
