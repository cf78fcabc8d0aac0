"""Seeded synthetic inputs for the fluid step.

The reference drives its step from PNG files (src/main.cpp:129-179); the
workloads here replace them with generated fields of the same shape and
layout (interleaved HWC, src/fluid.cpp:15-17):

* velocity: a sum of Gaussian vortices on the periodic grid, channels
  (u, v, p=0, b=0);
* image: C channels of smooth Gaussian blobs with values in [0, 1].

Random numbers come from a SplitMix64 stream written here (Marsaglia's polar
method for normals). Every function is evaluated with IEEE +, -, *, /, sqrt
and exact scaling only (exp and log below are written out as range reduction
plus a series), so a seed gives bit-identical fields on x86-64 and aarch64
hosts. Fields are evaluated in float64 and cast to float32 once.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace
from typing import List, Sequence

import numpy as np

_MASK = (1 << 64) - 1


_LN2_HI = 6.93147180369123816490e-01  # ln 2 split so k*_LN2_HI is exact for |k| < 2^20
_LN2_LO = 1.90821492927058770002e-10
_INV_LN2 = 1.4426950408889634


def det_exp(x):
    """exp(x) from IEEE arithmetic only: x = k ln2 + r (Cody-Waite), |r| <= ln2/2,
    e^r by its Taylor series to degree 14 (truncation < 1e-19), times 2^k."""
    x = np.asarray(x, np.float64)
    x = np.maximum(x, -700.0)
    k = np.round(x * _INV_LN2)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.ones_like(r)
    for n in range(14, 0, -1):
        p = 1.0 + p * r / n
    return np.ldexp(p, k.astype(np.int64))


def det_log(x: float) -> float:
    """log(x), x > 0, from IEEE arithmetic only: x = m 2^e with m in [1/sqrt2, sqrt2),
    log m = 2 atanh(s), s = (m-1)/(m+1), by its odd series to s^41."""
    m, e = math.frexp(x)
    if m < 0.7071067811865476:
        m *= 2.0
        e -= 1
    s = (m - 1.0) / (m + 1.0)
    s2 = s * s
    acc = 0.0
    for n in range(41, 0, -2):
        acc = 1.0 / n + s2 * acc
    return e * _LN2_HI + (e * _LN2_LO + 2.0 * s * acc)


class SplitMix64:
    """SplitMix64 generator (Steele, Lea, Flood 2014) with uniform/normal draws."""

    def __init__(self, seed: int):
        self.state = seed & _MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        u = (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def normal(self, mean: float = 0.0, std: float = 1.0) -> float:
        """Marsaglia's polar method (one of each pair is used)."""
        while True:
            a = self.uniform(-1.0, 1.0)
            b = self.uniform(-1.0, 1.0)
            q = a * a + b * b
            if 0.0 < q < 1.0:
                return mean + std * (a * math.sqrt(-2.0 * det_log(q) / q))


@dataclass(frozen=True)
class Vortex:
    cx: float
    cy: float
    radius: float
    circulation: float


def _size_scale(w: int, h: int) -> float:
    return math.sqrt(float(w) * float(h)) / 256.0


def draw_vortices(w: int, h: int, seed: int, count: int = 8,
                  radius_cells: Sequence[float] = (8.0, 32.0)) -> List[Vortex]:
    """Centres uniform on the grid, radius uniform in radius_cells scaled by
    grid size / 256, circulation N(0, 1)."""
    rng = SplitMix64(seed)
    s = _size_scale(w, h)
    out = []
    for _ in range(count):
        cx = rng.uniform(0.0, w)
        cy = rng.uniform(0.0, h)
        r = rng.uniform(radius_cells[0], radius_cells[1]) * s
        g = rng.normal()
        out.append(Vortex(cx, cy, r, g))
    return out


def perturb_vortices(base: Sequence[Vortex], seed: int, member: int,
                     circ_std: float = 0.05, pos_std: float = 2.0) -> List[Vortex]:
    """One ensemble member: circulations + N(0, circ_std), centres + N(0, pos_std) cells."""
    rng = SplitMix64((seed * 0x100000001B3 + 0x5851F42D4C957F2D * (member + 1)) & _MASK)
    return [replace(v, cx=v.cx + rng.normal(0.0, pos_std), cy=v.cy + rng.normal(0.0, pos_std),
                    circulation=v.circulation + rng.normal(0.0, circ_std)) for v in base]


def _min_image(coord: np.ndarray, centre: float, n: int) -> np.ndarray:
    d = coord - centre
    return d - n * np.round(d / n)


def velocity_from_vortices(w: int, h: int, vortices: Sequence[Vortex]) -> np.ndarray:
    """Interleaved (h, w, 4) float32 field: u, v from the vortices, p = b = 0.

    Each vortex has stream function psi = G R e^(1/2) exp(-r^2 / 2R^2), so
    u = dpsi/dy, v = -dpsi/dx peak at |G| on the ring r = R and the field is
    divergence-free; distances use the minimum image, so it is periodic. The
    Gaussian is evaluated as a product of its x and y factors.
    """
    x = np.arange(w, dtype=np.float64)
    y = np.arange(h, dtype=np.float64)
    u = np.zeros((h, w), np.float64)
    v = np.zeros((h, w), np.float64)
    e05 = float(det_exp(0.5))
    for vx in vortices:
        dx = _min_image(x, vx.cx, w)
        dy = _min_image(y, vx.cy, h)
        s2 = 2.0 * vx.radius * vx.radius
        e = det_exp(-(dy * dy) / s2)[:, None] * (e05 * det_exp(-(dx * dx) / s2))[None, :]
        u += (-vx.circulation / vx.radius) * dy[:, None] * e
        v += (vx.circulation / vx.radius) * dx[None, :] * e
    out = np.zeros((h, w, 4), np.float32)
    out[..., 0] = u
    out[..., 1] = v
    return out


def vortex_field(w: int, h: int, seed: int, count: int = 8) -> np.ndarray:
    """Seeded sum of `count` Gaussian vortices, interleaved (h, w, 4) float32."""
    return velocity_from_vortices(w, h, draw_vortices(w, h, seed, count))


def blob_image(w: int, h: int, channels: int, seed: int, count: int = 16,
               radius_cells: Sequence[float] = (8.0, 32.0)) -> np.ndarray:
    """Seeded image of `count` Gaussian blobs, interleaved (h, w, C) float32 in [0, 1]."""
    rng = SplitMix64(seed ^ 0xB10B5EED)
    s = _size_scale(w, h)
    x = np.arange(w, dtype=np.float64)
    y = np.arange(h, dtype=np.float64)
    img = np.zeros((h, w, channels), np.float64)
    for _ in range(count):
        cx = rng.uniform(0.0, w)
        cy = rng.uniform(0.0, h)
        r = rng.uniform(radius_cells[0], radius_cells[1]) * s
        colour = [rng.uniform() for _ in range(channels)]
        dx = _min_image(x, cx, w)
        dy = _min_image(y, cy, h)
        s2 = 2.0 * r * r
        e = det_exp(-(dy * dy) / s2)[:, None] * det_exp(-(dx * dx) / s2)[None, :]
        for k in range(channels):
            img[..., k] += colour[k] * e
    return np.clip(img, 0.0, 1.0).astype(np.float32)


def initial_state(w: int, h: int, channels: int, seed: int):
    """(vp, tmp, image, itmp) for one simulation: vortex velocity with p = b = 0
    in both velocity buffers, blob image, zeroed image scratch."""
    vp = vortex_field(w, h, seed)
    tmp = np.zeros_like(vp)
    img = blob_image(w, h, channels, seed)
    itmp = np.zeros_like(img)
    return vp, tmp, img, itmp
