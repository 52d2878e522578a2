"""TEST INFRASTRUCTURE ONLY: a numpy restatement of the seeded initial field of the rising
perturbed bubble (128x128x256, walls in z, R 16 at z 48, spherical-harmonic modes l = 2..6),
so that the CPU reference arm of the benchmark can build its input without loading the
solver library.

It follows the solver's own generator (mcb_workload, scenario 2): the same splitmix64
stream, the same mode draws, the same unit-crest normalisation of each real harmonic on a
1-degree grid, and the same tanh profile, phi = 0.5 + 0.5 tanh(2 (R(theta, p) - d) / W).
The reference itself places one unperturbed bubble (src/init.cu:27-49); this scenario is the
benchmark's generalisation of it. tests/test_oracle_cpu.py checks that both generators give
the same float32 field.
"""
from __future__ import annotations

import math

import numpy as np

_MASK = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea and Flood 2014), as the solver's host generator draws it."""

    def __init__(self, state: int):
        self.s = state & _MASK

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & _MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def uniform(self, a: float = 0.0, b: float = 1.0) -> float:
        u = (self.next() >> 11) * (1.0 / 9007199254740992.0)
        return a + (b - a) * u


def _seed_state(scenario: int, case_index: int, seed: int) -> int:
    return (seed * 0x2545F4914F6CDD1D + scenario * 0x9E37 + case_index * 0xD1B54A32D192ED03) & _MASK


def _legendre(l: int, m: int, x):
    """Associated Legendre P_l^m(x), m >= 0, by the three-term recurrence."""
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    pmm = np.ones_like(x)
    for i in range(1, m + 1):
        pmm = pmm * (-(2.0 * i - 1.0) * s)
    if l == m:
        return pmm
    pm1 = x * (2.0 * m + 1.0) * pmm
    if l == m + 1:
        return pm1
    pl = np.zeros_like(x)
    for ll in range(m + 2, l + 1):
        pl = ((2.0 * ll - 1.0) * x * pm1 - (ll + m - 1.0) * pmm) / (ll - m)
        pmm, pm1 = pm1, pl
    return pl


def _ylm(l: int, m: int, t, p):
    leg = _legendre(l, abs(m), np.cos(t))
    return leg * np.cos(m * p) if m >= 0 else leg * np.sin(-m * p)


def _image(d, n):
    h = 0.5 * n
    d = np.where(d > h, d - n, d)
    return np.where(d < -h, d + n, d)


def rising_bubble(seed: int = 1, scale: float = 1.0):
    """(shape (nz, ny, nx), phi float32, parameters) of the rising perturbed bubble."""
    rng = SplitMix64(_seed_state(2, 0, seed))
    scaled = lambda e: max(8, int(math.floor(e * scale + 0.5)))  # std::lround for e*s > 0
    nx, ny, nz = scaled(128), scaled(128), scaled(256)
    width = 4.0
    cx, cy, cz, r0 = 0.5 * (nx - 1), 0.5 * (ny - 1), 48.0 * scale, 16.0 * scale
    a = np.arange(181, dtype=np.float64)[:, None] * math.pi / 180.0
    c = np.arange(360, dtype=np.float64)[None, :] * math.pi / 180.0
    modes = []
    for l in range(2, 7):
        m = int(math.floor(rng.uniform() * (2 * l + 1))) - l
        m = min(m, l)
        amp = rng.uniform(0.0, 0.5) * scale
        mx = float(np.max(np.abs(_ylm(l, m, a, c))))
        modes.append((l, m, amp, 1.0 / mx if mx > 0 else 0.0))
    k = np.arange(nz, dtype=np.float64)[:, None, None]
    j = np.arange(ny, dtype=np.float64)[None, :, None]
    i = np.arange(nx, dtype=np.float64)[None, None, :]
    dx = np.broadcast_to(_image(i - cx, nx), (nz, ny, nx))
    dy = np.broadcast_to(_image(j - cy, ny), (nz, ny, nx))
    dz = np.broadcast_to(k - cz, (nz, ny, nx))
    d = np.sqrt(dx * dx + dy * dy + dz * dz)
    safe = np.where(d > 1e-12, d, 1.0)
    t = np.arccos(np.clip(dz / safe, -1.0, 1.0))
    p = np.arctan2(dy, dx)
    R = np.full(d.shape, r0)
    for l, m, amp, norm in modes:
        R = R + np.where(d > 1e-12, amp * norm * _ylm(l, m, t, p), 0.0)
    phi = (0.5 + 0.5 * np.tanh(2.0 * (R - d) / width)).astype(np.float32)
    params = {"nx": nx, "ny": ny, "nz": nz, "tau": 0.7, "sigma": 0.05, "width": width,
              "gravity": 1e-5, "tau_g": 1.0, "bc": 2}
    return phi, params
