"""Seeded synthetic inputs for the benchmark workloads and the parity tests.

No public dataset is involved: every initial state is generated from a numpy
``default_rng(seed)`` stream and written into ``formura_data`` after
``Formura_Init`` (the user's init hook, as ``examples/pearson2/main.c:13-22``
does), identically for the oracle and the GPU.
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np


def heat_config(n: int = 128, length: float = 1.0, extra: str = "") -> str:
    return f"length_per_node: [{length}, {length}, {length}]\ngrid_per_node: [{n}, {n}, {n}]\nwith_omp: 1\n" + extra


def heat_state(shape: Tuple[int, ...], seed: int = 0) -> Dict[str, np.ndarray]:
    """3D heat: i.i.d. uniform [0, 1)."""
    return {"q": np.random.default_rng(seed).random(shape)}


def gs_config(n: int = 4096, dx: float = 0.01, extra: str = "") -> str:
    length = repr(n * dx)
    return f"length_per_node: [{length}, {length}]\ngrid_per_node: [{n}, {n}]\nwith_omp: 1\n" + extra


def gs_perturb(u: np.ndarray, v: np.ndarray, seed: int = 0) -> Dict[str, np.ndarray]:
    """Gray-Scott: the program's init gives u=1, v=0 outside and u=0.5,
    v=0.25 inside the centred 10% square; add uniform noise in
    [-0.01, 0.01] to both fields."""
    rng = np.random.default_rng(seed)
    return {"u": u + rng.uniform(-0.01, 0.01, u.shape), "v": v + rng.uniform(-0.01, 0.01, v.shape)}


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    nb = float(np.linalg.norm(np.ravel(b)))
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b))) / (nb if nb > 0 else 1.0)


def hllc_config(n: int = 256, length: float = 1.0, extra: str = "") -> str:
    return f"length_per_node: [{length}, {length}, {length}]\ngrid_per_node: [{n}, {n}, {n}]\nwith_omp: 1\n" + extra


def hllc_state(shape: Tuple[int, int, int], seed: int = 0, gamma: float = 1.4,
               mach: float = 0.3, modes: int = 16, kmax: int = 4) -> Dict[str, np.ndarray]:
    """Compressible Euler initial state on the unit periodic box:
    rho = 1 + 0.1 * (sum of `modes` random-phase Fourier modes with
    1 <= |k| <= kmax, scaled to unit peak), p = 1, and a random solenoidal
    velocity (the curl of a random vector potential) scaled so that
    max |v| = mach * c0, c0 = sqrt(gamma * p / 1)."""
    rng = np.random.default_rng(seed)
    axes = [np.arange(n) / n for n in shape]
    X = np.meshgrid(*axes, indexing="ij")

    def random_k():
        while True:
            k = rng.integers(-kmax, kmax + 1, size=3)
            if 1 <= np.sqrt((k * k).sum()) <= kmax:
                return k

    s = np.zeros(shape)
    for _ in range(modes):
        k = random_k()
        s += np.cos(2 * np.pi * (k[0] * X[0] + k[1] * X[1] + k[2] * X[2]) + rng.uniform(0, 2 * np.pi))
    rho = 1.0 + 0.1 * s / np.abs(s).max()
    # velocity = curl A, computed spectrally so that div v = 0 on the grid
    A = []
    for _ in range(3):
        a = np.zeros(shape)
        for _ in range(modes):
            k = random_k()
            a += np.cos(2 * np.pi * (k[0] * X[0] + k[1] * X[1] + k[2] * X[2]) + rng.uniform(0, 2 * np.pi))
        A.append(a)
    kk = np.meshgrid(*[np.fft.fftfreq(n, 1.0 / n) * 2j * np.pi for n in shape], indexing="ij")
    Ah = [np.fft.fftn(a) for a in A]
    v = [np.real(np.fft.ifftn(kk[1] * Ah[2] - kk[2] * Ah[1])),
         np.real(np.fft.ifftn(kk[2] * Ah[0] - kk[0] * Ah[2])),
         np.real(np.fft.ifftn(kk[0] * Ah[1] - kk[1] * Ah[0]))]
    vmax = np.sqrt(v[0] ** 2 + v[1] ** 2 + v[2] ** 2).max()
    c0 = np.sqrt(gamma * 1.0 / 1.0)
    v = [x * (mach * c0 / vmax) for x in v]
    p = np.ones(shape)
    e = p / (gamma - 1.0) + 0.5 * rho * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
    return {"rho": rho, "mx": rho * v[0], "my": rho * v[1], "mz": rho * v[2], "e": e}
