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


def gaussians_3d(shape: Tuple[int, int, int], seed: int, count: int = 32,
                 wmin: float = 4.0, wmax: float = 16.0) -> np.ndarray:
    """Smooth periodic field: a sum of `count` Gaussians with random centres,
    widths uniform in [wmin, wmax] cells and amplitudes N(0, 1)."""
    rng = np.random.default_rng(seed)
    idx = [np.arange(n, dtype=np.float64) for n in shape]
    out = np.zeros(shape)
    for _ in range(count):
        c = [rng.uniform(0, n) for n in shape]
        w = rng.uniform(wmin, wmax)
        amp = rng.normal()
        g = 1.0
        parts = []
        for ax, n in enumerate(shape):
            d = np.abs(idx[ax] - c[ax])
            d = np.minimum(d, n - d)                 # periodic distance
            parts.append(np.exp(-0.5 * (d / w) ** 2))
        out += amp * parts[0][:, None, None] * parts[1][None, :, None] * parts[2][None, None, :]
    return out


def ensemble(count: int = 256, seed: int = 0, nmin: int = 64, nmax: int = 1024):
    """Gray-Scott ensemble: side lengths log-uniform in [nmin, nmax], feed
    rate F ~ U[0.02, 0.06] and kill rate k ~ U[0.05, 0.065] per grid."""
    rng = np.random.default_rng(seed)
    sides = np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), count))).astype(int)
    F = rng.uniform(0.02, 0.06, count)
    k = rng.uniform(0.05, 0.065, count)
    return [(int(n), float(f), float(kk)) for n, f, kk in zip(sides, F, k)]


def gs_square_state(n: int, seed: int) -> np.ndarray:
    """Gray-Scott initial state of an n x n grid: u = 1, v = 0 outside and
    u = 0.5, v = 0.25 inside the centred 10% square, plus uniform noise in
    [-0.01, 0.01] on both fields."""
    i = np.arange(n)
    inside = (i > 0.45 * n) & (i < 0.55 * n)
    sq = inside[:, None] & inside[None, :]
    st = gs_perturb(np.where(sq, 0.5, 1.0), np.where(sq, 0.25, 0.0), seed)
    return np.stack([st["u"], st["v"]])


def mhd_config(n: int = 64, length: float = 1.0, extra: str = "") -> str:
    return hllc_config(n, length, extra)


def mhd_state(shape: Tuple[int, int, int], seed: int = 0) -> Dict[str, np.ndarray]:
    """Ideal-MHD initial state: the compressible Euler state of hllc_state
    plus a magnetic field B = (0.3, 0, 0) + 0.05 * N(0, 1) per component,
    psi = 0, and the magnetic energy added to e."""
    st = hllc_state(shape, seed)
    rng = np.random.default_rng(seed + 7919)
    b = {"bx": 0.3 + 0.05 * rng.standard_normal(shape), "by": 0.05 * rng.standard_normal(shape),
         "bz": 0.05 * rng.standard_normal(shape), "psi": np.zeros(shape)}
    st["e"] = st["e"] + 0.5 * (b["bx"] ** 2 + b["by"] ** 2 + b["bz"] ** 2)
    st.update(b)
    return st
