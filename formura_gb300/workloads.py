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
