"""The integer-pipe binary64 operations (formura_gb300/csrc/fgb_softf64.h),
compiled for the host, against the host's IEEE 754 arithmetic: wherever the
fast path applies the result must be bit-identical to the correctly rounded
sum or product.  The inputs stress cancellation, exact ties, carries out of
rounding, exponent gaps across the sticky range, signed zeros, subnormal
operands and the ends of the fast-path exponent window."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "softf64_harness.cpp")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("softf64") / "libsoftf64.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", SRC, "-o", out])
    L = ctypes.CDLL(out)
    P = ctypes.POINTER(ctypes.c_double)
    B = ctypes.POINTER(ctypes.c_ubyte)
    for name in ("soft_add", "soft_sub", "soft_mul"):
        getattr(L, name).argtypes = [P, P, P, B, ctypes.c_long]
    L.soft_scaled_add.argtypes = [P, P, P, B, ctypes.c_long, ctypes.c_int, ctypes.c_int]
    return L


def _call(L, name, a, b, *extra):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    r = np.empty_like(a)
    fast = np.zeros(a.shape, dtype=np.uint8)
    P = ctypes.POINTER(ctypes.c_double)
    B = ctypes.POINTER(ctypes.c_ubyte)
    getattr(L, name)(a.ctypes.data_as(P), b.ctypes.data_as(P), r.ctypes.data_as(P), fast.ctypes.data_as(B),
                     a.size, *extra)
    return r, fast.astype(bool)


def _from_parts(sign, exp, mant):
    bits = (sign.astype(np.uint64) << np.uint64(63)) | (exp.astype(np.uint64) << np.uint64(52)) | \
        (mant.astype(np.uint64) & np.uint64(0x000FFFFFFFFFFFFF))
    return bits.view(np.float64)


def _sparse_mant(rng, n, bits=4):
    """Mantissas with few set bits: sums and products are often exact or
    exact ties."""
    m = np.zeros(n, dtype=np.uint64)
    for _ in range(bits):
        m |= np.uint64(1) << rng.integers(0, 52, n).astype(np.uint64)
    return m


def _operands(seed, n):
    rng = np.random.default_rng(seed)
    cases = []
    # 1. random bit patterns (every exponent, NaN and infinity included)
    cases.append((rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64),
                  rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64)))
    # 2. nearby exponents, both signs: cancellation and sticky
    ea = rng.integers(60, 2000, n)
    eb = np.clip(ea + rng.integers(-70, 71, n), 0, 2046)
    cases.append((_from_parts(rng.integers(0, 2, n), ea, rng.integers(0, 2**52, n, dtype=np.uint64)),
                  _from_parts(rng.integers(0, 2, n), eb, rng.integers(0, 2**52, n, dtype=np.uint64))))
    # 3. sparse mantissas: exact results and exact ties
    ea = rng.integers(900, 1100, n)
    eb = np.clip(ea + rng.integers(-56, 57, n), 1, 2046)
    cases.append((_from_parts(rng.integers(0, 2, n), ea, _sparse_mant(rng, n)),
                  _from_parts(rng.integers(0, 2, n), eb, _sparse_mant(rng, n))))
    # 4. all-ones mantissas: carries out of the rounding
    ones = np.full(n, 2**52 - 1, dtype=np.uint64) ^ (np.uint64(1) << rng.integers(0, 8, n).astype(np.uint64))
    cases.append((_from_parts(np.zeros(n, int), ea, ones),
                  _from_parts(rng.integers(0, 2, n), ea - rng.integers(0, 60, n), _sparse_mant(rng, n, 2))))
    # 5. the ends of the fast-path window and subnormal / zero operands
    edge = np.array([0, 1, 2, 3, 62, 63, 64, 65, 1022, 1023, 1024, 2043, 2044, 2045, 2046])
    ea = rng.choice(edge, n)
    eb = rng.choice(edge, n)
    cases.append((_from_parts(rng.integers(0, 2, n), ea, rng.integers(0, 2**52, n, dtype=np.uint64) * (ea > 0)),
                  _from_parts(rng.integers(0, 2, n), eb, _sparse_mant(rng, n) * rng.integers(0, 2, n).astype(np.uint64))))
    # 6. values of a stencil: O(1) numbers and their neighbours
    x = rng.random(n)
    cases.append((x, -x * (1 + rng.integers(-4, 5, n) * 2.0**-52)))
    return cases


def _check(got, fast, want, min_fast):
    g = got.view(np.uint64)[fast]
    w = want.view(np.uint64)[fast]
    bad = np.nonzero(g != w)[0]
    assert bad.size == 0, f"{bad.size} mismatches"
    assert fast.mean() >= min_fast, fast.mean()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_add_sub_bitwise(lib, seed):
    with np.errstate(all="ignore"):
        for i, (a, b) in enumerate(_operands(seed, 200_000)):
            r, f = _call(lib, "soft_add", a, b)
            _check(r, f, a + b, 0.3 if i in (0, 4) else 0.97)
            r, f = _call(lib, "soft_sub", a, b)
            _check(r, f, a - b, 0.3 if i in (0, 4) else 0.97)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_mul_bitwise(lib, seed):
    rng = np.random.default_rng(100 + seed)
    with np.errstate(all="ignore"):
        for i, (a, b) in enumerate(_operands(seed, 200_000)):
            if i in (1, 3):
                # bring b to [2^-300, 2^300] so that most products stay normal
                b = np.ldexp(np.frexp(b)[0], rng.integers(-300, 300, b.size))
            r, f = _call(lib, "soft_mul", a, b)
            _check(r, f, a * b, {0: 0.5, 1: 0.6, 3: 0.6, 4: 0.3}.get(i, 0.97))


def test_mul_exact_ties(lib):
    """Products of two 27-bit significands are exact in 54 bits: the last bit
    decides a tie, both ways."""
    rng = np.random.default_rng(7)
    n = 200_000
    ma = (rng.integers(2**26, 2**27, n) | 1).astype(np.float64)
    mb = (rng.integers(2**26, 2**27, n) | 1).astype(np.float64)
    a = ma * 2.0 ** rng.integers(-400, 400, n)
    b = mb * 2.0 ** rng.integers(-400, 400, n) * rng.choice([-1.0, 1.0], n)
    r, f = _call(lib, "soft_mul", a, b)
    _check(r, f, a * b, 1.0)


@pytest.mark.parametrize("k,negate", [(1, 1), (1, 0), (-1, 0), (2, 1), (-2, 1), (0, 1), (5, 0), (-7, 1)])
def test_scaled_add_bitwise(lib, k, negate):
    c = (-1.0 if negate else 1.0) * 2.0 ** k
    with np.errstate(all="ignore"):
        for i, (h, t) in enumerate(_operands(11 + k, 100_000)):
            r, f = _call(lib, "soft_scaled_add", h, t, k, negate)
            _check(r, f, c * h + t, 0.3 if i in (0, 4) else 0.9)


def test_signed_zeros(lib):
    z = np.array([0.0, -0.0, 0.0, -0.0, 1.5, -1.5, 0.0, -0.0])
    w = np.array([0.0, 0.0, -0.0, -0.0, -1.5, 1.5, 2.0, 3.0])
    r, f = _call(lib, "soft_add", z, w)
    assert f.all()
    assert np.array_equal(r.view(np.uint64), (z + w).view(np.uint64))
    r, f = _call(lib, "soft_mul", z, w)
    assert f[:4].all() and f[6:].all()
    assert np.array_equal(r.view(np.uint64)[f], (z * w).view(np.uint64)[f])
