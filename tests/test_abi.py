"""The C ABI library builds for sm_103a, loads, and exports every entry
point that include/formura_gb300.h declares (no compute calls: no GPU here)."""
import ctypes
import os
import re

import pytest

from formura_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "formura_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fgb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    path = B.build()
    return ctypes.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s


def test_program_registry_without_gpu(lib):
    lib.fgb_program_name.restype = ctypes.c_char_p
    names = {lib.fgb_program_name(i).decode() for i in range(lib.fgb_program_count())}
    assert {"heat3d", "gs2d"} <= names
    dim, nf, nu, s, sh = (ctypes.c_int() for _ in range(5))
    rc = lib.fgb_program_query(b"gs2d", ctypes.byref(dim), ctypes.byref(nf), ctypes.byref(nu),
                               ctypes.byref(s), ctypes.byref(sh))
    assert rc == 0 and dim.value == 2 and nf.value == 2 and s.value == 1 and sh.value == 1
    assert lib.fgb_program_query(b"nope", None, None, None, None, None) == -2


def test_open_errors_are_reported_not_fatal(lib):
    lib.fgb_last_error.restype = ctypes.c_char_p
    h = ctypes.c_void_p()
    shape = (ctypes.c_int * 2)(64, 64)
    # wrong dimension count is rejected before any device call
    rc = lib.fgb_open(b"gs2d", shape, 3, 0, None, 0, ctypes.byref(h))
    assert rc == -1 and b"dimensional" in lib.fgb_last_error()
    rc = lib.fgb_open(b"gs2d", shape, 2, 9, None, 0, ctypes.byref(h))
    assert rc == -1


def test_noalloc_rejects_grids_beyond_32bit_indexing(lib):
    """fgb_forward_noalloc applies fgb_open's size limit before it touches
    any pointer or the device: 1300^3 points exceed the 2^31 cells that the
    stage kernels' 32-bit indices cover, even though one step of heat3d
    would need scratch only for its uniform table."""
    lib.fgb_last_error.restype = ctypes.c_char_p
    fn = lib.fgb_forward_noalloc
    fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_int, ctypes.c_void_p]
    nu = ctypes.c_int()
    assert lib.fgb_program_query(b"heat3d", None, None, ctypes.byref(nu), None, None) == 0
    u = (ctypes.c_double * max(1, nu.value))(*([0.1] * max(1, nu.value)))
    shape = (ctypes.c_int * 3)(1300, 1300, 1300)
    # fake, never dereferenced device addresses far apart
    rc = fn(b"heat3d", shape, 3, 0, u, nu.value, ctypes.c_void_p(1 << 40), ctypes.c_void_p(1 << 44), 1, None)
    assert rc == -1 and b"larger than this build supports" in lib.fgb_last_error()
