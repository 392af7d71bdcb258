"""Error behaviour of the C ABI on a GPU: every bad request comes back as a
status code with a message (fgb_last_error), the grid stays usable, and no
call falls back to the host."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import FgbError, Grid, Library, builtin_program, program_uniforms

pytestmark = pytest.mark.gpu


def _gs_uniforms(n=64):
    src, _ = builtin_program("gs2d")
    return program_uniforms(src, W.gs_config(n), "gs2d")[1]


def test_unknown_program():
    with pytest.raises(FgbError, match="unknown program"):
        Library.get().query("no_such_program")


def test_bad_open_arguments():
    U = _gs_uniforms()
    with pytest.raises(FgbError, match="2-dimensional"):
        Grid("gs2d", (64, 64, 64), "f64", U)
    with pytest.raises(FgbError, match="uniform values"):
        Grid("gs2d", (64, 64), "f64", U[:-1])
    with pytest.raises(FgbError, match="points away"):
        Grid("hllc3d", (1, 16, 16), "f64", [0.0] * Library.get().query("hllc3d")["nuniforms"])


def test_bad_variant_and_recovery():
    U = _gs_uniforms()
    g = Grid("gs2d", (64, 64), "f32", U)
    x = np.stack([np.ones((64, 64)), np.zeros((64, 64))])
    g.upload(x)
    with pytest.raises(FgbError, match="no such variant"):
        g.set_variant(len(g.variants()) + 3)
    g.forward(3)                       # the grid still works after the error
    assert np.isfinite(g.download()).all()
    g.close()


def test_adjoint_missing_for_program_without_one():
    info = Library.get().query("hlld3d")
    g = Grid("hlld3d", (8, 8, 8), "f64", [1.0] * info["nuniforms"])
    with pytest.raises(FgbError, match="no adjoint"):
        g.backward(np.zeros((info["nfields"], 8, 8, 8)))
    g.close()


def test_adjoint_missing_in_fp16():
    U = _gs_uniforms()
    g = Grid("gs2d", (64, 64), "f16", U, scales=[1.0, 1.0])
    with pytest.raises(FgbError, match="no adjoint"):
        g.backward(np.zeros((2, 64, 64)))
    g.close()


def test_bounded_wait_runs_out_and_is_reported():
    """A kernel's wait on an mbarrier phase that nothing completes runs out
    after its poll limit (the library's fgb::mbar_wait_bounded); the kernel
    raises the grid's error word and returns.  The host then gets an error
    status with a message from fgb_synchronize, the context stays usable, and
    the same grid steps correctly afterwards.  Nothing faults and nothing is
    left in flight: the test kernel issues no copies."""
    import ctypes
    import os
    import subprocess
    import tempfile
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "formura_gb300", "csrc")
    so = os.path.join(tempfile.mkdtemp(), "libboundedwait.so")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                           "-Xcompiler", "-fPIC", "-shared", "-I", csrc,
                           os.path.join(here, "native", "bounded_wait.cu"), "-o", so])
    T = ctypes.CDLL(so)
    T.bounded_wait_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_float)]
    lib = Library.get().lib
    lib.fgb_internal_error_word.argtypes = [ctypes.c_void_p]
    lib.fgb_internal_error_word.restype = ctypes.c_void_p

    U = _gs_uniforms()
    x = W.gs_perturb(np.ones((64, 64)), np.zeros((64, 64)), seed=4)
    x = np.stack([x["u"], x["v"]])
    g = Grid("gs2d", (64, 64), "f64", U)
    g.upload(x)
    g.forward(5)
    expect = g.download()
    g.upload(x)
    word = lib.fgb_internal_error_word(g.h)
    assert word

    stored, ms = ctypes.c_int(), ctypes.c_float()
    # the phase completes: every block stores, the word stays clear
    assert T.bounded_wait_run(1, 8, word, ctypes.byref(stored), ctypes.byref(ms)) == 0
    assert stored.value == 8
    g.synchronize()
    # nothing completes the phase: every wait runs out, no block stores
    assert T.bounded_wait_run(0, 8, word, ctypes.byref(stored), ctypes.byref(ms)) == 0
    assert stored.value == 0
    assert ms.value < 60e3, f"the bounded wait took {ms.value} ms"
    with pytest.raises(FgbError, match="wait for its TMA load ran out"):
        g.synchronize()
    # reported once; the context and the grid still work
    g.synchronize()
    g.forward(5)
    assert np.array_equal(g.download(), expect)
    g.close()
    print(f"bounded wait ran out after {ms.value:.1f} ms")
