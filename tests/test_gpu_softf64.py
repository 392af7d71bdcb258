"""The integer-pipe binary64 operations on the GPU against the hardware's
__dadd_rn / __dsub_rn / __dmul_rn / __fma_rn: zero mismatches over 2^31
counter-generated operand pairs per seed, wherever the fast path applies."""
import ctypes
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("softgpu") / "libsoftgpu.so")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                           "-Xcompiler", "-fPIC", "-shared", os.path.join(HERE, "native", "softf64_gpu.cu"),
                           "-o", out])
    L = ctypes.CDLL(out)
    L.softf64_gpu_check.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]
    return L


@pytest.mark.parametrize("seed", [1, 2])
def test_soft_ops_match_hardware(lib, seed):
    n = 2**31
    out = (ctypes.c_ulonglong * 8)()
    assert lib.softf64_gpu_check(seed, n, out) == 0
    bad, fast = list(out[:4]), list(out[4:])
    assert bad == [0, 0, 0, 0], (bad, fast)
    # the fast path covers most operands of every kind
    assert all(f > 0.6 * n for f in fast), fast
