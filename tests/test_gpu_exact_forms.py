"""The shortened operations of the bit-faithful FP64 policy on the GPU
(division by a grid-independent constant through its host reciprocal, a
quotient through a shared reciprocal, both with their last rounding step on
the integer pipe, a multiply-add by a power of two, the comparisons on the
integer pipe, 1 - x on the integer pipe, quotients below 2^-1021 rounded on
the integer grid)
against the reference's separately rounded IEEE operations: bit for bit on
2^28 operands per seed wherever their range flag stays set; the operands
include subnormal, tiny, huge and non-finite values and signed zeros, for
which the flag drops and the kernels use the IEEE operations."""
import ctypes
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("exactgpu") / "libexactgpu.so")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                           "-Xcompiler", "-fPIC", "-shared", os.path.join(HERE, "native", "exact_forms_gpu.cu"),
                           "-o", out])
    L = ctypes.CDLL(out)
    L.exact_forms_gpu_check.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]
    return L


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_exact_forms_match_ieee(lib, seed):
    n = 2**28
    out = (ctypes.c_ulonglong * 13)()
    assert lib.exact_forms_gpu_check(seed, n, out) == 0
    bad, fast = list(out[:3]), list(out[3:6])
    assert out[6] == 0, ("comparison mismatches", out[6])
    # the integer rounding step of the divisions, lane by lane
    assert out[7] == 0, ("integer rounding step mismatches", out[7])
    assert out[8] > 0.2 * n, out[8]
    # 1 - x, warp by warp and its integer form lane by lane
    assert out[9] == 0, ("one_minus mismatches", out[9])
    assert 0.4 * n < out[10] < n, out[10]
    # quotients below 2^-1021 rounded on the integer grid, lane by lane (the
    # warp-level division above also meets them mixed with the other paths)
    assert out[11] == 0, ("subnormal quotient mismatches", out[11])
    assert out[12] > 0.02 * n, out[12]
    assert bad == [0, 0, 0], ("divu, divr, fma mismatches with the range flag set", bad)
    # the shortened forms apply to most operands, and not to all of them
    assert all(0.2 * n < f < n for f in fast), fast
