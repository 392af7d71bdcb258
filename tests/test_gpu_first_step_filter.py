"""first_step and filter functions on the GPU (Templates.hs:250-270, 305-309,
329-333): applied by the drop-in exactly where the reference applies them,
with their own roll; bit-exact against the oracle, without and with
temporal blocking."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import FormuraProgram, builtin_program
from oracle.reference_lib import ReferenceProgram
from conftest import bits_equal

pytestmark = pytest.mark.gpu

BASE = "length_per_node: [1.0, 1.0]\ngrid_per_node: [64, 64]\nfilter_interval: 3\n"
TB = "grid_per_block: [14, 14]\ntemporal_blocking_interval: 3\n"


@pytest.mark.parametrize("extra,calls,tag", [("", 10, "nb"), (TB, 4, "tb")])
def test_first_step_and_filter_bit_exact(extra, calls, tag):
    src, _ = builtin_program("smooth2d")
    cfg = BASE + extra
    ref = ReferenceProgram(src, cfg, f"smooth_{tag}_ref")
    gpu = FormuraProgram(src, cfg, "smooth2d", name=f"smooth_{tag}_gpu")
    a, b = ref.init(), gpu.init()
    assert a == b
    assert bits_equal(ref.get("q"), gpu.get("q"))        # first_step applied in Init
    x = ref.get("q") + 0.01 * np.random.default_rng(4).standard_normal((64, 64))
    ref.set("q", x)
    gpu.set("q", x)
    for _ in range(calls):
        assert ref.forward(1) == gpu.forward(1)
        assert bits_equal(ref.get("q"), gpu.get("q"))
    gpu.finalize()
