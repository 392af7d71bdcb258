"""Parity at the configured horizons: the drop-in against the oracle over the
full step counts of the Gray-Scott and HLLC workloads, compared bit for bit
at checkpoints along the way.

* Gray-Scott 4096^2 (Du=2e-5, Dv=1e-5, F=0.04, k=0.06, dx=0.01, dt=1), the
  seeded 10 % square plus noise, 20000 steps: by then v has decayed through
  the subnormal range far from the pattern, and a 1-ulp difference per step
  would have grown to about 3.5e-12 relative L2.
* HLLC Euler 256^3 (gamma 1.4, MUSCL-minmod, CFL 0.4), the seeded smooth
  density and solenoidal Mach-0.3 velocity, 500 steps.

Both sides start from the same seeded state written through the formura_data
hook, and both are driven through their generated C API
(Templates.hs:295-346: Formura_Forward advances the state and the offsets).
The oracle runs with OpenMP on the host cores: about 2.5 and 4 minutes on 16
Grace cores.
"""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import FormuraProgram, builtin_program
from oracle.reference_lib import ReferenceProgram
from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _run_pair(program, cfg, state, checkpoints, spf, tag):
    src, _ = builtin_program(program)
    ref = ReferenceProgram(src, cfg, f"{program}_{tag}_ref")
    gpu = FormuraProgram(src, cfg + f"gpu_steps_per_forward: {spf}\n", program, name=f"{program}_{tag}_gpu")
    assert ref.init() == gpu.init()
    for f in ref.fields:
        ref.set(f, state[f])
        gpu.set(f, state[f])
    done = 0
    for c in checkpoints:
        assert (c - done) % spf == 0
        ref.forward(c - done)
        gpu.forward((c - done) // spf)
        done = c
        assert ref.navi_dict() == gpu.navi_dict(), c
        for f in ref.fields:
            a, b = ref.get(f), gpu.get(f)
            assert bits_equal(a, b), f"step {c}, {f}: rel-L2 {W.rel_l2(b, a)}"
    gpu.finalize()
    return ref


def test_gray_scott_4096_bit_exact_over_20000_steps():
    n = 4096
    cfg = W.gs_config(n)
    src, _ = builtin_program("gs2d")
    # the init function's state (u=1, v=0 with the centred square) comes
    # from Formura_Init; the seeded noise is written on top of it
    probe = ReferenceProgram(src, cfg, "gs2d_horizon_ref")
    probe.init()
    st = W.gs_perturb(probe.get("u"), probe.get("v"), seed=0)
    del probe
    _run_pair("gs2d", cfg, st, [2000, 10000, 20000], 2000, "horizon")


def test_hllc_256_bit_exact_over_500_steps():
    n = 256
    cfg = W.hllc_config(n)
    st = W.hllc_state((n, n, n), seed=0)
    ref = _run_pair("hllc3d", cfg, st, [100, 500], 100, "horizon")
    # mass is conserved by the periodic finite-volume update
    rho0, rho = st["rho"].sum(), ref.get("rho").sum()
    assert abs(rho - rho0) < 1e-9 * abs(rho0)
