"""Driver programs run as executables on the GB300 pair and on the oracle
pair: their output files must be byte-identical.

* The driver in tests/native/driver_main.c (written against the generated
  API only: Formura_Init, writes into formura_data after Init and between
  calls, Formura_Forward until T_MAX, to_pos_x and the navigator in the
  output, Formura_Finalize) on the shipped programs.
* The reference's own example and sample drivers, unchanged, when a
  reference checkout is available (FORMURA_REFERENCE); skipped otherwise.
"""
import os

import pytest

from conftest import REFERENCE
import driver_pairs as DP

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _own_case(program, n):
    from formura_gb300 import workloads as W
    from formura_gb300.host import builtin_program
    src, _ = builtin_program(program)
    cfg = {"gs2d": W.gs_config, "heat3d": W.heat_config, "hllc3d": W.hllc_config}[program](n)
    return src, cfg


@pytest.mark.parametrize("program,n,t_max,t_out", [("gs2d", 64, 60, 20), ("heat3d", 16, 30, 10),
                                                   ("hllc3d", 16, 12, 4)])
def test_own_driver_outputs_identical(tmp_path, program, n, t_max, t_out):
    src, cfg = _own_case(program, n)
    main_c = os.path.join(HERE, "native", "driver_main.c")
    flags = [f'-DPAIR_HEADER="{program}.h"', f"-DT_MAX={t_max}", f"-DT_OUT={t_out}"]
    gdir, odir = str(tmp_path / "gpu"), str(tmp_path / "oracle")
    lib = DP.gpu_pair(gdir, program, src, cfg)
    gpu = DP.run(DP.link(main_c, gdir, program, lib, flags), str(tmp_path / "run_gpu"))
    DP.oracle_pair(odir, program, src, cfg)
    ref = DP.run(DP.link(main_c, odir, program, None, flags), str(tmp_path / "run_oracle"))
    assert len(ref) == t_max // t_out + 1
    assert gpu == ref


def _reference_drivers():
    if not os.path.isdir(REFERENCE):
        return []
    from test_drivers import DRIVERS
    return sorted(k for k, v in DRIVERS.items() if v[4])


@pytest.mark.parametrize("name", _reference_drivers() or ["(no reference checkout)"])
def test_reference_driver_outputs_identical(tmp_path, name):
    if not os.path.isdir(REFERENCE):
        pytest.skip("the reference tree is not present")
    from test_drivers import driver_sources
    main_c, base, src, cfg = driver_sources(name)
    gdir, odir = str(tmp_path / "gpu"), str(tmp_path / "oracle")
    lib = DP.gpu_pair(gdir, base, src, cfg)
    gpu = DP.run(DP.link(main_c, gdir, base, lib), str(tmp_path / "run_gpu"))
    DP.oracle_pair(odir, base, src, cfg)
    ref = DP.run(DP.link(main_c, odir, base), str(tmp_path / "run_oracle"))
    assert ref and gpu == ref
