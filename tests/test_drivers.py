"""The drop-in boundary on the CPU: the reference's own driver programs
(examples/*/main.c, sample/*/main.c) compile and link unchanged against the
C pair this backend generates, and that pair's header is the reference
generator's header byte for byte (Encode.hs:11-20, Templates.hs:53-115).

Each driver is built twice from its own .fmr, with a one-rank config (no
MPI shape; small grids where the sample's is large):
* against the GB300 pair (generator command with --lib: X.c, X.h and the
  program's kernel library); it links here, and runs on a GPU in
  test_gpu_drivers.py;
* against the oracle pair, built with OpenMP and run here: the deterministic
  drivers must write their data files.
These tests read the reference checkout and skip without it.
"""
import os

import pytest

from conftest import REFERENCE
import driver_pairs as DP

# driver: (folder, program file, grid for the one-rank config or None, deterministic)
DRIVERS = {
    "diffusion1": ("examples/diffusion1", "diffusion1.fmr", "diffusion1.yaml", None, True),
    "diffusion2": ("examples/diffusion2", "diffusion2.fmr", "diffusion2.yaml", "[32, 32]", True),
    "diffusion3": ("examples/diffusion3", "diffusion3.fmr", "diffusion3.yaml", "[16, 16, 16]", True),
    "pearson2": ("examples/pearson2", "pearson2.fmr", "pearson2.yaml", "[64, 64]", False),
    "1d_hllc": ("sample/1d_hllc", "hllc.fmr", "config.yaml", None, True),
    "3d_hllc": ("sample/3d_hllc", "3d_hllc.fmr", "config.yaml", None, True),
    "mhd_1d_hlld": ("sample/mhd_1d_hlld", "mhd_hlld.fmr", "config.yaml", None, True),
    "mhd_3d_hlld": ("sample/mhd_3d_hlld", "mhd_3d_hlld.fmr", "config.yaml", "[20, 20, 5]", True),
}


def driver_sources(name):
    folder, fmr, yml, grid, _ = DRIVERS[name]
    with open(os.path.join(REFERENCE, folder, fmr)) as f:
        src = f.read()
    with open(os.path.join(REFERENCE, folder, yml)) as f:
        cfg = DP.one_rank_config(f.read(), grid)
    return os.path.join(REFERENCE, folder, "main.c"), os.path.splitext(fmr)[0], src, cfg


@pytest.fixture(autouse=True)
def _needs_reference():
    if not os.path.isdir(REFERENCE):
        pytest.skip("the reference tree is not present")


@pytest.mark.parametrize("name", sorted(DRIVERS))
def test_reference_driver_links_unchanged(tmp_path, name):
    main_c, base, src, cfg = driver_sources(name)
    gdir, odir = str(tmp_path / "gpu"), str(tmp_path / "oracle")
    program = DP.gpu_pair(gdir, base, src, cfg)
    exe = DP.link(main_c, gdir, base, program)
    assert os.path.exists(exe)
    DP.oracle_pair(odir, base, src, cfg)
    # the generated header is the reference generator's, byte for byte
    with open(os.path.join(gdir, base + ".h")) as f, open(os.path.join(odir, base + ".h")) as g:
        assert f.read() == g.read()
    if DRIVERS[name][4]:
        exe = DP.link(main_c, odir, base)
        out = DP.run(exe, str(tmp_path / "run_oracle"))
        assert out, "the driver wrote no data files"


def test_own_driver_builds_against_both_pairs(tmp_path):
    """The driver used by the GPU test (tests/native/driver_main.c) builds
    against a shipped program's GB300 pair and runs against its oracle pair."""
    from formura_gb300 import workloads as W
    from formura_gb300.host import builtin_program
    src, _ = builtin_program("gs2d")
    cfg = W.gs_config(32)
    main_c = os.path.join(os.path.dirname(os.path.abspath(__file__)), "native", "driver_main.c")
    flags = ['-DPAIR_HEADER="gs2d.h"', "-DT_MAX=20", "-DT_OUT=5"]
    program = DP.gpu_pair(str(tmp_path / "gpu"), "gs2d", src, cfg)
    DP.link(main_c, str(tmp_path / "gpu"), "gs2d", program, flags)
    DP.oracle_pair(str(tmp_path / "oracle"), "gs2d", src, cfg)
    out = DP.run(DP.link(main_c, str(tmp_path / "oracle"), "gs2d", None, flags), str(tmp_path / "run"))
    assert sorted(out) == ["0.dat", "10.dat", "15.dat", "20.dat", "5.dat"]
