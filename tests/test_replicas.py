"""The N > 1 path of bench.py ("replicas only": one independent grid per
rank, no data-path collective), on CPU with the gloo backend and
world_size 2: the timed region is the slowest rank's, the rate is the whole
job's, and the reference arm runs on rank 0 alone."""
import io
import json
import os
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    got = bench.max_over_ranks(ms, ws, "cpu")
    out[rank] = (got, bench.whole_job_rate(1000, 10, got, ws))
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    ws = 2
    port = 29500 + os.getpid() % 2000
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
        res = dict(out)
    for r in range(ws):
        ms, rate = res[r]
        assert ms == 150.0
        assert rate == pytest.approx(2 * 1000 * 10 / 0.150 / 1e9)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    spec = bench.workload_spec("gs2d")

    class Args:
        warmup, steps, spf = 1, 1, 1000

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args, spec)
    assert buf.getvalue() == ""


def test_reference_arm_line_on_a_small_grid(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.setenv("RANK", "0")
    from formura_gb300 import workloads as W
    spec = bench.workload_spec("gs2d")
    # 64 + 2*1*4 = 72 = 2 blocks of 36 per axis
    spec.update(cfg=W.gs_config(64), shape=(64, 64), cpu_tb=[(4, 36)])

    class Args:
        warmup, steps, spf = 1, 3, 8

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args, spec)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GLUP/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert sorted(line["config"]["probed_configs_GLUPs"]) == ["NoBlocking",
                                                              "TemporalBlocking nt=4 grid_per_block=36"]
    # a bench step is spf time steps on both arms, whichever blocking wins
    assert line["config"]["time_steps_per_bench_step"] == 8
    assert line["config"]["timed_time_steps"].startswith("0..24")


@pytest.mark.parametrize("name", ["gs2d", "heat3d", "hllc3d", "hlld3d"])
def test_cpu_configs_of_the_workloads_are_valid(name):
    """Every temporal-blocking candidate of the CPU legs satisfies the
    reference's divisibility rule for its workload's grid and sleeve."""
    from formura_gb300.generator.config import decode_config
    from formura_gb300.generator.manifest import compile_program
    from formura_gb300.host import builtin_program
    spec = bench.workload_spec(name)
    src, _ = builtin_program(spec["program"])
    cfgs = bench.oracle_configs(spec)
    assert len(cfgs) == 1 + len(spec["cpu_tb"]) >= 2
    for label, _, cfg in cfgs:
        blocking = compile_program(src, decode_config(cfg)).om.config.blocking
        assert blocking.temporal == (label != "NoBlocking"), label
