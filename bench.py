"""Benchmark of the Formura_Forward hot path on GB300.

Workload (default): 2D Gray-Scott on a 4096^2 periodic grid, Du=2e-5,
Dv=1e-5, F=0.04, k=0.06, dx=0.01, dt=1, 20000 steps, FP64, seeded synthetic
initial state.  A bench "step" is one Formura_Forward-sized chunk of
``--spf`` time steps (default 100), so the default ``--steps 200`` covers the
configured 20000 time steps.

value  : GLUP/s (cells x time steps / s) with the state resident in HBM,
         device time by CUDA events on the grid's stream.
e2e    : the same metric through the drop-in C API (Formura_Forward with the
         host formura_data uploaded and downloaded on every call).
--impl reference : the oracle (the reference generator's C, restated and
         compiled with gcc -O3 -fopenmp) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits"],
                                         capture_output=True, text=True, timeout=5).stdout.strip()
                    if out:
                        self.samples.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for nm, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_spec(name: str):
    from formura_gb300 import workloads as W
    if name == "gs2d":
        n = 4096
        return {"program": "gs2d", "cfg": W.gs_config(n), "shape": (n, n), "fields": 2,
                "steps_total": 20000,
                "label": "gray-scott-2d 4096^2 periodic, Du=2e-5 Dv=1e-5 F=0.04 k=0.06 dx=0.01 dt=1, 20000 steps"}
    if name == "heat3d":
        n = 128
        return {"program": "heat3d", "cfg": W.heat_config(n), "shape": (n, n, n), "fields": 1,
                "steps_total": 1000,
                "label": "heat-3d 128^3 periodic, D*dt/dx^2=0.1, 1000 steps"}
    raise SystemExit(f"unknown workload {name}")


def initial_state(spec, prog):
    """Seeded initial state written through the init hook."""
    import numpy as np
    from formura_gb300 import workloads as W
    if spec["program"] == "gs2d":
        st = W.gs_perturb(prog.get("u"), prog.get("v"), seed=0)
        return np.stack([st["u"], st["v"]])
    return W.heat_state(spec["shape"], seed=0)["q"][None]


def run_reference(args, spec):
    """The oracle on the host cores: one bench step = one Formura_Forward
    call of the reference's generated C (one time step, NoBlocking)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from formura_gb300.host import builtin_program
    from oracle.reference_lib import ReferenceProgram
    src, _ = builtin_program(spec["program"])
    ref = ReferenceProgram(src, spec["cfg"], f"{spec['program']}_bench_ref")
    ref.init()
    st = initial_state(spec, ref)
    for i, f in enumerate(ref.fields):
        ref.set(f, st[i])
    for _ in range(args.warmup):
        ref.forward(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ref.forward(1)
    dt = time.perf_counter() - t0
    cells = 1
    for x in spec["shape"]:
        cells *= x
    v = cells * args.steps / dt / 1e9
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"metric": "GLUP/s", "value": v, "unit": "GLUP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": spec["label"], "time_steps_per_bench_step": 1,
                       "implementation": "oracle: reference generator's C (restated), gcc -O3 -fopenmp "
                                         "-ffp-contract=off, NoBlocking, 1 rank"},
            "cpu_baseline": {"value": v, "unit": "GLUP/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} time steps of the full grid after {args.warmup} warm-up steps"},
            "e2e": {"value": v, "unit": "GLUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def load_traffic(spec, precision):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(f"{spec['program']}:{precision}")


def storage_bytes(precision):
    return {"f64": 8, "f64fast": 8, "f32": 4, "f16": 2}[precision]


def time_grid(grid, spf, warmup, steps, torch, stream):
    for _ in range(warmup):
        grid.forward(spf)
    grid.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    l0 = grid.launches
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        grid.forward(spf)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), grid.launches - l0


def run_ours(args, spec):
    import numpy as np
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from formura_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from formura_gb300 import workloads as W
    from formura_gb300.host import FormuraProgram, Grid, builtin_program, program_uniforms

    src, _ = builtin_program(spec["program"])
    cells = 1
    for x in spec["shape"]:
        cells *= x
    nf = spec["fields"]
    spf = args.spf
    # initial state through the drop-in's Formura_Init (host init function)
    dp = FormuraProgram(src, spec["cfg"] + f"gpu_steps_per_forward: {spf}\n", spec["program"],
                        name=f"{spec['program']}_bench_e2e_{local}")
    dp.init()
    st0 = initial_state(spec, dp)
    for i, f in enumerate(dp.fields):
        dp.set(f, st0[i])
    _, U = program_uniforms(src, spec["cfg"], spec["program"])

    def open_grid(prec):
        sc = None
        if prec == "f16":
            sc = [float(max(1e-3, np.abs(st0[i]).max())) for i in range(nf)]
        g = Grid(spec["program"], spec["shape"], prec, U, scales=sc)
        g.upload(st0)
        return g

    g = open_grid(args.precision)
    stream = torch.cuda.ExternalStream(g.stream)
    sampler = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    sampler.start()
    ms, launches = time_grid(g, spf, args.warmup, args.steps, torch, stream)
    clocks = sampler.stop()
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    final64 = g.download()
    tsteps = args.steps * spf
    value = ws * cells * tsteps / (ms / 1e3) / 1e9

    # roofline of the dominant (only) kernel: one stage launch per time step
    per_launch_ms = ms / max(1, launches)
    bytes_per_launch = 2 * nf * storage_bytes(args.precision) * cells
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": load_traffic(spec, args.precision),
                "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_us": per_launch_ms * 1e3}

    # end to end through the drop-in C API: upload + spf steps + download per call
    for _ in range(2):
        dp.forward(1)
    t0 = time.perf_counter()
    e2e_calls = max(1, min(args.steps, args.e2e_steps))
    for _ in range(e2e_calls):
        dp.forward(1)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": ws * cells * e2e_calls * spf / e2e_s / 1e9, "unit": "GLUP/s",
           "h2d_bytes_per_step": nf * cells * 8, "d2h_bytes_per_step": nf * cells * 8,
           "steps": e2e_calls, "api": "Formura_Forward (drop-in C API, formura_data on the host)"}
    launches_e2e = 0

    variants = {}
    if rank == 0 and not args.no_variants and args.precision == "f64":
        for prec in ("f32", "f16"):
            gv = open_grid(prec)
            sv = torch.cuda.ExternalStream(gv.stream)
            vms, _ = time_grid(gv, spf, args.warmup, args.steps, torch, sv)
            fin = gv.download()
            errs = {f: W.rel_l2(fin[i], final64[i]) for i, f in enumerate(dp.fields)}
            variants[prec] = {"value": cells * tsteps / (vms / 1e3) / 1e9, "unit": "GLUP/s",
                              "speedup_vs_f64": (cells * tsteps / (vms / 1e3) / 1e9) / value * ws,
                              "rel_l2_vs_f64_oracle": errs,
                              "time_steps": (args.warmup + args.steps) * spf}
            gv.close()

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(spec, args)

    if rank == 0:
        line = {"metric": "GLUP/s", "value": value, "unit": "GLUP/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
                "config": {"workload": spec["label"], "time_steps_per_bench_step": spf,
                           "timed_time_steps": tsteps, "precision": args.precision,
                           "l2": "state (2 buffers x %d MB) larger than the 129 MB L2" %
                                 (nf * cells * storage_bytes(args.precision) // 2**20),
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if variants:
            line["variants"] = variants
        print(json.dumps(line), flush=True)
    g.close()
    dp.finalize()
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(spec, args):
    """The oracle timed on the host cores over a bounded sample."""
    from formura_gb300.host import builtin_program
    from oracle.reference_lib import ReferenceProgram
    src, _ = builtin_program(spec["program"])
    ref = ReferenceProgram(src, spec["cfg"], f"{spec['program']}_bench_ref")
    ref.init()
    st = initial_state(spec, ref)
    for i, f in enumerate(ref.fields):
        ref.set(f, st[i])
    ref.forward(2)
    t0 = time.perf_counter()
    ref.forward(4)
    per = (time.perf_counter() - t0) / 4
    n = int(max(4, min(spec["steps_total"], args.cpu_seconds / max(per, 1e-6))))
    t0 = time.perf_counter()
    ref.forward(n)
    dt = time.perf_counter() - t0
    cells = 1
    for x in spec["shape"]:
        cells *= x
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": cells * n / dt / 1e9, "unit": "GLUP/s", "cores": cores, "kind": "port",
            "sample": f"{n} time steps of the full {spec['label'].split(',')[0]} grid ({dt:.1f} s)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gs2d", choices=["gs2d", "heat3d"])
    ap.add_argument("--precision", default="f64", choices=["f64", "f64fast", "f32", "f16"])
    ap.add_argument("--spf", type=int, default=100, help="time steps per bench step")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    spec = workload_spec(args.workload)
    if args.steps is None:
        args.steps = max(1, spec["steps_total"] // args.spf) if args.impl == "ours" else 200
    if args.impl == "reference":
        run_reference(args, spec)
    else:
        run_ours(args, spec)


if __name__ == "__main__":
    main()
