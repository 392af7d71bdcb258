"""Benchmark of the Formura_Forward hot path on GB300.

Workload (default): 2D Gray-Scott on a 4096^2 periodic grid, Du=2e-5,
Dv=1e-5, F=0.04, k=0.06, dx=0.01, dt=1, 20000 steps, FP64, seeded synthetic
initial state.  A bench "step" is one Formura_Forward-sized chunk of
``--spf`` time steps (1000 for this workload), so ``--steps 20`` (the
default) covers the configured 20000 time steps.  The warm-up steps run
first; the state then goes back to the initial one, so the timed steps are
time steps 0 .. steps*spf of the workload.

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


def W_gs(n):
    from formura_gb300 import workloads as W
    return W.gs_config(n)


def W_heat(n):
    from formura_gb300 import workloads as W
    return W.heat_config(n)


def W_hllc(n):
    from formura_gb300 import workloads as W
    return W.hllc_config(n)


def W_mhd(n):
    from formura_gb300 import workloads as W
    return W.mhd_config(n)


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
        pw = []
        for smp in self.samples:
            try:
                pw.append(float(smp[3]))
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_min_mhz": min(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "power_w": statistics.median(pw) if pw else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def max_over_ranks(x: float, ws: int, device: str) -> float:
    """The slowest rank's time: every replica must finish its steps."""
    if ws <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells_per_rank: int, time_steps: int, ms: float, ws: int) -> float:
    """GLUP/s of the whole job: ws replicas, each advancing its own grid of
    cells_per_rank points by time_steps, in ms (the max over ranks)."""
    return ws * cells_per_rank * time_steps / (ms / 1e3) / 1e9


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
                "steps_total": 20000, "spf": 1000, "cpu_tb": [(16, 516), (32, 520)],
                "variants": ("f64fast", "f32", "f16"),
                "label": "gray-scott-2d 4096^2 periodic, Du=2e-5 Dv=1e-5 F=0.04 k=0.06 dx=0.01 dt=1, 20000 steps"}
    if name == "heat3d":
        n = 128
        return {"program": "heat3d", "cfg": W.heat_config(n), "shape": (n, n, n), "fields": 1,
                "steps_total": 1000, "spf": 100, "cpu_tb": [(4, 68), (8, 144)],
                "variants": ("f64fast", "f32"),
                "label": "heat-3d 128^3 periodic, D*dt/dx^2=0.1, 1000 steps"}
    if name == "hllc3d":
        n = 256
        return {"program": "hllc3d", "cfg": W.hllc_config(n), "shape": (n, n, n), "fields": 5,
                "steps_total": 500, "spf": 25, "cpu_cfg": W.hllc_config(128), "cpu_shape": (128, 128, 128),
                "variants": ("f64fast", "f32", "f16"),
                "cpu_tb": [(2, 68)],
                "label": "hllc-euler-3d 256^3 periodic, gamma=1.4, MUSCL-minmod + HLLC, CFL 0.4, 500 steps"}
    if name == "hlld3d":
        n = 128
        return {"program": "hlld3d", "cfg": W.mhd_config(n), "shape": (n, n, n), "fields": 9,
                "steps_total": 100, "spf": 5, "cpu_cfg": W.mhd_config(48), "cpu_shape": (48, 48, 48),
                "variants": ("f32", "f16"),
                "cpu_tb": [(2, 28)],
                "label": "hlld-mhd-3d 128^3 periodic, gamma=5/3, MUSCL-minmod + HLLD + GLM, CFL 0.3"}
    raise SystemExit(f"unknown workload {name}")


def initial_state(spec, prog):
    """Seeded initial state written through the init hook."""
    import numpy as np
    from formura_gb300 import workloads as W
    if spec["program"] == "gs2d":
        st = W.gs_perturb(prog.get("u"), prog.get("v"), seed=0)
        return np.stack([st["u"], st["v"]])
    if spec["program"] == "hllc3d":
        st = W.hllc_state(tuple(prog.shape), seed=0)
        return np.stack([st[f] for f in prog.fields])
    if spec["program"] == "hlld3d":
        st = W.mhd_state(tuple(prog.shape), seed=0)
        return np.stack([st[f] for f in prog.fields])
    return W.heat_state(spec["shape"], seed=0)["q"][None]


def oracle_configs(spec):
    """(label, config text) of the CPU runs of a workload: NoBlocking, and the
    reference's temporal blocking (Templates.hs:141-172, 311-334) at each
    candidate (time steps per call nt, grid_per_block), all valid under
    (N + 2*s*nt) mod grid_per_block == 0 (NumericalConfig.hs:123,142)."""
    cfg = spec.get("cpu_cfg", spec["cfg"])
    dim = len(spec.get("cpu_shape", spec["shape"]))
    out = [("NoBlocking", "nb", cfg)]
    for nt, gpb in spec.get("cpu_tb", []):
        out.append((f"TemporalBlocking nt={nt} grid_per_block={gpb}", f"tb{nt}_{gpb}",
                    cfg + f"temporal_blocking_interval: {nt}\ngrid_per_block: [{', '.join([str(gpb)] * dim)}]\n"))
    return out


class OracleRun:
    """The oracle (the reference generator's C, restated) of the bench
    workload under one config, loaded with the seeded initial state."""

    def __init__(self, spec, cfg, tag):
        from formura_gb300.host import builtin_program
        from oracle.reference_lib import ReferenceProgram
        src, _ = builtin_program(spec["program"])
        shape = spec.get("cpu_shape", spec["shape"])
        self.ref = ReferenceProgram(src, cfg, f"{spec['program']}_bench_ref_{shape[0]}_{tag}")
        self.spec = spec
        self.reset()
        self.cells = 1
        for x in shape:
            self.cells *= x

    def reset(self):
        """Back to step 0: Formura_Init, then the seeded state."""
        self.ref.init()
        st = initial_state(self.spec, self.ref)
        for i, f in enumerate(self.ref.fields):
            self.ref.set(f, st[i])

    def run(self, calls):
        """(time steps advanced, seconds) of `calls` Formura_Forward calls."""
        t0 = self.ref.navi.time_step
        c0 = time.perf_counter()
        self.ref.forward(calls)
        return self.ref.navi.time_step - t0, time.perf_counter() - c0

    def steps_per_call(self):
        t0 = self.ref.navi.time_step
        self.ref.forward(1)
        return self.ref.navi.time_step - t0


def best_oracle(spec):
    """Every CPU config of the workload, probed over two calls after one;
    returns (label, OracleRun of the fastest, {label: probe GLUP/s})."""
    probes, best = {}, None
    for label, tag, cfg in oracle_configs(spec):
        run = OracleRun(spec, cfg, tag)
        run.run(1)
        steps, dt = run.run(2)
        rate = run.cells * steps / dt / 1e9
        probes[label] = rate
        if best is None or rate > best[2]:
            best = (label, run, rate)
    return best[0], best[1], probes


def run_reference(args, spec):
    """The oracle on the host cores: one bench step = one Formura_Forward
    call of the reference's generated C under the faster of NoBlocking and
    the temporal-blocking candidates (one or nt time steps per call)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    label, run, probes = best_oracle(spec)
    # a bench step is args.spf time steps, as in the GPU arm: spf / nt
    # Formura_Forward calls of the reference's generated C
    nt = run.steps_per_call()
    calls = max(1, args.spf // nt)
    run.run(args.warmup * calls)
    # the timed steps cover time steps 0 .. steps*spf of the workload
    run.reset()
    steps, dt = run.run(args.steps * calls)
    v = run.cells * steps / dt / 1e9
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"metric": "GLUP/s", "value": v, "unit": "GLUP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": spec["label"], "time_steps_per_bench_step": steps // args.steps,
                       "timed_time_steps": f"0..{steps} (from the initial state)",
                       "implementation": f"oracle: reference generator's C (restated), gcc -O3 -fopenmp "
                                         f"-ffp-contract=off, {label}, 1 rank",
                       "probed_configs_GLUPs": probes},
            "cpu_baseline": {"value": v, "unit": "GLUP/s", "cores": cores, "kind": "port",
                             "sample": f"time steps 0..{steps} ({args.steps * calls} Formura_Forward calls, "
                                       f"{label}) of the full grid, after {args.warmup} warm-up bench steps"},
            "e2e": {"value": v, "unit": "GLUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def load_traffic(spec, precision, variant=-1):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/traffic.json), or None.  Keys are program:precision for
    the one-step kernel and program:precision:tb<variant> for a fused one."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    key = f"{spec['program']}:{precision}" + (f":tb{variant}" if variant >= 0 else "")
    return d.get(key)


def dfma_rate():
    """FP64 fused multiply-adds per second of this GPU, measured now by the
    probe library built beside the product (best of 5 launches), or None."""
    import ctypes
    from formura_gb300 import build as B
    if not os.path.exists(B.PROBE_LIB):
        return None
    lib = ctypes.CDLL(B.PROBE_LIB)
    lib.fgb_probe_dfma_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = ctypes.c_double()
    if lib.fgb_probe_dfma_rate(5, ctypes.byref(out)) != 0:
        return None
    return out.value


def fp64_pipe(spec, precision, value, peak_fma_per_s):
    """The bound of the bit-faithful FP64 kernels: FP64-pipe instructions per
    lattice update (ncu sm__inst_executed_pipe_fp64.sum of one step's stage
    kernels / updates, committed in profiles/fp64_pipe.json) times the update
    rate, against the DFMA rate measured in this run."""
    if precision != "f64" or not peak_fma_per_s:
        return None
    p = os.path.join(ROOT, "profiles", "fp64_pipe.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    per = d.get("per_update", {}).get(spec["program"])
    if per is None:
        return None
    peak = peak_fma_per_s / 1e9
    achieved = value * per
    return {"instructions_per_update": per, "achieved_ginst_per_s": achieved, "peak_ginst_per_s": peak,
            "frac": achieved / peak,
            "peak_source": "DFMA rate measured in this run (8 independent FMA chains per thread, "
                           "8 x 256-thread blocks per SM, best of 5 launches)"}


def storage_bytes(precision):
    return {"f64": 8, "f64fast": 8, "f32": 4, "f16": 2}[precision]


L2_BYTES = 129 * 2**20


def time_grid(grid, spf, warmup, steps, torch, stream, flush=None, reset=None, per_step=None):
    """Device time of `steps` bench steps of `spf` time steps each, after
    `warmup` untimed bench steps and `reset()` (back to the initial state, so
    that the timed steps cover time steps 0 .. steps*spf of the workload).
    With a flush buffer (states that fit in L2) every bench step is timed on
    its own after the buffer was overwritten, and the times are summed.
    `per_step`, a list, receives each bench step's time."""
    for _ in range(warmup):
        grid.forward(spf)
    grid.synchronize()
    if reset is not None:
        reset(grid)
        grid.synchronize()
    l0 = grid.launches
    torch.cuda.synchronize()
    if flush is None:
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        evs[0].record(stream)
        for i in range(steps):
            grid.forward(spf)
            evs[i + 1].record(stream)
        evs[-1].synchronize()
        torch.cuda.synchronize()
        if per_step is not None:
            per_step.extend(evs[i].elapsed_time(evs[i + 1]) for i in range(steps))
        return evs[0].elapsed_time(evs[-1]), grid.launches - l0
    evs = []
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.add_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            grid.forward(spf)
            e1.record(stream)
            evs.append((e0, e1))
    torch.cuda.synchronize()
    if per_step is not None:
        per_step.extend(a.elapsed_time(b) for a, b in evs)
    return sum(a.elapsed_time(b) for a, b in evs), grid.launches - l0


# Error bounds of the reduced-precision forms, relative L2 against the FP64
# result of the same steps: 1e-12 for FP64 with contraction (the bound of the
# FP64 drop-in) and 1e-5 for FP32 storage.  FP16 storage has no bound of its
# own; its error is stated against the FP32 bound.
BOUNDS = {"f64fast": 1e-12, "f32": 1e-5, "f16": 1e-5}


def run_sweep(args, spec):
    """Every kernel the autotuner chooses among for this workload, size and
    precision (the generic stage kernels, index -1, and each fused variant),
    timed on its own with CUDA events over --steps bench steps of --spf time
    steps after --warmup, from the workload's initial state: one JSON line
    per kernel.  A measurement aid; the bench line itself keeps the
    autotuner's choice."""
    import numpy as np
    import torch
    from formura_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from formura_gb300.host import FormuraProgram, Grid, builtin_program, program_uniforms
    src, _ = builtin_program(spec["program"])
    cells = 1
    for x in spec["shape"]:
        cells *= x
    dp = FormuraProgram(src, spec["cfg"] + "gpu_steps_per_forward: 1\ngpu_autotune: 0\n", spec["program"],
                        name=f"{spec['program']}_sweep")
    dp.init()
    st0 = initial_state(spec, dp)
    _, U = program_uniforms(src, spec["cfg"], spec["program"])
    sc = None
    if args.precision == "f16":
        sc = [float(max(1e-3, np.abs(st0[i]).max())) for i in range(spec["fields"])]
    g = Grid(spec["program"], spec["shape"], args.precision, U, scales=sc)
    stream = torch.cuda.ExternalStream(g.stream)
    for v in [-1] + [v["index"] for v in g.variants()]:
        g.upload(st0)
        try:
            g.set_variant(v)
        except Exception as e:   # does not fit this grid or this device
            print(json.dumps({"sweep": spec["label"], "variant": v, "skipped": str(e)[:120]}), flush=True)
            continue
        ms, launches = time_grid(g, args.spf, args.warmup, args.steps, torch, stream, None,
                                 lambda grid: grid.upload(st0))
        tsteps = args.steps * args.spf
        kernel = g.variants()[v] if v >= 0 else "generic stage kernels"
        print(json.dumps({"sweep": spec["label"], "precision": args.precision, "variant": v, "kernel": kernel,
                          "value": cells * tsteps / (ms / 1e3) / 1e9, "unit": "GLUP/s",
                          "ms_per_time_step": ms / tsteps, "time_steps": tsteps, "launches": launches}),
              flush=True)
    g.close()


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
    dp = FormuraProgram(src, spec["cfg"] + f"gpu_steps_per_forward: {spf}\ngpu_autotune: 0\n", spec["program"],
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

    def reset(grid):
        grid.upload(st0)

    g = open_grid(args.precision)
    if args.variant is not None:
        g.set_variant(args.variant)
        tuned = args.variant
    else:
        tuned = g.autotune(32) if not args.no_autotune else -1
    variant = next((v for v in g.variants() if v["index"] == tuned), None)
    stream = torch.cuda.ExternalStream(g.stream)
    sampler = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    sampler.start()
    flush_buf = []

    def flush_for(prec):
        # states that fit in L2 get an L2 flush before every timed bench step
        if 2 * nf * cells * storage_bytes(prec) > L2_BYTES:
            return None
        if not flush_buf:
            flush_buf.append(torch.zeros(2 * L2_BYTES // 4, dtype=torch.int32, device="cuda"))
        return flush_buf[0]

    flush = flush_for(args.precision)
    step_ms = []
    ms, launches = time_grid(g, spf, args.warmup, args.steps, torch, stream, flush, reset, step_ms)
    clocks = sampler.stop()
    ms = max_over_ranks(ms, ws, "cuda")
    final64 = g.download()
    tsteps = args.steps * spf
    value = whole_job_rate(cells, tsteps, ms, ws)

    # roofline: algorithmic bytes per lattice update (one read and one write
    # of every state field, no credit for temporal reuse) times the updates
    # one launch performs, over the launch's average duration.  One-step
    # kernels update every cell once per launch; a fused kernel of depth K
    # updates every cell K times, so it can read above 1.0.
    per_step_ms = ms / tsteps
    bytes_per_step = 2 * nf * storage_bytes(args.precision) * cells
    fused = g.variants()[g.variant]["steps"] if g.variant >= 0 else 1
    if fused > 1:
        kernels_per_step = launches / tsteps
        per_launch = bytes_per_step * fused
        launch_us = per_step_ms * 1e3 * tsteps / max(1, launches)
    else:
        kernels_per_step = max(1, round(launches / max(1, tsteps)))
        per_launch = bytes_per_step if kernels_per_step == 1 else None
        launch_us = per_step_ms * 1e3 / kernels_per_step
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_step / (per_step_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": load_traffic(spec, args.precision, g.variant),
                "algorithmic_bytes_per_lattice_update": 2 * nf * storage_bytes(args.precision),
                "algorithmic_bytes_per_launch": per_launch,
                "time_steps_per_launch": fused, "kernels_per_step": kernels_per_step,
                "avg_launch_us": launch_us, "avg_step_us": per_step_ms * 1e3}

    # reduced-precision forms over the same time steps from the same state,
    # timed the same way; their error is the relative L2 per field against
    # the FP64 result of the same step
    variants, vgrids = {}, {}
    if rank == 0 and not args.no_variants and args.precision == "f64":
        for prec in spec.get("variants", ()):
            gv = open_grid(prec)
            tv = gv.autotune(32) if not args.no_autotune else -1
            sv = torch.cuda.ExternalStream(gv.stream)
            vms, _ = time_grid(gv, spf, args.warmup, args.steps, torch, sv, flush_for(prec), reset)
            fin = gv.download()
            errs = {f: W.rel_l2(fin[i], final64[i]) for i, f in enumerate(dp.fields)}
            vv = cells * tsteps / (vms / 1e3) / 1e9
            variants[prec] = {"kernel": next((v for v in gv.variants() if v["index"] == tv), "one step per launch"),
                              "value": vv, "unit": "GLUP/s", "speedup_vs_f64": vv / value * ws,
                              "rel_l2_vs_f64_at_horizon": errs, "horizon_time_steps": tsteps,
                              "bound": BOUNDS[prec], "meets_bound_at_horizon": max(errs.values()) <= BOUNDS[prec],
                              "l2_flushed": flush_for(prec) is not None}
            vgrids[prec] = gv

    # end to end through the drop-in C API: upload + spf steps + download per
    # Formura_Forward call.  Two warm-up calls, then formura_data goes back to
    # the initial state and the calls are timed one by one, with nothing else
    # between them.  A line of another precision times a drop-in built with
    # that precision (gpu_precision, and its kernel chosen at Formura_Init as
    # here).
    de = dp
    if args.precision != "f64":
        extra = (f"gpu_steps_per_forward: {spf}\ngpu_precision: {args.precision}\n"
                 f"gpu_autotune: {0 if args.no_autotune else 1}\n")
        if args.precision == "f16":
            extra += "gpu_field_scales: [" + ", ".join(
                repr(float(max(1e-3, np.abs(st0[i]).max()))) for i in range(nf)) + "]\n"
        de = FormuraProgram(src, spec["cfg"] + extra, spec["program"],
                            name=f"{spec['program']}_bench_e2e_{args.precision}_{local}")
        de.init()
    for _ in range(2):
        de.forward(1)
    for i, f in enumerate(de.fields):
        de.set(f, st0[i])
    e2e_sampler = ClockSampler(local)
    e2e_sampler.start()
    e2e_calls = max(1, min(args.steps, args.e2e_steps))
    e2e_s = 0.0
    call_ms = []
    for c in range(e2e_calls):
        t0 = time.perf_counter()
        de.forward(1)
        call_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_s += call_ms[-1] / 1e3
    e2e_clocks = e2e_sampler.stop()
    # the error of each reduced-precision form along the horizon, after the
    # timed calls (untimed): the FP64 drop-in and the forms advance the same
    # steps from the same state, checkpoint by checkpoint
    track = {p: [] for p in vgrids}
    if vgrids:
        for i, f in enumerate(dp.fields):
            dp.set(f, st0[i])
        for gv in vgrids.values():
            reset(gv)
        for c in range(e2e_calls):
            dp.forward(1)
            ref = [dp.get(f) for f in dp.fields]
            for p, gv in vgrids.items():
                gv.forward(spf)
                fin = gv.download()
                track[p].append(((c + 1) * spf, max(W.rel_l2(fin[i], ref[i]) for i in range(nf))))
    e2e = {"value": ws * cells * e2e_calls * spf / e2e_s / 1e9, "unit": "GLUP/s",
           "h2d_bytes_per_step": nf * cells * 8, "d2h_bytes_per_step": nf * cells * 8,
           "steps": e2e_calls, "time_steps": e2e_calls * spf,
           "api": f"Formura_Forward (drop-in C API, formura_data on the host, gpu_precision {args.precision})",
           "call_ms": [round(x, 2) for x in call_ms],
           "clocks": e2e_clocks}
    for p, gv in vgrids.items():
        above = [s for s, e in track[p] if e > BOUNDS[p]]
        variants[p]["max_rel_l2_by_time_step"] = [[s, e] for s, e in track[p]]
        variants[p]["first_checkpoint_above_bound"] = above[0] if above else None
        gv.close()

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(spec, args)

    if rank == 0:
        line = {"metric": "GLUP/s", "value": value, "unit": "GLUP/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
                "config": {"workload": spec["label"], "time_steps_per_bench_step": spf,
                           "timed_time_steps": f"0..{tsteps} (from the initial state, after {args.warmup} "
                                               f"warm-up bench steps)",
                           "precision": args.precision,
                           "kernel": variant if variant else "one step per launch (generic stage kernel)",
                           "l2": ("state (2 buffers x %d MB) larger than the 129 MB L2" if flush is None else
                                  "state (2 buffers x %d MB) fits in the 129 MB L2: a 258 MB buffer is "
                                  "overwritten before every timed bench step") %
                                 (nf * cells * storage_bytes(args.precision) // 2**20),
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
                "bench_step_ms": [round(x, 3) for x in step_ms]}
        fp64 = fp64_pipe(spec, args.precision, value / ws, dfma_rate())
        if fp64 is not None:
            line["fp64_pipe_bound"] = fp64
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if variants:
            line["variants"] = variants
        print(json.dumps(line), flush=True)
    g.close()
    if de is not dp:
        de.finalize()
    dp.finalize()
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(spec, args):
    """The oracle timed on the host cores over a bounded sample (about
    --cpu-seconds), under the faster of NoBlocking and temporal blocking."""
    label, run, probes = best_oracle(spec)
    steps, dt = run.run(1)
    calls = int(max(2, min(spec["steps_total"] / max(steps, 1), args.cpu_seconds / max(dt, 1e-6))))
    steps, dt = run.run(calls)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    grid = "x".join(str(x) for x in spec.get("cpu_shape", spec["shape"]))
    return {"value": run.cells * steps / dt / 1e9, "unit": "GLUP/s", "cores": cores, "kind": "port",
            "sample": f"{steps} time steps of the {spec['program']} workload on a {grid} grid ({dt:.1f} s, {label})",
            "probed_configs_GLUPs": probes}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gs2d",
                    choices=["gs2d", "heat3d", "hllc3d", "hlld3d", "adjoint", "hllc_adjoint", "batch"])
    ap.add_argument("--precision", default="f64", choices=["f64", "f64fast", "f32", "f16"])
    ap.add_argument("--spf", type=int, default=None,
                    help="time steps per bench step (default: the workload's, e.g. 1000 for Gray-Scott, so that "
                         "--steps 20 covers its 20000 time steps)")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--variant", type=int, default=None, help="use this temporal-blocking kernel (no autotune)")
    ap.add_argument("--size", type=int, default=None, help="grid points per axis (smaller profiling cases)")
    ap.add_argument("--sweep", action="store_true",
                    help="time every kernel the autotuner chooses among, one JSON line each, and exit")
    ap.add_argument("--adj-n", type=int, default=512)
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--probes", type=int, default=64)
    ap.add_argument("--time-steps", type=int, default=20)
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=5000)
    args = ap.parse_args()
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.workload == "hllc_adjoint":
        run_hllc_adjoint(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    spec = workload_spec(args.workload)
    if args.size:
        n = args.size
        make = {"gs2d": W_gs, "heat3d": W_heat, "hllc3d": W_hllc, "hlld3d": W_mhd}[args.workload]
        spec["cfg"] = make(n)
        spec["shape"] = tuple([n] * len(spec["shape"]))
        spec["label"] = spec["label"].replace(spec["label"].split(" ")[1], f"{n}^{len(spec['shape'])}", 1)
    if args.spf is None:
        args.spf = spec["spf"]
    if args.steps is None:
        args.steps = max(1, spec["steps_total"] // args.spf)
    if args.sweep:
        run_sweep(args, spec)
    elif args.impl == "reference":
        run_reference(args, spec)
    else:
        run_ours(args, spec)



def run_adjoint(args):
    """Diffusion adjoint and inverse-problem gradient (512^3, D*dt/dx^2 = 0.1,
    200 steps): dJ/du_0 of J = 0.5*||u_T - u_target||^2 by the generated
    adjoint with binomial checkpointing (8 snapshots), in FP64 and FP32,
    checked against central differences (eps 1e-6, FP64) on random probes."""
    import numpy as np
    import torch
    from formura_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from formura_gb300 import workloads as W
    from formura_gb300.host import Grid, builtin_program, program_uniforms
    n, nsteps, snaps = args.adj_n, args.adj_steps, 8
    shape = (n, n, n)
    src, _ = builtin_program("heat3d")
    _, U = program_uniforms(src, W.heat_config(n), "heat3d")

    def field(seed):
        rng = np.random.default_rng(seed)
        dev = "cuda"
        idx = torch.arange(n, dtype=torch.float64, device=dev)
        out = torch.zeros(shape, dtype=torch.float64, device=dev)
        for _ in range(32):
            c = [rng.uniform(0, n) for _ in range(3)]
            w = rng.uniform(4.0, 16.0)
            amp = rng.normal()
            parts = []
            for ax in range(3):
                d = (idx - c[ax]).abs()
                d = torch.minimum(d, n - d)
                parts.append(torch.exp(-0.5 * (d / w) ** 2))
            out += amp * parts[0][:, None, None] * parts[1][None, :, None] * parts[2][None, None, :]
        return out.cpu().numpy()[None]

    u0, target = field(0), field(1)
    cells = n ** 3
    res = {}
    for prec in ("f64", "f32"):
        g = Grid("heat3d", shape, prec, U)
        stream = torch.cuda.ExternalStream(g.stream)
        g.upload(u0)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        g.forward(5)
        g.synchronize()
        ev[0].record(stream)
        g.forward(args.time_steps)
        ev[1].record(stream)
        g.adjoint_steps(1)
        g.synchronize()
        ev[2].record(stream)
        g.adjoint_steps(args.time_steps)
        ev[3].record(stream)
        ev[3].synchronize()
        t_fwd = ev[0].elapsed_time(ev[1]) / args.time_steps
        t_adj = ev[2].elapsed_time(ev[3]) / args.time_steps
        t0 = time.perf_counter()
        uT, grad = g.gradient(u0, nsteps, snaps, lambda uT: uT - target)
        t_grad = time.perf_counter() - t0
        st = g.gradient_stats()
        res[prec] = {"forward_ms_per_step": t_fwd, "adjoint_ms_per_step": t_adj,
                     "adjoint_over_forward": t_adj / t_fwd,
                     "forward_GLUPs": cells / (t_fwd / 1e3) / 1e9, "adjoint_GLUPs": cells / (t_adj / 1e3) / 1e9,
                     "gradient_seconds": t_grad, "gradient_forward_steps": st["forward_steps"],
                     "gradient_adjoint_steps": st["adjoint_steps"], "grad": grad,
                     "loss": 0.5 * float(np.vdot(uT - target, uT - target))}
        g.close()
    # central differences of the bit-faithful FP64 forward, which equals the
    # oracle (the reference generator's C) bit for bit
    fd_grid = Grid("heat3d", shape, "f64", U)

    def loss(u):
        fd_grid.upload(u)
        fd_grid.forward(nsteps)
        d = fd_grid.download() - target
        return 0.5 * float(np.vdot(d, d))

    rng = np.random.default_rng(2)
    eps = 1e-6
    errs64, errs32 = [], []
    for _ in range(args.probes):
        v = rng.standard_normal(u0.shape)
        fd = (loss(u0 + eps * v) - loss(u0 - eps * v)) / (2 * eps)
        errs64.append(abs(float(np.vdot(res["f64"]["grad"], v)) - fd) / abs(fd))
        errs32.append(abs(float(np.vdot(res["f32"]["grad"], v)) - fd) / abs(fd))
    fd_grid.close()
    g32_vs_64 = W.rel_l2(res["f32"]["grad"], res["f64"]["grad"])
    for p in res:
        res[p].pop("grad")
    line = {"metric": "GLUP/s", "value": res["f64"]["adjoint_GLUPs"], "unit": "GLUP/s",
            "n_gpus": 1, "steps": args.time_steps, "warmup": 5, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"diffusion adjoint {n}^3 periodic, D*dt/dx^2=0.1, {nsteps} steps, "
                                   f"32 Gaussians, binomial checkpointing {snaps} snapshots",
                       "value_is": "adjoint step rate (FP64)"},
            "adjoint": res,
            "fd_check": {"probes": args.probes, "eps": eps, "max_rel_err_f64": max(errs64),
                         "median_rel_err_f64": float(np.median(errs64)),
                         "max_rel_err_f32": max(errs32), "median_rel_err_f32": float(np.median(errs32))},
            "grad_f32_rel_l2_vs_f64": g32_vs_64}
    print(json.dumps(line), flush=True)



def run_hllc_adjoint(args):
    """Euler adjoint (HLLC 3D, the smooth Mach-0.3 state): dJ/d rho_0 of
    J = 0.5*||u_T - u_target||^2 over --adj-steps steps (100 by default) with
    binomial checkpointing (8 snapshots), in FP64 and FP32, by the generated
    two-pass adjoint of the three-stage step; checked against central
    differences of the bit-exact FP64 forward on random density directions."""
    import numpy as np
    import torch
    from formura_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from formura_gb300 import workloads as W
    from formura_gb300.host import Grid, builtin_program, program_uniforms
    n, nsteps, snaps = args.adj_n, args.adj_steps, 8
    shape = (n, n, n)
    fields = ["e", "mx", "my", "mz", "rho"]
    src, _ = builtin_program("hllc3d")
    _, U = program_uniforms(src, W.hllc_config(n), "hllc3d")
    st = W.hllc_state(shape, 0)
    u0 = np.stack([st[f] for f in fields])
    target = u0 + 0.01 * np.random.default_rng(1).standard_normal(u0.shape)
    cells = n ** 3
    res = {}
    for prec in ("f64", "f32"):
        g = Grid("hllc3d", shape, prec, U)
        stream = torch.cuda.ExternalStream(g.stream)
        g.upload(u0)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        g.forward(2)
        g.synchronize()
        ev[0].record(stream)
        g.forward(args.time_steps)
        ev[1].record(stream)
        g.adjoint_steps(1)
        g.synchronize()
        ev[2].record(stream)
        g.adjoint_steps(args.time_steps)
        ev[3].record(stream)
        ev[3].synchronize()
        t_fwd = ev[0].elapsed_time(ev[1]) / args.time_steps
        t_adj = ev[2].elapsed_time(ev[3]) / args.time_steps
        t0 = time.perf_counter()
        uT, grad = g.gradient(u0, nsteps, snaps, lambda uT: uT - target)
        t_grad = time.perf_counter() - t0
        gs = g.gradient_stats()
        res[prec] = {"forward_ms_per_step": t_fwd, "adjoint_ms_per_step": t_adj,
                     "adjoint_over_forward": t_adj / t_fwd,
                     "forward_GLUPs": cells / (t_fwd / 1e3) / 1e9, "adjoint_GLUPs": cells / (t_adj / 1e3) / 1e9,
                     "gradient_seconds": t_grad, "gradient_forward_steps": gs["forward_steps"],
                     "gradient_adjoint_steps": gs["adjoint_steps"], "grad": grad}
        g.close()
    fd_grid = Grid("hllc3d", shape, "f64", U)

    def loss(u):
        fd_grid.upload(u)
        fd_grid.forward(nsteps)
        d = fd_grid.download() - target
        return 0.5 * float(np.vdot(d, d))

    rng = np.random.default_rng(2)
    eps = 1e-7
    ir = fields.index("rho")
    errs = {"f64": [], "f32": []}
    for _ in range(args.probes):
        v = np.zeros_like(u0)
        v[ir] = rng.standard_normal(shape)
        fd = (loss(u0 + eps * v) - loss(u0 - eps * v)) / (2 * eps)
        for p in errs:
            errs[p].append(abs(float(np.vdot(res[p]["grad"], v)) - fd) / abs(fd))
    fd_grid.close()
    g32_vs_64 = W.rel_l2(res["f32"]["grad"][ir], res["f64"]["grad"][ir])
    for p in res:
        res[p].pop("grad")
    line = {"metric": "GLUP/s", "value": res["f64"]["adjoint_GLUPs"], "unit": "GLUP/s",
            "n_gpus": 1, "steps": args.time_steps, "warmup": 3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"hllc-euler-3d adjoint {n}^3 periodic, smooth Mach-0.3 state, {nsteps} steps, "
                                   f"gradient w.r.t. initial density, binomial checkpointing {snaps} snapshots",
                       "value_is": "adjoint step rate (FP64)"},
            "adjoint": res,
            "fd_check": {"probes": args.probes, "eps": eps, "direction": "density only",
                         "max_rel_err_f64": max(errs["f64"]), "median_rel_err_f64": float(np.median(errs["f64"])),
                         "max_rel_err_f32": max(errs["f32"]), "median_rel_err_f32": float(np.median(errs["f32"]))},
            "grad_rho_f32_rel_l2_vs_f64": g32_vs_64}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """Batched Gray-Scott ensemble: 256 grids, sides log-uniform in
    [64, 1024], F ~ U[0.02, 0.06], k ~ U[0.05, 0.065], 5000 steps, FP32
    storage, persistent launches over one tile queue, time loop replayed
    from a CUDA graph, kernel picked by the autotuner; against 256
    sequential plain FP64 runs on the same GPU."""
    import numpy as np
    import torch
    from formura_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from formura_gb300 import workloads as W
    from formura_gb300.host import Batch, Grid, builtin_program, program_uniforms
    src, _ = builtin_program("gs2d")
    members = W.ensemble(args.count, 0)
    U, X = [], []
    for i, (n, F, k) in enumerate(members):
        _, u = program_uniforms(src, W.gs_config(n), "gs2d", params={"F": F, "kappa": k})
        U.append(u)
        X.append(W.gs_square_state(n, 1000 + i))
    cells = sum(n * n for n, _, _ in members)
    steps = args.batch_steps
    b = Batch("gs2d", [(n, n) for n, _, _ in members], "f32", U)
    for i, x in enumerate(X):
        b.upload(i, x)
    chosen = b.autotune(32)
    kernel = b.variants()[chosen]
    for i, x in enumerate(X):
        b.upload(i, x)
    stream = torch.cuda.ExternalStream(b.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(0)
    sampler.start()
    l0 = b.launches
    b.synchronize()
    e0.record(stream)
    b.forward(steps)
    e1.record(stream)
    e1.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    launches = b.launches - l0
    f32_final = [b.download(i) for i in range(len(members))]
    b.close()
    value = cells * steps / (ms / 1e3) / 1e9
    # 256 sequential plain FP64 runs (the bit-faithful drop-in kernels)
    t0 = time.perf_counter()
    f64_final = []
    for i, (n, _, _) in enumerate(members):
        g = Grid("gs2d", (n, n), "f64", U[i])
        g.upload(X[i])
        g.forward(steps)
        f64_final.append(g.download())
        g.close()
    t64 = time.perf_counter() - t0
    # per grid, the larger of the two fields' relative L2 distances, both
    # against the final FP64 field and against the initial field's norm
    # (where a pattern dies out, v decays towards 0 and the final field's
    # norm is no yardstick)
    errs, errs_final = [], []
    for i in range(len(members)):
        d = [float(np.linalg.norm(f32_final[i][j] - f64_final[i][j])) for j in range(2)]
        errs.append(max(d[j] / float(np.linalg.norm(X[i][j])) for j in range(2)))
        errs_final.append(max(d[j] / max(float(np.linalg.norm(f64_final[i][j])), 1e-300) for j in range(2)))
    v64 = cells * steps / t64 / 1e9
    line = {"metric": "GLUP/s", "value": value, "unit": "GLUP/s", "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"batched gray-scott ensemble: {len(members)} grids, sides log-uniform "
                                   f"[64,1024], F~U[.02,.06], k~U[.05,.065], {steps} steps",
                       "cells_total": cells, "kernel": kernel,
                       "launch": "persistent CTAs over one tile queue; 64-step chunks replayed from a CUDA graph"},
            "gpu_launches": launches, "clocks": clocks,
            "sequential_f64": {"value": v64, "unit": "GLUP/s", "seconds": t64,
                               "note": "256 sequential fgb_open/forward/download runs, bit-faithful FP64"},
            "speedup_vs_sequential_f64": value / v64,
            "rel_l2_f32_vs_f64": {"median": float(np.median(errs)), "max": float(np.max(errs)),
                                  "normalised_by": "L2 norm of the initial field",
                                  "grids_within_1e-5": int(sum(e <= 1e-5 for e in errs))},
            "rel_l2_f32_vs_f64_final": {"median": float(np.median(errs_final)), "max": float(np.max(errs_final)),
                                        "normalised_by": "L2 norm of the final FP64 field",
                                        "grids_within_1e-5": int(sum(e <= 1e-5 for e in errs_final))},
            "grids": len(members)}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
