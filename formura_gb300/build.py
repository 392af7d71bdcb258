"""Build of the CUDA library ``libformura_gb300.so`` (sm_103a).

For every program shipped in ``formura_gb300/programs`` (a ``.fmr`` file with
its ``.yaml`` numerical config) the generator emits the stage functors into
``formura_gb300/_gen/prog_<name>.cu``; the translation units are compiled in
parallel with nvcc and linked together with the runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import json
import os
import shutil
import subprocess
import sys
from typing import Dict, List, Optional

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GEN = os.path.join(HERE, "_gen")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libformura_gb300.so")
PROBE_LIB = os.path.join(BUILD, "libfgb_probe.so")   # FP64 pipe throughput probe
PROGRAMS = os.path.join(HERE, "programs")
CSRC = os.path.join(HERE, "csrc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-O3", "--expt-relaxed-constexpr"]
# extra nvcc options for experiments (for example -DFGB_DIVU_IEEE)
NVCC_FLAGS += os.environ.get("FGB_NVCC_EXTRA", "").split()


def program_names() -> List[str]:
    return sorted(f[:-4] for f in os.listdir(PROGRAMS)
                  if f.endswith(".fmr") and os.path.exists(os.path.join(PROGRAMS, f[:-4] + ".yaml")))


def program_sources(name: str):
    with open(os.path.join(PROGRAMS, name + ".fmr")) as f:
        src = f.read()
    with open(os.path.join(PROGRAMS, name + ".yaml")) as f:
        cfg = f.read()
    return src, cfg


def runtime_params(cfg_text: str) -> List[str]:
    from .generator.config import decode_config
    nc = decode_config(cfg_text)
    v = nc.gpu.get("gpu_runtime_params")
    if v is None:
        return []
    if not isinstance(v, list):
        raise ValueError("gpu_runtime_params must be a list of constant names")
    return [str(x) for x in v]


def library_runtime_params(name: str) -> List[str]:
    """Runtime parameters the library's kernels of `name` were compiled with."""
    return runtime_params(program_sources(name)[1])


def generate(names: Optional[List[str]] = None) -> Dict[str, str]:
    """Emit device code for each program; return name -> .cu path."""
    from .generator.config import decode_config
    from .generator.cuda import emit_cuda
    from .generator.manifest import compile_program
    os.makedirs(GEN, exist_ok=True)
    out = {}
    registered: List[str] = []
    for name in names or program_names():
        src, cfg = program_sources(name)
        mm = compile_program(src, decode_config(cfg))
        kp = emit_cuda(mm, name, runtime_params(cfg))
        text = kp.source
        subs = []
        for graph in ("first_step", "filter"):
            if getattr(mm, graph) is not None:
                sub = emit_cuda(mm, name, runtime_params(cfg), graph)
                text += "\n" + sub.source
                subs.append(f"{name}__{graph}")
        path = os.path.join(GEN, f"prog_{name}.cu")
        _write_if_changed(path, text)
        meta = {"name": name, "fields": kp.fields, "dim": kp.dim, "sleeve": kp.sleeve,
                "shift": kp.shift, "nuniforms": len(kp.uniform_exprs),
                "stages": len(kp.stages), "mids": len(kp.mids), "subprograms": subs}
        _write_if_changed(os.path.join(GEN, f"prog_{name}.json"), json.dumps(meta, indent=1) + "\n")
        out[name] = path
        registered.extend([name] + subs)
    reg = ['#include "../csrc/fgb_internal.h"']
    names = sorted(registered)
    reg += [f'extern "C" const FgbProgramDesc* fgb_program_{n}(void);' for n in names]
    reg.append('extern "C" const FgbProgramGetter fgb_builtin_programs[] = {'
               + ", ".join(f"&fgb_program_{n}" for n in names) + "};")
    reg.append(f'extern "C" const int fgb_builtin_program_count = {len(names)};')
    _write_if_changed(os.path.join(GEN, "fgb_registry.cu"), "\n".join(reg) + "\n")
    return out


def _write_if_changed(path: str, text: str):
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


def _digest(paths: List[str], extra: str) -> str:
    h = hashlib.sha1(extra.encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def _compile(src: str, obj: str, deps: List[str]) -> str:
    stamp = obj + ".hash"
    dig = _digest([src] + deps, " ".join(NVCC_FLAGS))
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == dig:
        return obj
    cmd = ["nvcc", *NVCC_FLAGS, "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stderr[-6000:])
    with open(stamp, "w") as f:
        f.write(dig)
    return obj


def build(names: Optional[List[str]] = None, jobs: Optional[int] = None, verbose: bool = False) -> str:
    """Generate, compile and link; returns the library path."""
    if shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build formura_gb300")
    gen = generate(names)
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in ("fgb_internal.h", "fgb_templates.cuh", "fgb_fused.cuh")
            if os.path.exists(os.path.join(CSRC, f))] + [os.path.join(ROOT, "include", "formura_gb300.h")]
    units = [(os.path.join(CSRC, "fgb_runtime.cu"), os.path.join(BUILD, "fgb_runtime.o")),
             (os.path.join(CSRC, "fgb_noalloc.cu"), os.path.join(BUILD, "fgb_noalloc.o")),
             (os.path.join(CSRC, "fgb_batch.cu"), os.path.join(BUILD, "fgb_batch.o")),
             (os.path.join(CSRC, "fgb_lazy.cu"), os.path.join(BUILD, "fgb_lazy.o")),
             (os.path.join(GEN, "fgb_registry.cu"), os.path.join(BUILD, "fgb_registry.o"))]
    units += [(p, os.path.join(BUILD, f"prog_{n}.o")) for n, p in gen.items()]
    jobs = jobs or max(2, min(len(units), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], deps), units))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["nvcc", *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    probe_obj = _compile(os.path.join(CSRC, "fgb_probe.cu"), os.path.join(BUILD, "fgb_probe.o"), [])
    tmp = PROBE_LIB + f".tmp{os.getpid()}"
    cmd = ["nvcc", *ARCH, "-shared", "-o", tmp, probe_obj, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    os.replace(tmp, PROBE_LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    build(verbose=True)
