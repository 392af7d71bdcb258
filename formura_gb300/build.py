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
import re
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


def generate(names: Optional[List[str]] = None, sources: Optional[Dict[str, tuple]] = None,
             gen_dir: str = GEN) -> Dict[str, str]:
    """Emit device code for each program and the registry of the library;
    return name -> .cu path.  Programs are the shipped ones (`names`, default
    all) or, with `sources`, name -> (.fmr text, .yaml text)."""
    from .generator.config import decode_config
    from .generator.cuda import emit_cuda
    from .generator.manifest import compile_program
    os.makedirs(gen_dir, exist_ok=True)
    out = {}
    registered: List[str] = []
    if sources is None:
        sources = {name: program_sources(name) for name in (names or program_names())}
    for name, (src, cfg) in sources.items():
        mm = compile_program(src, decode_config(cfg))
        kp = emit_cuda(mm, name, runtime_params(cfg))
        text = kp.source
        subs = []
        for graph in ("first_step", "filter"):
            if getattr(mm, graph) is not None:
                sub = emit_cuda(mm, name, runtime_params(cfg), graph)
                text += "\n" + sub.source
                subs.append(f"{name}__{graph}")
        path = os.path.join(gen_dir, f"prog_{name}.cu")
        _write_if_changed(path, text)
        meta = {"name": name, "fields": kp.fields, "dim": kp.dim, "sleeve": kp.sleeve,
                "shift": kp.shift, "nuniforms": len(kp.uniform_exprs),
                "stages": len(kp.stages), "mids": len(kp.mids), "subprograms": subs}
        _write_if_changed(os.path.join(gen_dir, f"prog_{name}.json"), json.dumps(meta, indent=1) + "\n")
        out[name] = path
        registered.extend([name] + subs)
    reg = ['#include "fgb_internal.h"']
    names = sorted(registered)
    reg += [f'extern "C" const FgbProgramDesc* fgb_program_{n}(void);' for n in names]
    reg.append('extern "C" const FgbProgramGetter fgb_builtin_programs[] = {'
               + ", ".join(f"&fgb_program_{n}" for n in names) + "};")
    reg.append(f'extern "C" const int fgb_builtin_program_count = {len(names)};')
    _write_if_changed(os.path.join(gen_dir, "fgb_registry.cu"), "\n".join(reg) + "\n")
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


RUNTIME_UNITS = ("fgb_runtime", "fgb_noalloc", "fgb_batch", "fgb_lazy")


def _deps() -> List[str]:
    return [os.path.join(CSRC, f) for f in ("fgb_internal.h", "fgb_templates.cuh", "fgb_fused.cuh", "fgb_fused_ms.cuh", "fgb_wait.cuh")
            if os.path.exists(os.path.join(CSRC, f))] + [os.path.join(ROOT, "include", "formura_gb300.h")]


def _link(objs: List[str], out: str):
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["nvcc", *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    os.replace(tmp, out)


def _library(gen: Dict[str, str], gen_dir: str, obj_dir: str, out: str, jobs: Optional[int]):
    """Compile the runtime (program-independent objects, cached in the
    library's build folder), the programs and their registry; link `out`."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(obj_dir, exist_ok=True)
    deps = _deps()
    units = [(os.path.join(CSRC, u + ".cu"), os.path.join(BUILD, u + ".o")) for u in RUNTIME_UNITS]
    units.append((os.path.join(gen_dir, "fgb_registry.cu"), os.path.join(obj_dir, "fgb_registry.o")))
    units += [(p, os.path.join(obj_dir, f"prog_{n}.o")) for n, p in gen.items()]
    jobs = jobs or max(2, min(len(units), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], deps), units))
    _link(objs, out)


def program_identifier(name: str) -> str:
    """A library program name usable in C identifiers (the generated kernels
    live in namespace fgb_gen_<name>): '3d_hllc' becomes 'p3d_hllc'."""
    ident = re.sub(r"\W", "_", name)
    return "p" + ident if not ident or ident[0].isdigit() else ident


def build_program_library(name: str, fmr_src: str, yaml_text: str, out: str,
                          jobs: Optional[int] = None, verbose: bool = False) -> str:
    """A library like libformura_gb300.so whose kernels are those of one
    user program (a .fmr with its numerical config), registered under
    `name`: the counterpart of running the reference's `formura` on a new
    program.  The generated C body (generator/cli.py) opens the program by
    that name.  Returns the library path."""
    if shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build formura_gb300")
    if program_identifier(name) != name:
        raise ValueError(f"program name {name!r} is not a C identifier; use {program_identifier(name)!r}")
    key = hashlib.sha1((name + "\0" + fmr_src + "\0" + yaml_text).encode()).hexdigest()[:12]
    gen_dir = os.path.join(BUILD, "user", f"{name}_{key}")
    gen = generate(sources={name: (fmr_src, yaml_text)}, gen_dir=gen_dir)
    _library(gen, gen_dir, gen_dir, out, jobs)
    if verbose:
        print("built", out)
    return out


def build(names: Optional[List[str]] = None, jobs: Optional[int] = None, verbose: bool = False) -> str:
    """Generate, compile and link; returns the library path."""
    if shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build formura_gb300")
    gen = generate(names)
    _library(gen, GEN, BUILD, LIB, jobs)
    _link([_compile(os.path.join(CSRC, "fgb_probe.cu"), os.path.join(BUILD, "fgb_probe.o"), [])], PROBE_LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    build(verbose=True)
