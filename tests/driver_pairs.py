"""Driver programs linked against generated C pairs, as a Formura user builds
them (the reference's Makefiles: ``gcc main.c X.c -o main``).

* ``gpu_pair``: ``X.c``/``X.h`` from this backend's generator command
  (``generator/cli.py --lib``) plus ``lib<program>_gb300.so`` with the
  program's kernels.
* ``oracle_pair``: the reference generator's ``X.c``/``X.h`` (restated,
  ``oracle/emit_reference_c.py``), no MPI, built with OpenMP.
* ``link``: compile a driver's ``main.c`` unchanged against either pair.
* ``run``: run it in a fresh folder with the ``data/`` directory the
  drivers write to; returns the SHA-256 of every file written there.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from typing import Dict, Optional

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def one_rank_config(text: str, grid: Optional[str] = None) -> str:
    """A config for one rank, one step per Formura_Forward: MPI shape and
    temporal blocking dropped, optionally another grid_per_node."""
    keep = []
    for line in text.splitlines():
        key = line.split(":")[0].strip()
        if key in ("mpi_shape", "grid_per_block", "temporal_blocking_interval"):
            continue
        if key == "grid_per_node" and grid is not None:
            line = f"grid_per_node: {grid}"
        keep.append(line)
    return "\n".join(keep) + "\n"


def gpu_pair(d: str, base: str, fmr_src: str, cfg_text: str) -> str:
    """Generate base.c / base.h and the program's library in `d`; returns
    the library's program name (the -l name is <program>_gb300)."""
    from formura_gb300 import build as B
    from formura_gb300.generator import cli
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, base + ".fmr"), "w") as f:
        f.write(fmr_src)
    with open(os.path.join(d, base + ".yaml"), "w") as f:
        f.write(cfg_text)
    rc = cli.main(["--lib", os.path.join(d, base + ".fmr")])
    if rc != 0:
        raise RuntimeError(f"generator failed for {base}")
    return B.program_identifier(base)


def oracle_pair(d: str, base: str, fmr_src: str, cfg_text: str):
    from formura_gb300.generator.config import decode_config
    from formura_gb300.generator.manifest import compile_program
    from oracle.emit_reference_c import Emitter
    os.makedirs(d, exist_ok=True)
    h, c = Emitter(compile_program(fmr_src, decode_config(cfg_text)), base + ".h").emit()
    with open(os.path.join(d, base + ".h"), "w") as f:
        f.write(h)
    with open(os.path.join(d, base + ".c"), "w") as f:
        f.write(c)


def link(main_c: str, d: str, base: str, program: Optional[str] = None, cflags=()) -> str:
    """Compile `main_c` unchanged with the pair in `d` (GPU pair when
    `program` names its library, else the oracle pair); returns the binary."""
    exe = os.path.join(d, "main")
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", *cflags, "-I", d, main_c,
           os.path.join(d, base + ".c"), "-o", exe]
    if program is not None:
        cmd += ["-I", os.path.join(ROOT, "include"), "-L", d, f"-l{program}_gb300", f"-Wl,-rpath,{d}"]
    else:
        cmd += ["-fopenmp"]
    cmd += ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    return exe


def run(exe: str, workdir: str, timeout: float = 600) -> Dict[str, str]:
    os.makedirs(os.path.join(workdir, "data"), exist_ok=True)
    r = subprocess.run([exe], cwd=workdir, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"{exe} exited {r.returncode}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    out = {}
    for name in sorted(os.listdir(os.path.join(workdir, "data"))):
        with open(os.path.join(workdir, "data", name), "rb") as f:
            out[name] = hashlib.sha256(f.read()).hexdigest()
    return out
