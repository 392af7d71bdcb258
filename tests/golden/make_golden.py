"""Writes the golden fixtures of tests/golden: the oracle's output (the
reference generator's C, restated, compiled with gcc) for small seeded runs
of the shipped programs.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from formura_gb300 import workloads as W  # noqa: E402
from formura_gb300.host import builtin_program  # noqa: E402
from oracle.reference_lib import ReferenceProgram  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def make(name, program, cfg, steps, state_fn):
    src, _ = builtin_program(program)
    ref = ReferenceProgram(src, cfg, f"mkgold_{name}")
    ref.init()
    st = state_fn(ref)
    for f in ref.fields:
        ref.set(f, st[f])
    nav = ref.forward(steps)
    d = {"program": program, "config": cfg, "steps": steps, "offset_x": nav["offset_x"]}
    for f in ref.fields:
        d["in_" + f] = st[f]
        d["out_" + f] = ref.get(f)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **d)
    print("wrote", name)


if __name__ == "__main__":
    make("heat3d_16_10", "heat3d", W.heat_config(16), 10, lambda r: W.heat_state((16, 16, 16), 11))
    make("gs2d_64_50", "gs2d", W.gs_config(64), 50, lambda r: W.gs_perturb(r.get("u"), r.get("v"), 12))
