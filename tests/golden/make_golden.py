"""Writes the golden fixtures of tests/golden from the reference's own
programs, run through the restated Formura generator (the oracle):

* examples/diffusion3/diffusion3.fmr on a 16^3 grid (heat workload);
* examples/pearson2/pearson2.fmr with the Gray-Scott workload's feed rate
  f = 0.04 (the other parameters already match) on 64^2;
* sample/3d_hllc/3d_hllc.fmr with Courant number 0.4 on 16^3;
* sample/mhd_3d_hlld/mhd_3d_hlld.fmr on 12^3 (magnetised random state).

Each fixture stores the seeded input state, the config, the step count and
the output state and grid offset.  The shipped programs (heat3d, gs2d,
hllc3d, hlld3d) must reproduce them bit for bit.

A fifth fixture, sod1d_t100, holds the exact Riemann solution table of
sample/1d_hllc (ref_data/exact.dat: x, rho, u, p, e at step 100) and the
primitive profile of that sample's own program after 100 steps through the
oracle, the accuracy a shock-tube run of the shipped sod1d program is held to.  Needs the reference tree; run from
the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from formura_gb300 import workloads as W  # noqa: E402
from oracle.reference_lib import ReferenceProgram  # noqa: E402

REF = os.environ.get("FORMURA_REFERENCE", "/root/reference")
OUT = os.path.dirname(os.path.abspath(__file__))


def reference_source(path, edits=()):
    with open(os.path.join(REF, path)) as f:
        src = f.read()
    for old, new in edits:
        assert old in src, old
        src = src.replace(old, new)
    return src


def make(name, src, cfg, steps, state_fn, field_map):
    ref = ReferenceProgram(src, cfg, f"mkgold_{name}")
    ref.init()
    st = state_fn(ref)
    for mine, theirs in field_map.items():
        ref.set(theirs, st[mine])
    nav = ref.forward(steps)
    d = {"config": cfg, "steps": steps, "offset_x": nav["offset_x"], "time_step": nav["time_step"]}
    for mine, theirs in field_map.items():
        d["in_" + mine] = st[mine]
        d["out_" + mine] = ref.get(theirs)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **d)
    print("wrote", name)


def make_sod(name="sod1d_t100", steps=100):
    exact = np.loadtxt(os.path.join(REF, "sample/1d_hllc/ref_data/exact.dat"))
    ref = ReferenceProgram(reference_source("sample/1d_hllc/hllc.fmr"),
                           reference_source("sample/1d_hllc/config.yaml"), "mkgold_sod")
    ref.init()
    nav = ref.forward(steps)
    rho = ref.get("rho")
    u = ref.get("rhou") / rho
    ek = 0.5 * rho * (u * u + (ref.get("rhov") / rho) ** 2 + (ref.get("rhow") / rho) ** 2)
    p = 0.4 * (ref.get("e") - ek)
    x = np.array([ref.to_pos("x", i) for i in range(rho.size)])
    np.savez_compressed(os.path.join(OUT, name + ".npz"), exact_x=exact[:, 0], exact_rho=exact[:, 1],
                        exact_u=exact[:, 2], exact_p=exact[:, 3], sample_x=x, sample_rho=rho, sample_u=u,
                        sample_p=p, steps=steps, time_step=nav["time_step"])
    print("wrote", name)


if __name__ == "__main__":
    make("heat3d_16_10", reference_source("examples/diffusion3/diffusion3.fmr"), W.heat_config(16), 10,
         lambda r: W.heat_state((16, 16, 16), 11), {"q": "q"})
    make("gs2d_64_50", reference_source("examples/pearson2/pearson2.fmr",
                                        [("double :: f = 0.03", "double :: f = 0.04")]),
         W.gs_config(64), 50,
         lambda r: W.gs_perturb(np.ones((64, 64)), np.zeros((64, 64)), 12), {"u": "u", "v": "v"})
    make("hllc3d_16_5", reference_source("sample/3d_hllc/3d_hllc.fmr",
                                         [("double :: C_cfl = 0.8", "double :: C_cfl = 0.4")]),
         W.hllc_config(16), 5, lambda r: W.hllc_state((16, 16, 16), 13),
         {"e": "e", "mx": "rhou", "my": "rhov", "mz": "rhow", "rho": "rho"})
    make("hlld3d_12_3", reference_source("sample/mhd_3d_hlld/mhd_3d_hlld.fmr"), W.mhd_config(12), 3,
         lambda r: W.mhd_state((12, 12, 12), 14),
         {"bx": "B_x", "by": "B_y", "bz": "B_z", "e": "e", "mx": "rhou", "my": "rhov", "mz": "rhow",
          "psi": "psi", "rho": "rho"})
    make_sod()
