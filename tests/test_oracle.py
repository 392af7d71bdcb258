"""The oracle (the reference generator's C, restated) checked on the CPU.

Pins, in the absence of numeric golden vectors in the reference (its tests
cover config decoding only, test/NumericalConfigSpec.hs):
* temporal blocking and no blocking give identical states (two independent
  code paths of Templates.hs: 300-310 versus 311-381);
* the generated loop nests equal independent numpy restatements of the
  stencils bit for bit, including the per-step roll of the array content;
* committed golden fixtures (tests/golden, made by make_golden.py) are
  reproduced, so the oracle is the same on every machine;
* the reference's own example programs compile and behave the same way
  (when the reference tree is available).
"""
import os

import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import builtin_program
from oracle.reference_lib import ReferenceProgram

from conftest import REFERENCE as REF
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def heat_numpy(q, steps, dx):
    """Independent restatement of heat3d.fmr's update, same operation order."""
    dt = (0.1 * dx) * dx
    for _ in range(steps):
        def curv(ax):
            return ((np.roll(q, -1, ax) + np.roll(q, 1, ax)) - 2.0 * q) / dx ** 2
        q = q + dt * ((curv(0) + curv(1)) + curv(2))
        q = np.roll(q, (1, 1, 1), (0, 1, 2))
    return q


def gs_numpy(u, v, steps, dx):
    Du, Dv, F, k = 2.0e-5, 1.0e-5, 0.04, 0.06
    c = dx * dx
    for _ in range(steps):
        def lap(a):
            return ((np.roll(a, -1, 0) + np.roll(a, 1, 0)) - 2.0 * a) / c + \
                   ((np.roll(a, -1, 1) + np.roll(a, 1, 1)) - 2.0 * a) / c
        un = u + ((Du * lap(u) - (u * v) * v) + F * (1.0 - u))
        vn = v + ((Dv * lap(v) + (u * v) * v) - (F + k) * v)
        u = np.roll(un, (1, 1), (0, 1))
        v = np.roll(vn, (1, 1), (0, 1))
    return u, v


def test_heat_oracle_equals_numpy_bitwise():
    n = 12
    src, _ = builtin_program("heat3d")
    ref = ReferenceProgram(src, W.heat_config(n), "heat_np")
    ref.init()
    x = W.heat_state((n, n, n), 5)["q"]
    ref.set("q", x)
    nav = ref.forward(7)
    assert nav["time_step"] == 7 and nav["offset_x"] == n - 7
    assert np.array_equal(ref.get("q"), heat_numpy(x, 7, 1.0 / n))


def test_gs_oracle_equals_numpy_bitwise():
    n = 32
    src, _ = builtin_program("gs2d")
    ref = ReferenceProgram(src, W.gs_config(n), "gs_np")
    ref.init()
    u0, v0 = ref.get("u"), ref.get("v")
    inside = (np.arange(n) > 0.45 * n) & (np.arange(n) < 0.55 * n)
    sq = inside[:, None] & inside[None, :]
    assert np.array_equal(u0, np.where(sq, 0.5, 1.0)) and np.array_equal(v0, np.where(sq, 0.25, 0.0))
    st = W.gs_perturb(u0, v0, 4)
    ref.set("u", st["u"])
    ref.set("v", st["v"])
    ref.forward(20)
    u, v = gs_numpy(st["u"], st["v"], 20, 0.01)
    assert np.array_equal(ref.get("u"), u) and np.array_equal(ref.get("v"), v)


def test_temporal_blocking_equals_no_blocking():
    src, _ = builtin_program("heat3d")
    n = 12
    nb = ReferenceProgram(src, W.heat_config(n), "heat_nb")
    tb = ReferenceProgram(src, W.heat_config(n, extra="grid_per_block: [4, 4, 4]\n"
                                                     "temporal_blocking_interval: 2\n"), "heat_tb")
    nb.init()
    tb.init()
    x = W.heat_state((n, n, n), 1)["q"]
    nb.set("q", x)
    tb.set("q", x)
    nb.forward(6)
    tb.forward(3)
    assert nb.navi_dict() == tb.navi_dict()
    assert np.array_equal(nb.get("q"), tb.get("q"))


@pytest.mark.parametrize("name,program", [("heat3d_16_10", "heat3d"), ("gs2d_64_50", "gs2d"),
                                          ("hllc3d_16_5", "hllc3d"), ("hlld3d_12_3", "hlld3d")])
def test_golden_fixture_reproduced(name, program):
    """The shipped programs reproduce, bit for bit, the reference's own
    example programs (fixtures made by tests/golden/make_golden.py)."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    src, _ = builtin_program(program)
    ref = ReferenceProgram(src, str(d["config"]), f"golden_{name}")
    ref.init()
    for f in ref.fields:
        ref.set(f, d["in_" + f])
    nav = ref.forward(int(d["steps"]))
    for f in ref.fields:
        assert np.array_equal(ref.get(f), d["out_" + f]), f
    assert nav["offset_x"] == int(d["offset_x"]) and nav["time_step"] == int(d["time_step"])


def _ref_file(*p):
    path = os.path.join(REF, *p)
    if not os.path.exists(path):
        pytest.skip("reference tree not available")
    return open(path).read()


def test_reference_diffusion3_blocking_paths_agree():
    src = _ref_file("examples", "diffusion3", "diffusion3.fmr")
    tb_cfg = _ref_file("examples", "diffusion3", "diffusion3.yaml")
    tb = ReferenceProgram(src, tb_cfg, "ref_d3_tb")
    nb = ReferenceProgram(src, "length_per_node: [1.0,1.0,1.0]\ngrid_per_node: [100,100,100]\n", "ref_d3_nb")
    for p in (tb, nb):
        p.init()
    assert np.array_equal(tb.get("q"), nb.get("q"))
    x = W.heat_state((100, 100, 100), 3)["q"]
    tb.set("q", x)
    nb.set("q", x)
    tb.forward(2)
    nb.forward(10)
    assert tb.navi_dict() == nb.navi_dict()
    assert np.array_equal(tb.get("q"), nb.get("q"))
    # examples/diffusion3/diffusion3.fmr: (q[i+1] + q[i-1] - 2*q[i])/dx**2
    q, dx = x, 0.01
    dt = (0.1 * dx) * dx
    for _ in range(10):
        def d2(ax):
            return ((np.roll(q, -1, ax) + np.roll(q, 1, ax)) - 2.0 * q) / dx ** 2
        q = np.roll(q + dt * ((d2(0) + d2(1)) + d2(2)), (1, 1, 1), (0, 1, 2))
    assert np.array_equal(nb.get("q"), q)


def test_reference_samples_compile():
    from formura_gb300.generator.config import decode_config
    from formura_gb300.generator.manifest import compile_program
    cases = {("sample", "3d_hllc", "3d_hllc.fmr", "config.yaml"): (2, 64, ["e", "rho", "rhou", "rhov", "rhow"]),
             ("sample", "1d_hllc", "hllc.fmr", "config.yaml"): (2, 28, ["e", "rho", "rhou", "rhov", "rhow"]),
             ("sample", "mhd_3d_hlld", "mhd_3d_hlld.fmr", "config.yaml"): (2, 108, None),
             ("examples", "pearson2", "pearson2.fmr", "pearson2.yaml"): (1, 2, ["u", "v"])}
    for (a, b, f, y), (sleeve, nman, fields) in cases.items():
        mm = compile_program(_ref_file(a, b, f), decode_config(_ref_file(a, b, y)))
        assert mm.om.config.sleeve == sleeve
        assert len(mm.step) == nman
        if fields:
            assert mm.fields == fields


def test_sod_shock_tube_oracle_matches_exact_solution():
    """Physics pin of the oracle: the shipped 1D shock-tube program, run 100
    steps through the restated generator, against the exact Riemann solution
    table of the reference's 1D HLLC sample (tests/golden/sod1d_t100.npz).
    Its L1 error over the waves equals that of the sample's own program."""
    from formura_gb300.host import builtin_program
    src, cfg = builtin_program("sod1d")
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "sod1d_t100.npz"))
    r = ReferenceProgram(src, cfg, "sod_oracle")
    r.init()
    nav = r.forward(100)
    assert nav["time_step"] == int(d["time_step"]) == 100
    rho = r.get("rho")
    u = r.get("m") / rho
    p = 0.4 * (r.get("e") - 0.5 * rho * u * u)
    x = np.array([r.to_pos("x", i) for i in range(rho.size)])
    sel = (x > 1.2) & (x < 2.8)
    xs = d["sample_x"]
    ss = (xs > 1.2) & (xs < 2.8)
    for name, v in (("rho", rho), ("u", u), ("p", p)):
        err = np.mean(np.abs(v[sel] - np.interp(x[sel], d["exact_x"], d["exact_" + name])))
        err_sample = np.mean(np.abs(d["sample_" + name][ss] - np.interp(xs[ss], d["exact_x"], d["exact_" + name])))
        assert err < 0.01 and err <= 1.01 * err_sample + 1e-12, (name, err, err_sample)



def _physical(ref, field):
    """A field of formura_data in physical order: index i holds position
    (i + offset) mod N (Templates.hs:221-225, 346)."""
    nav = ref.navi_dict()
    a = ref.get(field)
    return np.roll(a, tuple(nav[f"offset_{ax}"] for ax in "xyz"), (0, 1, 2))


def _euler_case(ref, names, length, c_cfl, steps, seed):
    """Steps the oracle and the numpy restatement of 3d_hllc.fmr from the
    same smooth state; returns the largest relative max-norm difference and
    whether every field agrees bit for bit."""
    import numpy_euler as NE
    ref.init()
    shape = ref.shape
    st = W.hllc_state(shape, seed=seed)
    rho, m, e = st["rho"], (st["mx"], st["my"], st["mz"]), st["e"]
    for name, val in zip(names, (rho, m[0], m[1], m[2], e)):
        ref.set(name, val)
    ref.forward(steps)
    E = NE.Euler3D(shape, length, c_cfl=c_cfl)
    for _ in range(steps):
        rho, m, e = E.step(rho, m, e)
    worst, exact = 0.0, True
    for name, val in zip(names, (rho, m[0], m[1], m[2], e)):
        got = _physical(ref, name)
        worst = max(worst, float(np.abs(got - val).max() / np.abs(val).max()))
        exact = exact and np.array_equal(got, val)
    return worst, exact


def test_hllc_oracle_equals_numpy_restatement():
    """The shipped hllc3d program through the oracle against the numpy
    restatement of the reference's 3d_hllc.fmr (no shared front end):
    5 steps at 12^3 from the smooth Mach-0.3 state, CFL 0.4."""
    n = 12
    src, _ = builtin_program("hllc3d")
    ref = ReferenceProgram(src, W.hllc_config(n), "hllc_np")
    worst, exact = _euler_case(ref, ("rho", "mx", "my", "mz", "e"), (1.0, 1.0, 1.0), 0.4, 5, 3)
    assert exact, f"largest relative difference {worst}"


def test_reference_3d_hllc_oracle_equals_numpy_restatement():
    """The reference's own 3d_hllc.fmr (its CFL 0.8 and box) through the
    oracle, against the same numpy restatement: 4 steps at 12 x 12 x 12."""
    path = os.path.join(REF, "sample", "3d_hllc", "3d_hllc.fmr")
    if not os.path.exists(path):
        pytest.skip("the reference tree is not present")
    with open(path) as f:
        src = f.read()
    cfg = "length_per_node: [0.1, 0.5, 0.1]\ngrid_per_node: [12, 12, 12]\n"
    ref = ReferenceProgram(src, cfg, "ref3dhllc_np")
    worst, exact = _euler_case(ref, ("rho", "rhou", "rhov", "rhow", "e"), (0.1, 0.5, 0.1), 0.8, 4, 5)
    assert exact, f"largest relative difference {worst}"


def _mhd_case(ref, names, length, steps, seed):
    """As _euler_case, for the HLLD program (9 fields, psi seeded too)."""
    import numpy_mhd as NM
    ref.init()
    shape = ref.shape
    st = W.mhd_state(shape, seed=seed)
    st["psi"] = 0.01 * np.random.default_rng(seed + 1).standard_normal(shape)
    comps = [st[k] for k in ("rho", "mx", "my", "mz", "bx", "by", "bz", "e", "psi")]
    for name, val in zip(names, comps):
        ref.set(name, val)
    ref.forward(steps)
    M = NM.MHD3D(shape, length)
    for _ in range(steps):
        comps = M.step(comps)
    worst, exact = 0.0, True
    for name, val in zip(names, comps):
        got = _physical(ref, name)
        worst = max(worst, float(np.abs(got - val).max() / np.abs(val).max()))
        exact = exact and np.array_equal(got, val)
    return worst, exact


def test_hlld_oracle_equals_numpy_restatement():
    """The shipped hlld3d program through the oracle against the numpy
    restatement of the reference's mhd_3d_hlld.fmr: 3 steps at 10^3."""
    n = 10
    src, _ = builtin_program("hlld3d")
    ref = ReferenceProgram(src, W.mhd_config(n), "hlld_np")
    worst, exact = _mhd_case(ref, ("rho", "mx", "my", "mz", "bx", "by", "bz", "e", "psi"),
                             (1.0, 1.0, 1.0), 3, 2)
    assert exact, f"largest relative difference {worst}"


def test_reference_mhd_3d_hlld_oracle_equals_numpy_restatement():
    """The reference's own mhd_3d_hlld.fmr through the oracle, against the
    same numpy restatement: 3 steps at 10 x 10 x 6 of its box."""
    path = os.path.join(REF, "sample", "mhd_3d_hlld", "mhd_3d_hlld.fmr")
    if not os.path.exists(path):
        pytest.skip("the reference tree is not present")
    with open(path) as f:
        src = f.read()
    length = (3.141592653589793, 3.141592653589793, 0.15707963267948966)
    cfg = f"length_per_node: [{length[0]}, {length[1]}, {length[2]}]\ngrid_per_node: [10, 10, 6]\n"
    ref = ReferenceProgram(src, cfg, "refmhd_np")
    worst, exact = _mhd_case(ref, ("rho", "rhou", "rhov", "rhow", "B_x", "B_y", "B_z", "e", "psi"),
                             length, 3, 4)
    assert exact, f"largest relative difference {worst}"
