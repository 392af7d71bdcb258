"""Parity of the GB300 drop-in against the oracle, through the generated C API.

Both sides are driven exactly like a Formura driver program: Formura_Init,
the seeded state written into formura_data, Formura_Forward called in a loop,
formura_data and Formura_Navi read back.  The FP64 form must match the
oracle bit for bit (rel-L2 0, well inside the 1e-12 bound); integer grid
indexing (offset_*, time_step) must be identical.
"""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import FormuraProgram, builtin_program
from oracle.reference_lib import ReferenceProgram
from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _pair(program, cfg_text, gpu_extra="", tag="t"):
    src, _ = builtin_program(program)
    ref = ReferenceProgram(src, cfg_text, f"{program}_{tag}_ref")
    gpu = FormuraProgram(src, cfg_text + gpu_extra, program, name=f"{program}_{tag}_gpu")
    return ref, gpu


def _check_navi(a, b):
    assert a == b, (a, b)


@pytest.mark.parametrize("n,steps,spf", [(16, 9, 1), (32, 40, 8), (20, 33, 11)])
def test_heat_f64_bit_exact(n, steps, spf):
    cfg = W.heat_config(n)
    ref, gpu = _pair("heat3d", cfg, f"gpu_steps_per_forward: {spf}\n", f"n{n}s{spf}")
    _check_navi(ref.init(), gpu.init())
    x = W.heat_state((n, n, n), seed=n)["q"]
    ref.set("q", x)
    gpu.set("q", x)
    calls = steps // spf
    for _ in range(calls):
        ref.forward(spf)
        gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    a, b = ref.get("q"), gpu.get("q")
    assert bits_equal(a, b), f"max |diff| {np.abs(a - b).max()}"
    gpu.finalize()


def test_heat_full_config_bit_exact():
    """128^3, D*dt/dx^2 = 0.1, 1000 steps, uniform [0,1) from a seed."""
    n, steps = 128, 1000
    cfg = W.heat_config(n)
    ref, gpu = _pair("heat3d", cfg, "gpu_steps_per_forward: 1000\n", "full")
    ref.init()
    gpu.init()
    x = W.heat_state((n, n, n), seed=0)["q"]
    ref.set("q", x)
    gpu.set("q", x)
    ref.forward(steps)
    gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    a, b = ref.get("q"), gpu.get("q")
    assert bits_equal(a, b), f"rel-L2 {W.rel_l2(b, a)}"
    # the periodic explicit scheme conserves the total up to rounding
    assert abs(b.sum() - x.sum()) < 1e-9 * x.size
    gpu.finalize()


@pytest.mark.parametrize("n,steps,spf", [(64, 50, 1), (96, 300, 50)])
def test_gray_scott_f64_bit_exact(n, steps, spf):
    cfg = W.gs_config(n)
    ref, gpu = _pair("gs2d", cfg, f"gpu_steps_per_forward: {spf}\n", f"n{n}s{spf}")
    _check_navi(ref.init(), gpu.init())
    for f in ("u", "v"):
        assert bits_equal(ref.get(f), gpu.get(f)), "init differs"
    st = W.gs_perturb(ref.get("u"), ref.get("v"), seed=7)
    for f in ("u", "v"):
        ref.set(f, st[f])
        gpu.set(f, st[f])
    for _ in range(steps // spf):
        ref.forward(spf)
        gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    for f in ("u", "v"):
        a, b = ref.get(f), gpu.get(f)
        assert bits_equal(a, b), f"{f}: max |diff| {np.abs(a - b).max()}"
    gpu.finalize()


def test_gray_scott_4096_bit_exact_200_steps():
    n, steps = 4096, 200
    cfg = W.gs_config(n)
    ref, gpu = _pair("gs2d", cfg, f"gpu_steps_per_forward: {steps}\n", "big")
    ref.init()
    gpu.init()
    st = W.gs_perturb(ref.get("u"), ref.get("v"), seed=0)
    for f in ("u", "v"):
        ref.set(f, st[f])
        gpu.set(f, st[f])
    ref.forward(steps)
    gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    for f in ("u", "v"):
        assert bits_equal(ref.get(f), gpu.get(f))
    gpu.finalize()


@pytest.mark.parametrize("prec,tol", [("f64fast", 1e-12), ("f32", 1e-5), ("f16", 5e-2)])
def test_gray_scott_reduced_precision(prec, tol):
    """FP32 / FP16 storage and FP64 with contraction: relative L2 against the
    FP64 oracle after 500 steps at 128^2 (tolerance stated per form)."""
    n, steps = 128, 500
    cfg = W.gs_config(n)
    extra = f"gpu_precision: {prec}\ngpu_steps_per_forward: {steps}\n"
    if prec == "f16":
        extra += "gpu_field_scales: [1.0, 0.5]\n"
    ref, gpu = _pair("gs2d", cfg, extra, prec)
    ref.init()
    gpu.init()
    st = W.gs_perturb(ref.get("u"), ref.get("v"), seed=3)
    for f in ("u", "v"):
        ref.set(f, st[f])
        gpu.set(f, st[f])
    ref.forward(steps)
    gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    for f in ("u", "v"):
        err = W.rel_l2(gpu.get(f), ref.get(f))
        assert err < tol, f"{prec} {f}: rel-L2 {err}"
    gpu.finalize()


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name,program", [("heat3d_16_10", "heat3d"), ("gs2d_64_50", "gs2d"),
                                          ("hllc3d_16_5", "hllc3d"), ("hlld3d_12_3", "hlld3d")])
def test_gpu_reproduces_reference_program_fixture(name, program):
    """The GPU reproduces, bit for bit, the output of the reference's own
    example program (diffusion3 / pearson2 / 3d_hllc) on the same input."""
    import os
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    src, _ = builtin_program(program)
    steps = int(d["steps"])
    gpu = FormuraProgram(src, str(d["config"]) + f"gpu_steps_per_forward: {steps}\n", program,
                         name=f"{program}_fix")
    gpu.init()
    for f in gpu.fields:
        gpu.set(f, d["in_" + f])
    nav = gpu.forward(1)
    assert nav["offset_x"] == int(d["offset_x"]) and nav["time_step"] == int(d["time_step"])
    for f in gpu.fields:
        assert bits_equal(gpu.get(f), d["out_" + f]), f
    gpu.finalize()


def test_hllc_f64_bit_exact_and_conservative():
    n, steps = 32, 24
    cfg = W.hllc_config(n)
    ref, gpu = _pair("hllc3d", cfg, f"gpu_steps_per_forward: 8\n", "n32")
    ref.init()
    gpu.init()
    st = W.hllc_state((n, n, n), seed=5)
    for f in ref.fields:
        ref.set(f, st[f])
        gpu.set(f, st[f])
    for _ in range(steps // 8):
        ref.forward(8)
        gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    for f in ref.fields:
        a, b = ref.get(f), gpu.get(f)
        assert bits_equal(a, b), f"{f}: rel-L2 {W.rel_l2(b, a)}"
        # periodic flux-difference form conserves every total
        assert abs(b.sum() - st[f].sum()) <= 1e-10 * max(1.0, np.abs(st[f]).sum())
    gpu.finalize()


def test_hllc_f32_storage():
    n, steps = 32, 24
    cfg = W.hllc_config(n)
    ref, gpu = _pair("hllc3d", cfg, f"gpu_precision: f32\ngpu_steps_per_forward: {steps}\n", "f32")
    ref.init()
    gpu.init()
    st = W.hllc_state((n, n, n), seed=6)
    for f in ref.fields:
        ref.set(f, st[f])
        gpu.set(f, st[f])
    ref.forward(steps)
    gpu.forward(1)
    for f in ("rho", "e"):
        err = W.rel_l2(gpu.get(f), ref.get(f))
        assert err < 1e-5, f"{f}: rel-L2 {err}"
    gpu.finalize()


def test_hlld_f64_bit_exact():
    n, steps = 20, 6
    cfg = W.mhd_config(n)
    ref, gpu = _pair("hlld3d", cfg, "gpu_steps_per_forward: 3\n", "n20")
    ref.init()
    gpu.init()
    st = W.mhd_state((n, n, n), seed=3)
    for f in ref.fields:
        ref.set(f, st[f])
        gpu.set(f, st[f])
    for _ in range(steps // 3):
        ref.forward(3)
        gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    for f in ref.fields:
        assert bits_equal(ref.get(f), gpu.get(f)), f
    gpu.finalize()


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_hllc_conserved_totals_fp64(prec):
    """FP64 totals of mass, momentum and energy over 50 steps of HLLC (FP64
    reductions also for FP32 storage)."""
    from formura_gb300.host import Grid, program_uniforms
    n = 32
    src, _ = builtin_program("hllc3d")
    _, U = program_uniforms(src, W.hllc_config(n), "hllc3d")
    st = W.hllc_state((n, n, n), seed=8)
    x = np.stack([st[f] for f in ("e", "mx", "my", "mz", "rho")])
    g = Grid("hllc3d", (n, n, n), prec, U)
    g.upload(x)
    t0 = g.totals()
    stored = x if prec == "f64" else x.astype(np.float32).astype(np.float64)
    assert np.allclose(t0, stored.reshape(5, -1).sum(axis=1), rtol=1e-12, atol=1e-12)
    g.forward(50)
    t1 = g.totals()
    scale = np.abs(x).reshape(5, -1).sum(axis=1)
    drift = np.abs(t1 - t0) / scale
    assert (drift < (1e-13 if prec == "f64" else 1e-5)).all(), drift
    g.close()


def _sod_profile(p):
    rho = p.get("rho")
    u = p.get("m") / rho
    pr = 0.4 * (p.get("e") - 0.5 * rho * u * u)
    x = np.array([p.to_pos("x", i) for i in range(rho.size)])
    return x, rho, u, pr


def test_sod_shock_tube_bit_exact_and_accurate():
    """1D shock tube, 400 cells, 100 steps through the drop-in: bit-identical
    to the oracle, and as close to the exact Riemann solution of the
    reference's 1D HLLC sample (L1 over the waves) as that sample's own
    program is."""
    import os
    src, cfg = builtin_program("sod1d")
    ref, gpu = _pair("sod1d", cfg, "", "sod")
    _check_navi(ref.init(), gpu.init())
    for f in ("e", "m", "rho"):
        assert bits_equal(ref.get(f), gpu.get(f))
    ref.forward(100)
    for _ in range(100):
        gpu.forward(1)
    _check_navi(ref.navi_dict(), gpu.navi_dict())
    for f in ("e", "m", "rho"):
        assert bits_equal(ref.get(f), gpu.get(f)), f
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "sod1d_t100.npz"))
    x, rho, u, pr = _sod_profile(gpu)
    sel = (x > 1.2) & (x < 2.8)
    for name, v in (("rho", rho), ("u", u), ("p", pr)):
        err = np.mean(np.abs(v[sel] - np.interp(x[sel], d["exact_x"], d["exact_" + name])))
        xs = d["sample_x"]
        ss = (xs > 1.2) & (xs < 2.8)
        err_sample = np.mean(np.abs(d["sample_" + name][ss] - np.interp(xs[ss], d["exact_x"], d["exact_" + name])))
        assert err <= 1.01 * err_sample + 1e-12, (name, err, err_sample)
    gpu.finalize()


def test_two_grids_interleaved_match_sequential_runs():
    """Two grids of different programs, each on its own stream, advanced in
    interleaved calls give the same bits as when each runs alone."""
    from formura_gb300.host import Grid, program_uniforms
    src_h, _ = builtin_program("heat3d")
    src_g, _ = builtin_program("gs2d")
    _, Uh = program_uniforms(src_h, W.heat_config(32), "heat3d")
    _, Ug = program_uniforms(src_g, W.gs_config(128), "gs2d")
    xh = W.heat_state((32, 32, 32), seed=4)["q"][None]
    st = W.gs_perturb(np.ones((128, 128)), np.zeros((128, 128)), 5)
    xg = np.stack([st["u"], st["v"]])
    alone = []
    for prog, shape, U, x in (("heat3d", (32, 32, 32), Uh, xh), ("gs2d", (128, 128), Ug, xg)):
        g = Grid(prog, shape, "f64", U)
        g.upload(x)
        g.forward(30)
        alone.append(g.download())
        g.close()
    a = Grid("heat3d", (32, 32, 32), "f64", Uh)
    b = Grid("gs2d", (128, 128), "f64", Ug)
    a.upload(xh)
    b.upload(xg)
    for _ in range(10):
        a.forward(3)
        b.forward(3)
    assert bits_equal(a.download(), alone[0])
    assert bits_equal(b.download(), alone[1])
    a.close()
    b.close()


def _tiny(rng, shape, scale_exp):
    """Values around 2^scale_exp (subnormal for scale_exp < -1022), a fifth
    of them exact +0 and a fifth exact -0."""
    x = rng.uniform(-1.0, 1.0, shape) * 2.0 ** scale_exp
    r = rng.random(shape)
    x[r < 0.2] = 0.0
    x[(r >= 0.2) & (r < 0.4)] = -0.0
    return x


@pytest.mark.parametrize("program,n", [("heat3d", 12), ("heat3d", 16), ("gs2d", 32), ("sod1d", None),
                                       ("hllc3d", 8)])
def test_tiny_values_and_signed_zeros_bit_exact(program, n):
    """States with subnormal and tiny values and signed zeros, where the
    shortened division and multiply-add forms of the exact policy must hand
    over to the IEEE instructions: bit patterns (zero signs included) equal
    to the oracle's after every call."""
    rng = np.random.default_rng(11)
    if program == "heat3d":
        cfg = W.heat_config(n)      # 1/dx^2 a power of two for n = 16, not for n = 12
    elif program == "gs2d":
        cfg = W.gs_config(n)
    elif program == "hllc3d":
        cfg = W.hllc_config(n)
    else:
        _, cfg = builtin_program(program)
    ref, gpu = _pair(program, cfg, "", f"tiny{n}")
    ref.init()
    gpu.init()
    shape = ref.get(ref.fields[0]).shape
    st = {}
    if program == "heat3d":
        st["q"] = _tiny(rng, shape, -1030)
        st["q"][:, :, : n // 2] = _tiny(rng, (n, n, n // 2), -950)
    elif program == "gs2d":
        st["u"] = 1.0 - 0.1 * rng.random(shape)
        st["v"] = _tiny(rng, shape, -1040)
        st["v"][: n // 2] = _tiny(rng, (n // 2, n), -960)
        st["v"][n // 4: n // 2, n // 4: n // 2] = 0.25
    else:
        for f in ref.fields:
            st[f] = ref.get(f).copy()
        momenta = [f for f in ref.fields if f.startswith("m")]
        for f in momenta:
            st[f] = _tiny(rng, shape, -1030)
            st[f].reshape(-1)[::3] = 0.1 * rng.uniform(-1, 1, st[f].reshape(-1)[::3].shape)
    for f in ref.fields:
        ref.set(f, st[f])
        gpu.set(f, st[f])
    for _ in range(6):
        ref.forward(1)
        gpu.forward(1)
        for f in ref.fields:
            assert bits_equal(ref.get(f), gpu.get(f)), f
    gpu.finalize()


def test_gray_scott_decay_through_subnormals_bit_exact():
    """Gray-Scott without a pattern: v decays by about e^-0.1 per step, so a
    field of +-1e-300 enters the subnormal range after some 180 steps (the
    regime of the 4096^2 run's far field after some 7000 steps).
    The state after every 50 steps equals the oracle's bit for bit."""
    n = 64
    cfg = W.gs_config(n)
    ref, gpu = _pair("gs2d", cfg, "gpu_steps_per_forward: 50\n", "decay")
    ref.init()
    gpu.init()
    rng = np.random.default_rng(5)
    u = 1.0 - 0.01 * rng.random((n, n))
    v = 1e-300 * rng.uniform(-1.0, 1.0, (n, n))
    for f, x in (("u", u), ("v", v)):
        ref.set(f, x)
        gpu.set(f, x)
    subnormal_seen = False
    for _ in range(8):
        ref.forward(50)
        gpu.forward(1)
        a = ref.get("v")
        subnormal_seen |= bool(((a != 0) & (np.abs(a) < 2.2250738585072014e-308)).any())
        for f in ("u", "v"):
            assert bits_equal(ref.get(f), gpu.get(f)), f
    assert subnormal_seen
    gpu.finalize()
