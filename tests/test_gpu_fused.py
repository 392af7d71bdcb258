"""Temporal-blocking kernels (several steps per launch in shared-memory
tiles): every variant gives the same state as one step per launch, bit for
bit in FP64 and FP32, including grids that are not multiples of the tile and
step counts that are not multiples of the fused depth, and grids shorter
than a tile's halo (every index wraps through the modulo path)."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import Grid, Library, builtin_program, program_uniforms
from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _state(shape, seed):
    st = W.gs_perturb(np.ones(shape), np.zeros(shape), seed)
    u, v = st["u"], st["v"]
    # a square of active pattern so both fields vary
    c = tuple(slice(s // 3, 2 * s // 3) for s in shape)
    u[c] = 0.5 + 0.01 * np.random.default_rng(seed).random(u[c].shape)
    v[c] = 0.25
    return np.stack([u, v])


@pytest.mark.parametrize("shape", [(256, 256), (100, 70), (64, 200), (3, 5), (1, 9)])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_every_variant_matches_single_steps(shape, prec):
    src, _ = builtin_program("gs2d")
    _, U = program_uniforms(src, W.gs_config(shape[0]), "gs2d")
    x = _state(shape, 1)
    steps = 37
    g = Grid("gs2d", shape, prec, U)
    g.upload(x)
    g.forward(steps)
    ref = g.download()
    assert len(g.variants()) >= 4
    for v in g.variants():
        g.upload(x)
        try:
            g.set_variant(v["index"])
        except Exception:
            continue            # does not fit this device's shared memory
        g.forward(steps)
        got = g.download()
        assert bits_equal(got, ref), v
    g.close()


def test_autotune_preserves_state_and_picks_a_variant():
    shape = (512, 512)
    src, _ = builtin_program("gs2d")
    _, U = program_uniforms(src, W.gs_config(shape[0]), "gs2d")
    x = _state(shape, 2)
    g = Grid("gs2d", shape, "f32", U)
    g.upload(x)
    before = g.download()
    chosen = g.autotune(32)
    assert chosen >= -1 and g.variant == chosen
    assert bits_equal(g.download(), before)
    g.close()


def test_f16_fused_close_to_f32():
    shape = (256, 256)
    src, _ = builtin_program("gs2d")
    _, U = program_uniforms(src, W.gs_config(shape[0]), "gs2d")
    x = _state(shape, 3)
    a = Grid("gs2d", shape, "f32", U)
    a.upload(x)
    a.forward(64)
    b = Grid("gs2d", shape, "f16", U, scales=[1.0, 0.5])
    b.upload(x)
    b.autotune(16)
    b.forward(64)
    fa, fb = a.download(), b.download()
    for i in range(2):
        assert W.rel_l2(fb[i], fa[i]) < 2e-2


@pytest.mark.parametrize("shape", [(48, 48, 48), (40, 50, 70), (8, 40, 36), (96, 20, 130), (40, 72, 128), (3, 5, 4),
                                   (1, 2, 7)])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_3d_streaming_variants_match_single_steps(shape, prec):
    """The 2.5D streaming kernels (K steps per launch, planes of the slowest
    axis in a shared-memory ring) equal one step per launch bit for bit."""
    src, _ = builtin_program("heat3d")
    _, U = program_uniforms(src, W.heat_config(shape[2]), "heat3d")
    x = np.random.default_rng(5).random((1,) + shape)
    steps = 37
    g = Grid("heat3d", shape, prec, U)
    g.upload(x)
    g.forward(steps)
    ref = g.download()
    variants = g.variants()
    assert len(variants) >= 4
    tried = 0
    for v in variants:
        g.upload(x)
        try:
            g.set_variant(v["index"])
        except Exception:
            continue            # does not fit this device's shared memory
        tried += 1
        g.forward(steps)
        got = g.download()
        assert bits_equal(got, ref), v
    assert tried >= 3
    g.close()


@pytest.mark.parametrize("shape", [(48, 48, 48), (8, 40, 36), (40, 72, 128), (3, 5, 4), (20, 9, 260)])
def test_3d_one_step_variants_match_in_f16(shape):
    """With FP16 storage every step stores half values, so the one-step
    variants (four-point row vectors) equal the generic stage kernel bit for
    bit as well; the multi-step tiles keep FP32 values between their steps
    and are left out here."""
    src, _ = builtin_program("heat3d")
    _, U = program_uniforms(src, W.heat_config(shape[2]), "heat3d")
    x = np.random.default_rng(6).random((1,) + shape)
    steps = 13
    g = Grid("heat3d", shape, "f16", U, scales=[1.0])
    g.upload(x)
    g.forward(steps)
    ref = g.download()
    tried = 0
    for v in g.variants():
        if v["steps"] != 1:
            continue
        g.upload(x)
        g.set_variant(v["index"])
        tried += 1
        g.forward(steps)
        assert bits_equal(g.download(), ref), v
    assert tried >= 2
    g.close()


@pytest.mark.parametrize("program,shape", [("hllc3d", (24, 24, 24)), ("hllc3d", (20, 30, 18)),
                                           ("hllc3d", (7, 9, 13)), ("hllc3d", (40, 16, 33)),
                                           ("hlld3d", (12, 14, 10)), ("hlld3d", (24, 24, 24))])
@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f16", 3e-3)])
def test_multistage_fused_variants(program, shape, prec, tol):
    """The one-launch multi-stage kernels (every stage's arrays in
    shared-memory plane rings, 2.5D streaming) give the same bits for every
    tile shape, so the rings and halos do not depend on the tiling.  Against
    the stage-per-kernel path they agree to FP32 rounding: both run the same
    generated stage functors, but nvcc contracts a product and a sum into one
    FMA where it sees fit, and its choices differ between the two kernels
    (HLLD FP32: about 0.4 % of the points differ after one step, by at most
    9e-6 relative; after nine steps the GLM field psi is 1.6e-6 apart in
    relative L2).  Relative L2 bound per field: 1e-5, the FP32 form's error
    bound against FP64 (FP32), 3e-3 (FP16
    storage, whose 11-bit rounding turns a one-ulp FP32 difference into one
    FP16 ulp, 5e-4 relative, at the points where the rounding flips)."""
    src, _ = builtin_program(program)
    cfg = {"hllc3d": W.hllc_config, "hlld3d": W.mhd_config}[program](shape[2])
    _, U = program_uniforms(src, cfg, program)
    st = (W.hllc_state if program == "hllc3d" else W.mhd_state)(shape, seed=4)
    fields = Library.get().fields(program)
    x = np.stack([st[f] for f in fields])
    sc = [float(max(1e-3, np.abs(x[i]).max())) for i in range(len(fields))] if prec == "f16" else None
    steps = 9
    g = Grid(program, shape, prec, U, scales=sc)
    g.upload(x)
    g.forward(steps)
    ref = g.download()
    first = None
    tried = 0
    for v in g.variants():
        g.upload(x)
        try:
            g.set_variant(v["index"])
        except Exception:
            continue            # needs more shared memory than this device has
        tried += 1
        g.forward(steps)
        got = g.download()
        if first is None:
            first = got
        assert bits_equal(got, first), v
        for i in range(len(fields)):
            assert W.rel_l2(got[i], ref[i]) <= tol, (v, fields[i], W.rel_l2(got[i], ref[i]))
    assert tried >= 2
    g.close()
