"""Batched Gray-Scott ensembles: every grid of a batch (mixed extents, its own
feed and kill rates) matches the same grid run alone, bit for bit, for every
batched kernel variant, with and without the CUDA-graph replay."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import Batch, Grid, builtin_program, program_uniforms
from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _members(count, seed):
    src, _ = builtin_program("gs2d")
    out = []
    for i, (n, F, k) in enumerate(W.ensemble(count, seed, nmin=40, nmax=300)):
        _, U = program_uniforms(src, W.gs_config(n), "gs2d", params={"F": F, "kappa": k})
        out.append((n, U, W.gs_square_state(n, 100 + i)))
    return out


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_batch_matches_single_grids(prec):
    members = _members(9, 1)
    steps = 70                                    # one graph chunk (64) + leftovers
    ref = []
    for n, U, x in members:
        g = Grid("gs2d", (n, n), prec, U)
        g.upload(x)
        g.forward(steps)
        ref.append(g.download())
        g.close()
    b = Batch("gs2d", [(n, n) for n, _, _ in members], prec, [U for _, U, _ in members])
    assert len(b.variants()) >= 4
    for v in b.variants():
        for i, (_, _, x) in enumerate(members):
            b.upload(i, x)
        b.set_variant(v["index"])
        b.forward(steps)
        for i in range(len(members)):
            assert bits_equal(b.download(i), ref[i]), (v, i)
    b.close()


def test_batch_autotune_keeps_state():
    members = _members(5, 2)
    b = Batch("gs2d", [(n, n) for n, _, _ in members], "f32", [U for _, U, _ in members])
    for i, (_, _, x) in enumerate(members):
        b.upload(i, x)
    before = [b.download(i) for i in range(len(members))]
    v = b.autotune(16)
    assert v == b.variant
    for i in range(len(members)):
        assert bits_equal(b.download(i), before[i])
    b.close()
