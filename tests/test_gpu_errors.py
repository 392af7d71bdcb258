"""Error behaviour of the C ABI on a GPU: every bad request comes back as a
status code with a message (fgb_last_error), the grid stays usable, and no
call falls back to the host."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import FgbError, Grid, Library, builtin_program, program_uniforms

pytestmark = pytest.mark.gpu


def _gs_uniforms(n=64):
    src, _ = builtin_program("gs2d")
    return program_uniforms(src, W.gs_config(n), "gs2d")[1]


def test_unknown_program():
    with pytest.raises(FgbError, match="unknown program"):
        Library.get().query("no_such_program")


def test_bad_open_arguments():
    U = _gs_uniforms()
    with pytest.raises(FgbError, match="2-dimensional"):
        Grid("gs2d", (64, 64, 64), "f64", U)
    with pytest.raises(FgbError, match="uniform values"):
        Grid("gs2d", (64, 64), "f64", U[:-1])
    with pytest.raises(FgbError, match="points away"):
        Grid("hllc3d", (1, 16, 16), "f64", [0.0] * Library.get().query("hllc3d")["nuniforms"])


def test_bad_variant_and_recovery():
    U = _gs_uniforms()
    g = Grid("gs2d", (64, 64), "f32", U)
    x = np.stack([np.ones((64, 64)), np.zeros((64, 64))])
    g.upload(x)
    with pytest.raises(FgbError, match="no such variant"):
        g.set_variant(len(g.variants()) + 3)
    g.forward(3)                       # the grid still works after the error
    assert np.isfinite(g.download()).all()
    g.close()


def test_adjoint_missing_for_program_without_one():
    info = Library.get().query("hlld3d")
    g = Grid("hlld3d", (8, 8, 8), "f64", [1.0] * info["nuniforms"])
    with pytest.raises(FgbError, match="no adjoint"):
        g.backward(np.zeros((info["nfields"], 8, 8, 8)))
    g.close()


def test_adjoint_missing_in_fp16():
    U = _gs_uniforms()
    g = Grid("gs2d", (64, 64), "f16", U, scales=[1.0, 1.0])
    with pytest.raises(FgbError, match="no adjoint"):
        g.backward(np.zeros((2, 64, 64)))
    g.close()
