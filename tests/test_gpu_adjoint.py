"""Reverse mode on the GPU: the generated adjoint step and the checkpointed
gradient (binomial checkpointing), checked by dot-product tests, by
invariance to the number of checkpoints, by central finite differences, and
through torch.autograd.gradcheck."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import Grid, builtin_program, program_uniforms

pytestmark = pytest.mark.gpu


def _grid(program, n, prec="f64"):
    src, _ = builtin_program(program)
    cfg = {"heat3d": W.heat_config, "gs2d": W.gs_config}[program](n)
    _, U = program_uniforms(src, cfg, program)
    shape = (n, n, n) if program == "heat3d" else (n, n)
    return Grid(program, shape, prec, U), shape


def test_heat_dot_product_one_step():
    g, shape = _grid("heat3d", 24)
    rng = np.random.default_rng(0)
    v = rng.standard_normal((1,) + shape)
    w = rng.standard_normal((1,) + shape)
    g.upload(v)
    g.forward(1)
    Av = g.download()                        # the step is linear: A v
    g.upload(np.zeros((1,) + shape))
    ATw = g.backward(w)
    lhs, rhs = float(np.vdot(Av, w)), float(np.vdot(v, ATw))
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), 1.0)


def test_gray_scott_dot_product_tangent():
    g, shape = _grid("gs2d", 64)
    rng = np.random.default_rng(1)
    st = W.gs_perturb(np.ones(shape), np.zeros(shape), 2)
    u = np.stack([st["u"], st["v"]])
    u[:, 20:40, 20:40] = [[[0.5]], [[0.25]]]
    v = rng.standard_normal(u.shape)
    w = rng.standard_normal(u.shape)
    eps = 1e-6
    g.upload(u + eps * v)
    g.forward(1)
    fp = g.download()
    g.upload(u - eps * v)
    g.forward(1)
    fm = g.download()
    jv = (fp - fm) / (2 * eps)
    g.upload(u)
    jtw = g.backward(w)
    lhs, rhs = float(np.vdot(jv, w)), float(np.vdot(v, jtw))
    assert abs(lhs - rhs) <= 1e-7 * abs(lhs)


@pytest.mark.parametrize("program", ["heat3d", "gs2d"])
def test_checkpointing_does_not_change_the_gradient(program):
    g, shape = _grid(program, 32 if program == "heat3d" else 96)
    rng = np.random.default_rng(3)
    if program == "heat3d":
        u0 = W.gaussians_3d(shape, 4, count=8)[None]
    else:
        st = W.gs_perturb(np.ones(shape), np.zeros(shape), 5)
        u0 = np.stack([st["u"], st["v"]])
        u0[:, 30:60, 30:60] = [[[0.5]], [[0.25]]]
    target = u0 + 0.1 * rng.standard_normal(u0.shape)
    nsteps = 37
    grads = []
    for snaps in (nsteps, 8, 3, 1):
        uT, gr = g.gradient(u0, nsteps, snaps, lambda uT: uT - target)
        st = g.gradient_stats()
        assert st["adjoint_steps"] == nsteps
        if snaps == nsteps:
            assert st["forward_steps"] <= 2 * nsteps
        grads.append(gr)
    for gr in grads[1:]:
        assert np.array_equal(gr, grads[0])
    assert np.array_equal(g.download(), u0)     # the state is u_0 again


@pytest.mark.parametrize("prec,tol", [("f64", 1e-6), ("f32", 2e-2)])
def test_heat_gradient_against_central_differences(prec, tol):
    n, nsteps = 32, 50
    g, shape = _grid("heat3d", n, prec)
    f64, _ = _grid("heat3d", n, "f64fast")
    u0 = W.gaussians_3d(shape, 7, count=8)[None]
    target = W.gaussians_3d(shape, 8, count=8)[None]
    _, grad = g.gradient(u0, nsteps, 8, lambda uT: uT - target)

    def loss(u):
        f64.upload(u)
        f64.forward(nsteps)
        d = f64.download() - target
        return 0.5 * float(np.vdot(d, d))

    rng = np.random.default_rng(9)
    eps = 1e-6
    for _ in range(6):
        v = rng.standard_normal(u0.shape)
        fd = (loss(u0 + eps * v) - loss(u0 - eps * v)) / (2 * eps)
        ad = float(np.vdot(grad, v))
        assert abs(fd - ad) <= tol * abs(fd), (fd, ad)


def test_torch_gradcheck_small_rollout():
    torch = pytest.importorskip("torch")
    from formura_gb300.autograd import rollout
    g, shape = _grid("gs2d", 16)
    st = W.gs_perturb(np.ones(shape), np.zeros(shape), 11)
    u0 = np.stack([st["u"], st["v"]])
    u0[:, 5:10, 5:10] = [[[0.5]], [[0.3]]]
    x = torch.tensor(u0, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda t: rollout(t, g, 3, 2), (x,), eps=1e-6, atol=1e-7, rtol=1e-5)
