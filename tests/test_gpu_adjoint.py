"""Reverse mode on the GPU: the generated adjoint step and the checkpointed
gradient (binomial checkpointing), checked by dot-product tests, by
invariance to the number of checkpoints, by central finite differences, and
through torch.autograd.gradcheck."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import Grid, builtin_program, program_uniforms
from oracle.reference_lib import ReferenceProgram

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


# ---------------------------------------------------------------------------
# multi-stage steps: HLLC Euler (3 stages) and the 1D shock tube
# ---------------------------------------------------------------------------
HLLC_FIELDS = ["e", "mx", "my", "mz", "rho"]


def _hllc(n, prec="f64", seed=0):
    src, _ = builtin_program("hllc3d")
    _, U = program_uniforms(src, W.hllc_config(n), "hllc3d")
    st = W.hllc_state((n, n, n), seed)
    return Grid("hllc3d", (n, n, n), prec, U), np.stack([st[f] for f in HLLC_FIELDS])


def _tangent_dot(g, u, v, w, eps):
    g.upload(u + eps * v)
    g.forward(1)
    fp = g.download()
    g.upload(u - eps * v)
    g.forward(1)
    fm = g.download()
    jv = (fp - fm) / (2 * eps)
    g.upload(u)
    jtw = g.backward(w)
    return float(np.vdot(jv, w)), float(np.vdot(v, jtw))


def test_hllc_dot_product_one_step():
    # a rough state: no limiter sits within the difference step of a switch
    g, u = _hllc(16)
    rng = np.random.default_rng(4)
    u = u * (1 + 0.05 * rng.uniform(-1, 1, u.shape))
    v = rng.standard_normal(u.shape) * np.abs(u).max(axis=(1, 2, 3), keepdims=True)
    w = rng.standard_normal(u.shape)
    lhs, rhs = _tangent_dot(g, u, v, w, 1e-7)
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs), (lhs, rhs)


def test_sod_dot_product_one_step():
    src, cfg = builtin_program("sod1d")
    _, U = program_uniforms(src, cfg, "sod1d")
    g = Grid("sod1d", (400,), "f64", U)
    rng = np.random.default_rng(5)
    r = rng.uniform(-1, 1, (3, 400))
    u = np.stack([2.5 + 0.1 * r[0], 0.3 * r[1], 1 + 0.1 * r[2]])
    lhs, rhs = _tangent_dot(g, u, rng.standard_normal(u.shape), rng.standard_normal(u.shape), 1e-7)
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs), (lhs, rhs)


def test_hllc_checkpointing_does_not_change_the_gradient():
    g, u0 = _hllc(12, seed=1)
    target = u0 * 1.01
    nsteps = 9
    grads = []
    for snaps in (nsteps, 3, 1):
        _, gr = g.gradient(u0, nsteps, snaps, lambda uT: uT - target)
        assert g.gradient_stats()["adjoint_steps"] == nsteps
        grads.append(gr)
    for gr in grads[1:]:
        assert np.array_equal(gr, grads[0])


@pytest.mark.parametrize("prec,tol", [("f64", 2e-3), ("f32", 3e-2)])
def test_hllc_density_gradient_against_central_differences(prec, tol):
    """dJ/d rho_0 of J = 0.5 ||u_T - u_target||^2 over the smooth
    Mach-0.3 state, checked on random density directions.  The minmod
    limiter is only piecewise smooth (its min switches where the two
    one-sided slopes cross, at every inflection of the field), so central
    differences carry an O(eps)-wide kink error: 2e-4 at this size."""
    n, nsteps = 16, 20
    g, u0 = _hllc(n, prec, seed=2)
    f64, _ = _hllc(n, "f64", seed=2)
    target = u0 + 0.01 * np.random.default_rng(6).standard_normal(u0.shape)
    _, grad = g.gradient(u0, nsteps, 4, lambda uT: uT - target)

    def loss(u):
        f64.upload(u)
        f64.forward(nsteps)
        d = f64.download() - target
        return 0.5 * float(np.vdot(d, d))

    rng = np.random.default_rng(7)
    eps = 1e-7
    ir = HLLC_FIELDS.index("rho")
    for _ in range(4):
        v = np.zeros_like(u0)
        v[ir] = rng.standard_normal(u0.shape[1:])
        fd = (loss(u0 + eps * v) - loss(u0 - eps * v)) / (2 * eps)
        ad = float(np.vdot(grad, v))
        assert abs(fd - ad) <= tol * abs(fd), (fd, ad)


@pytest.mark.parametrize("program", ["hllc3d", "sod1d"])
def test_f32_backward_matches_f64(program):
    """The FP32 adjoint step gathers the linear update stage's partial sums
    directly; the FP64 step stores and gathers them.  On the same state and
    seed both give the same lambda up to FP32 rounding."""
    rng = np.random.default_rng(6)
    if program == "hllc3d":
        g64, u = _hllc(16)
        g32, _ = _hllc(16, "f32")
    else:
        src, cfg = builtin_program("sod1d")
        _, U = program_uniforms(src, cfg, "sod1d")
        g64, g32 = Grid("sod1d", (400,), "f64", U), Grid("sod1d", (400,), "f32", U)
        r = rng.uniform(-1, 1, (3, 400))
        u = np.stack([2.5 + 0.1 * r[0], 0.3 * r[1], 1 + 0.1 * r[2]])
    w = rng.standard_normal(u.shape)
    lam = []
    for g in (g64, g32):
        g.upload(u)
        lam.append(g.backward(w))
        g.close()
    assert W.rel_l2(lam[1], lam[0]) < 1e-4, W.rel_l2(lam[1], lam[0])


# ---------------------------------------------------------------------------
# reference gradients by differencing the oracle (the reference generator's
# C, run on the host), as the finite-difference check of the adjoint
# ---------------------------------------------------------------------------
def _oracle_loss(program, cfg, fields, nsteps, target, tag):
    """J(u) = 0.5 ||u_T - target||^2 with u_T from the oracle: Formura_Init,
    u written into formura_data, nsteps Formura_Forward calls."""
    src, _ = builtin_program(program)
    ref = ReferenceProgram(src, cfg, f"{program}_fd_{tag}")

    def loss(u):
        ref.init()
        for i, f in enumerate(fields):
            ref.set(f, u[i])
        ref.forward(nsteps)
        d = np.stack([ref.get(f) for f in fields]) - target
        return 0.5 * float(np.vdot(d, d))
    return loss


@pytest.mark.parametrize("prec,tol", [("f64", 1e-6), ("f32", 2e-2)])
def test_heat_gradient_against_oracle_differences(prec, tol):
    """dJ/du_0 of the diffusion rollout (32^3, 50 steps, 8 checkpoints)
    against central differences (eps 1e-6) of the oracle's loss on random
    directions."""
    n, nsteps = 32, 50
    g, shape = _grid("heat3d", n, prec)
    u0 = W.gaussians_3d(shape, 7, count=8)[None]
    target = W.gaussians_3d(shape, 8, count=8)[None]
    _, grad = g.gradient(u0, nsteps, 8, lambda uT: uT - target)
    loss = _oracle_loss("heat3d", W.heat_config(n), ["q"], nsteps, target, "heat")
    rng = np.random.default_rng(19)
    eps = 1e-6
    for _ in range(6):
        v = rng.standard_normal(u0.shape)
        fd = (loss(u0 + eps * v) - loss(u0 - eps * v)) / (2 * eps)
        ad = float(np.vdot(grad, v))
        assert abs(fd - ad) <= tol * abs(fd), (fd, ad)


@pytest.mark.parametrize("prec,tol", [("f64", 2e-3), ("f32", 3e-2)])
def test_hllc_density_gradient_against_oracle_differences(prec, tol):
    """dJ/d rho_0 of the Euler rollout (16^3, 20 steps, the smooth Mach-0.3
    state) against central differences (eps 1e-7) of the oracle's loss on
    random density directions; the limiter's kinks bound the agreement as in
    the GPU-forward check above."""
    n, nsteps = 16, 20
    g, u0 = _hllc(n, prec, seed=2)
    target = u0 + 0.01 * np.random.default_rng(6).standard_normal(u0.shape)
    _, grad = g.gradient(u0, nsteps, 4, lambda uT: uT - target)
    loss = _oracle_loss("hllc3d", W.hllc_config(n), HLLC_FIELDS, nsteps, target, "hllc")
    rng = np.random.default_rng(17)
    eps = 1e-7
    ir = HLLC_FIELDS.index("rho")
    for _ in range(4):
        v = np.zeros_like(u0)
        v[ir] = rng.standard_normal(u0.shape[1:])
        fd = (loss(u0 + eps * v) - loss(u0 - eps * v)) / (2 * eps)
        ad = float(np.vdot(grad, v))
        assert abs(fd - ad) <= tol * abs(fd), (fd, ad)
