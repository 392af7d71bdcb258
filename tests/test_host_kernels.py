"""The generated device code, run on the CPU.

Each shipped program's generated file (formura_gb300/_gen/prog_<name>.cu) is
compiled with g++ against a host stand-in of the kernel templates
(tests/native/hostshim): the same stage functors, one grid point at a time,
every operation rounded once in binary64.  This checks the CUDA emitter
without a GPU:

* its stage code reproduces the oracle (the reference generator's C,
  restated) bit for bit over several steps, roll included;
* its adjoints (the one-pass adjoint of single-stage steps and the two-pass
  adjoint of multi-stage steps) are the transpose of the step's Jacobian:
  <J v, w> against <v, J^T w>, with J v by central differences.  The states
  are random rather than smooth, so that no limiter sits near a switch."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from formura_gb300 import build as B
from formura_gb300 import workloads as W
from formura_gb300.host import builtin_program, program_uniforms
from oracle.reference_lib import ReferenceProgram

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(HERE, "native", "hostshim")


@pytest.fixture(scope="module")
def generated():
    return B.generate()


def _host_lib(generated, program, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("host") / f"host_{program}.so")
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", SHIM,
                           "-x", "c++", generated[program], "-o", out])
    return ctypes.CDLL(out)


class HostProgram:
    def __init__(self, lib, program, shape, U):
        P = ctypes.POINTER(ctypes.c_double)
        self.f = getattr(lib, f"host_forward_{program}")
        self.b = getattr(lib, f"host_backward_{program}")
        self.f.argtypes = [ctypes.POINTER(ctypes.c_int), P, P, P]
        self.b.argtypes = [ctypes.POINTER(ctypes.c_int), P, P, P, P]
        self.n = (ctypes.c_int * len(shape))(*shape)
        self.U = np.ascontiguousarray(U, dtype=np.float64)
        self.P = P

    def forward(self, u):
        u = np.ascontiguousarray(u)
        out = np.empty_like(u)
        self.f(self.n, self.U.ctypes.data_as(self.P), u.ctypes.data_as(self.P), out.ctypes.data_as(self.P))
        return out

    def backward(self, u, lam):
        u, lam = np.ascontiguousarray(u), np.ascontiguousarray(lam)
        out = np.empty_like(u)
        rc = self.b(self.n, self.U.ctypes.data_as(self.P), u.ctypes.data_as(self.P), lam.ctypes.data_as(self.P),
                    out.ctypes.data_as(self.P))
        assert rc == 0, "no adjoint"
        return out


def _case(program, rng):
    """(config, shape, fields, random state) of a small case."""
    if program == "heat3d":
        n = 10
        return W.heat_config(n), (n, n, n), ["q"], rng.random((1, n, n, n))
    if program == "gs2d":
        n = 24
        u = np.stack([1.0 - 0.5 * rng.random((n, n)), 0.25 * rng.random((n, n))])
        return W.gs_config(n), (n, n), ["u", "v"], u
    if program == "smooth2d":
        # a filter interval past the steps run: Formura_Forward is the step alone
        cfg = "length_per_node: [1.0, 1.0]\ngrid_per_node: [64, 64]\nfilter_interval: 1000\nwith_omp: 1\n"
        return cfg, (64, 64), ["q"], rng.random((1, 64, 64))
    if program == "sod1d":
        _, cfg = builtin_program(program)
        r = rng.uniform(-1, 1, (3, 400))
        return cfg, (400,), ["e", "m", "rho"], np.stack([2.5 + 0.1 * r[0], 0.3 * r[1], 1 + 0.1 * r[2]])
    if program == "hllc3d":
        n = 8
        st = W.hllc_state((n, n, n), 3)
        f = ["e", "mx", "my", "mz", "rho"]
        u = np.stack([st[k] for k in f])
        return W.hllc_config(n), (n, n, n), f, u * (1 + 0.05 * rng.uniform(-1, 1, u.shape))
    if program == "hlld3d":
        n = 8
        st = W.mhd_state((n, n, n), 4)
        f = ["bx", "by", "bz", "e", "mx", "my", "mz", "psi", "rho"]
        return W.mhd_config(n), (n, n, n), f, np.stack([st[k] for k in f])
    raise KeyError(program)


@pytest.mark.parametrize("program", ["heat3d", "gs2d", "smooth2d", "sod1d", "hllc3d", "hlld3d"])
def test_generated_step_matches_oracle(generated, tmp_path_factory, program):
    rng = np.random.default_rng(1)
    cfg, shape, fields, u = _case(program, rng)
    src, _ = builtin_program(program)
    _, U = program_uniforms(src, cfg, program)
    host = HostProgram(_host_lib(generated, program, tmp_path_factory), program, shape, U)
    ref = ReferenceProgram(src, cfg, f"host_{program}")
    ref.init()
    assert ref.fields == fields
    for i, f in enumerate(fields):
        ref.set(f, u[i])
    steps = 3
    ref.forward(steps)
    x = u
    filt = None
    if program == "smooth2d":
        # Formura_Forward applies the filter after a step whose time_step
        # (before the increment) is a multiple of the interval: here step 0
        from formura_gb300.generator.config import decode_config
        from formura_gb300.generator.cuda import emit_cuda, uniform_table
        from formura_gb300.generator.manifest import compile_program
        mm = compile_program(src, decode_config(cfg))
        kf = emit_cuda(mm, program, [], "filter")
        filt = HostProgram(_host_lib(generated, program, tmp_path_factory), program + "__filter", shape,
                           uniform_table(mm, kf))
    for k in range(steps):
        x = host.forward(x)
        if filt is not None and k % 1000 == 0:
            x = filt.forward(x)
    for i, f in enumerate(fields):
        assert np.array_equal(x[i], ref.get(f)), f


@pytest.mark.parametrize("program", ["heat3d", "gs2d", "sod1d", "hllc3d"])
def test_generated_adjoint_is_the_transpose(generated, tmp_path_factory, program):
    rng = np.random.default_rng(2)
    cfg, shape, fields, u = _case(program, rng)
    src, _ = builtin_program(program)
    _, U = program_uniforms(src, cfg, program)
    host = HostProgram(_host_lib(generated, program, tmp_path_factory), program, shape, U)
    v = rng.standard_normal(u.shape) * np.abs(u).max()
    w = rng.standard_normal(u.shape)
    eps = 1e-7
    jv = (host.forward(u + eps * v) - host.forward(u - eps * v)) / (2 * eps)
    jtw = host.backward(u, w)
    lhs, rhs = float(np.vdot(jv, w)), float(np.vdot(v, jtw))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs), (lhs, rhs)


# ---------------------------------------------------------------------------
# the reference's own programs through the CUDA emitter (this container only)
# ---------------------------------------------------------------------------
REFERENCE_PROGRAMS = {
    "diffusion1": ("examples/diffusion1/diffusion1.fmr", "examples/diffusion1/diffusion1.yaml", None),
    "diffusion2": ("examples/diffusion2/diffusion2.fmr", "examples/diffusion2/diffusion2.yaml", None),
    "diffusion3": ("examples/diffusion3/diffusion3.fmr", "examples/diffusion3/diffusion3.yaml", "[20, 20, 20]"),
    "pearson2": ("examples/pearson2/pearson2.fmr", "examples/pearson2/pearson2.yaml", "[64, 64]"),
    "hllc1d": ("sample/1d_hllc/hllc.fmr", "sample/1d_hllc/config.yaml", None),
    "hllc3d_sample": ("sample/3d_hllc/3d_hllc.fmr", "sample/3d_hllc/config.yaml", "[12, 12, 12]"),
    "hlld1d": ("sample/mhd_1d_hlld/mhd_hlld.fmr", "sample/mhd_1d_hlld/config.yaml", None),
    "hlld3d_sample": ("sample/mhd_3d_hlld/mhd_3d_hlld.fmr", "sample/mhd_3d_hlld/config.yaml", "[10, 10, 10]"),
}


def _one_rank_config(text, grid=None):
    """The sample's config for one rank, one step per Formura_Forward: MPI
    shape and temporal blocking dropped, optionally a smaller grid."""
    keep = []
    for line in text.splitlines():
        key = line.split(":")[0].strip()
        if key in ("mpi_shape", "grid_per_block", "temporal_blocking_interval"):
            continue
        if key == "grid_per_node" and grid is not None:
            line = f"grid_per_node: {grid}"
        keep.append(line)
    return "\n".join(keep) + "\n"


@pytest.mark.parametrize("name", sorted(REFERENCE_PROGRAMS))
def test_reference_program_through_cuda_emitter(tmp_path, name):
    """The CUDA emitter's code for the reference's own example and sample
    programs, run on the host, equals the oracle bit for bit from each
    program's own initial state."""
    from formura_gb300.generator.config import decode_config
    from formura_gb300.generator.cuda import emit_cuda, uniform_table
    from formura_gb300.generator.manifest import compile_program
    from conftest import REFERENCE
    if not os.path.isdir(REFERENCE):
        pytest.skip("the reference tree is not present")
    fmr, yml, grid = REFERENCE_PROGRAMS[name]
    with open(os.path.join(REFERENCE, fmr)) as f:
        src = f.read()
    with open(os.path.join(REFERENCE, yml)) as f:
        cfg = _one_rank_config(f.read(), grid)
    mm = compile_program(src, decode_config(cfg))
    kp = emit_cuda(mm, f"ref_{name}", [], stage_adjoint=False)
    cu = tmp_path / f"ref_{name}.cu"
    cu.write_text(kp.source)
    so = str(tmp_path / f"ref_{name}.so")
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", SHIM,
                           "-x", "c++", str(cu), "-o", so])
    ref = ReferenceProgram(src, cfg, f"refemit_{name}")
    ref.init()
    u = np.stack([ref.get(f) for f in ref.fields])
    shape = u.shape[1:]
    host = HostProgram(ctypes.CDLL(so), f"ref_{name}", shape, uniform_table(mm, kp))
    steps = 3
    ref.forward(steps)
    for _ in range(steps):
        u = host.forward(u)
    for i, f in enumerate(ref.fields):
        assert np.array_equal(u[i], ref.get(f)), f


# ---------------------------------------------------------------------------
# the divisor list that selects the power-of-two kernels of a grid
# ---------------------------------------------------------------------------
_DIV_PROGRAM = """dimension :: 1
axes :: x

begin function q = init()
  double [] :: q = 0
end function

begin function q_new = step(q)
  q_new = q + (q[i+1] + q[i-1]) / dx{extra}
end function
"""


@pytest.mark.parametrize("extra,count", [("", 1), (" + (q[i+1] - q[i-1]) / 4.0", 1),
                                         (" + (q[i+1] - q[i-1]) / 3.0", -1)])
def test_divisor_slots_for_the_power_of_two_kernels(extra, count):
    """A grid steps with the kernels whose division by a constant is one
    product only if every divisor is a power of two.  The generator lists the
    uniform-table slots the host checks; a literal divisor that is a power of
    two needs no slot (it is a product already), and one that is not makes
    the program ineligible (-1)."""
    import re
    from formura_gb300.generator.config import decode_config
    from formura_gb300.generator.cuda import emit_cuda
    from formura_gb300.generator.manifest import compile_program
    cfg = "length_per_node: [1.0]\ngrid_per_node: [16]\nwith_omp: 1\n"
    kp = emit_cuda(compile_program(_DIV_PROGRAM.format(extra=extra), decode_config(cfg)), "divtest", [],
                   stage_adjoint=False)
    assert re.findall(r"kNumDivisors = (-?\d+)", kp.source) == [str(count)]


def test_shipped_programs_divisor_slots(generated):
    """heat3d, gs2d and hllc3d divide by their grid spacings only (table
    slots), so grids whose spacing is a power of two take the single-product
    kernels."""
    import re
    for program, n in (("heat3d", 3), ("gs2d", 4), ("hllc3d", 3)):
        with open(generated[program]) as f:
            src = f.read()
        assert re.findall(r"kNumDivisors = (-?\d+)", src)[0] == str(n), program
