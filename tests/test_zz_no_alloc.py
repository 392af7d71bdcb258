"""fgb_forward_noalloc: stepping on caller-owned device buffers with no device
allocation inside the call.  Its callers cannot allocate device memory while
they run (their host owns the memory pool, or forbids allocation during a
run), so the entry point draws its scratch from a fixed static device array.

The test allocates the caller's buffers itself (with torch), then checks the
no-allocation entry point against the allocating one (fgb_open / fgb_upload /
fgb_forward / fgb_download) on two calls in a row.  FP64 results must be
identical bit for bit, the same bar as the other FP64 tests; the FP32 form
must agree to the same relative L2 bound (1e-6 here, on identical
arithmetic it is in practice zero).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import Grid, Library, builtin_program, program_uniforms

pytestmark = pytest.mark.gpu


def _noalloc(lib, program, shape, precision, U, d_in, d_out, nsteps, stream):
    L = lib.lib
    L.fgb_last_error.restype = ctypes.c_char_p
    L.fgb_forward_noalloc.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    shp = (ctypes.c_int * len(shape))(*shape)
    u = (ctypes.c_double * max(1, len(U)))(*U)
    return L.fgb_forward_noalloc(program.encode(), shp, len(shape), precision, u, len(U),
                                 ctypes.c_void_p(d_in), ctypes.c_void_p(d_out), nsteps, ctypes.c_void_p(stream))


@pytest.mark.parametrize("program,shape,prec,steps", [
    ("gs2d", (256, 256), "f64", (7, 4)),
    ("heat3d", (40, 40, 40), "f64", (5, 6)),
    ("hllc3d", (20, 20, 20), "f64", (3, 2)),
    ("gs2d", (256, 256), "f32", (8, 3)),
])
def test_noalloc_matches_allocating_path(program, shape, prec, steps):
    import torch
    lib = Library.get()
    src, _ = builtin_program(program)
    n = shape[0]
    cfg = {"gs2d": W.gs_config, "heat3d": W.heat_config, "hllc3d": W.hllc_config}[program](n)
    _, U = program_uniforms(src, cfg, program)
    if program == "gs2d":
        st = W.gs_perturb(np.ones(shape), np.zeros(shape), seed=9)
        state = np.stack([st["u"], st["v"]])
    elif program == "heat3d":
        state = W.heat_state(shape, seed=9)["q"][None]
    else:
        st = W.hllc_state(shape, seed=9)
        state = np.stack([st[f] for f in ("e", "mx", "my", "mz", "rho")])
    pnum = {"f64": 0, "f32": 2}[prec]
    tdtype = {"f64": torch.float64, "f32": torch.float32}[prec]

    # caller-owned device buffers
    d_a = torch.tensor(state, dtype=tdtype, device="cuda").contiguous()
    d_b = torch.empty_like(d_a)
    s = torch.cuda.current_stream().cuda_stream

    # reference: the allocating path
    g = Grid(program, shape, prec, U)
    g.upload(state)
    expect = []
    for k in steps:
        g.forward(k)
        expect.append(g.download())
    g.close()

    # two calls in a row: a -> b, then b -> a
    a_before = d_a.clone()
    rc = _noalloc(lib, program, shape, pnum, U, d_a.data_ptr(), d_b.data_ptr(), steps[0], s)
    assert rc == 0, lib.lib.fgb_last_error()
    torch.cuda.synchronize()
    # the input state is left as it was
    assert torch.equal(d_a, a_before)
    got1 = d_b.cpu().numpy().astype(np.float64)
    rc = _noalloc(lib, program, shape, pnum, U, d_b.data_ptr(), d_a.data_ptr(), steps[1], s)
    assert rc == 0, lib.lib.fgb_last_error()
    torch.cuda.synchronize()
    got2 = d_a.cpu().numpy().astype(np.float64)
    for got, ref in ((got1, expect[0]), (got2, expect[1])):
        if prec == "f64":
            assert np.array_equal(got, ref)
        else:
            assert W.rel_l2(got, ref) < 1e-6


def test_noalloc_rejects_oversize_and_overlap():
    import torch
    lib = Library.get()
    lib.lib.fgb_last_error.restype = ctypes.c_char_p
    src, _ = builtin_program("gs2d")
    _, U = program_uniforms(src, W.gs_config(2048), "gs2d")
    # 3072^2 x 2 fields x 8 B = 144 MiB of state: the ping-pong buffer exceeds 64 MiB
    shape = (3072, 3072)
    a = torch.zeros((2,) + shape, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    rc = _noalloc(lib, "gs2d", shape, 0, U, a.data_ptr(), b.data_ptr(), 2, 0)
    assert rc == -1 and b"bytes of scratch" in lib.lib.fgb_last_error()
    # overlapping input and output
    shape = (64, 64)
    a = torch.zeros((3, 64, 64), dtype=torch.float64, device="cuda")
    rc = _noalloc(lib, "gs2d", shape, 0, U, a.data_ptr(), a[1].data_ptr(), 1, 0)
    assert rc == -1 and b"overlap" in lib.lib.fgb_last_error()
