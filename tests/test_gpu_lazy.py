"""Lazy host synchronisation of formura_data (gpu_host_sync: lazy): the
drop-in keeps the state on the device between Formura_Forward calls; a read
of formura_data by the driver downloads it, a write is uploaded before the
next call.  Results must match the oracle bit for bit."""
import numpy as np
import pytest

from formura_gb300 import workloads as W
from formura_gb300.host import FormuraProgram, builtin_program
from oracle.reference_lib import ReferenceProgram

pytestmark = pytest.mark.gpu


def test_lazy_sync_reads_and_writes():
    n = 64
    src, _ = builtin_program("gs2d")
    cfg = W.gs_config(n)
    ref = ReferenceProgram(src, cfg, "gs_lazy_ref")
    gpu = FormuraProgram(src, cfg + "gpu_host_sync: lazy\ngpu_steps_per_forward: 5\n", "gs2d", name="gs_lazy_gpu")
    ref.init()
    gpu.init()
    st = W.gs_perturb(ref.get("u"), ref.get("v"), seed=21)
    for f in ("u", "v"):
        ref.set(f, st[f])
        gpu.set(f, st[f])
    # several calls without touching formura_data: no copies
    for _ in range(4):
        ref.forward(5)
        gpu.forward(1)
    assert ref.navi_dict() == gpu.navi_dict()
    for f in ("u", "v"):                       # first read downloads
        assert np.array_equal(ref.get(f), gpu.get(f))
    # the driver writes between calls (like examples/pearson2/main.c)
    u = gpu.get("u")
    u[10:20, 30:40] += 0.05
    gpu.set("u", u)
    ref.set("u", u)
    for _ in range(3):
        ref.forward(5)
        gpu.forward(1)
    for f in ("u", "v"):
        assert np.array_equal(ref.get(f), gpu.get(f))
    gpu.finalize()
    for f in ("u", "v"):                       # after Finalize the host copy is current
        assert np.array_equal(ref.get(f), gpu.get(f))
