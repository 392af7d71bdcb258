"""Which arrays the GPU step stores (generator/cuda.py: store_shared_operands).

The MUSCL programs' face states (qL = q - s/2, qR = q + s/2) are stored as
their shared slope s; the step's results stay bit-identical (the GPU and
host parity tests compare bit patterns).  A program with a stage adjoint
keeps its own arrays for the adjoint, generated in a second namespace, and
both share one uniform table."""
import re

import pytest

from formura_gb300.generator.config import decode_config
from formura_gb300.generator.cuda import build_stages, emit_cuda, gpu_step_program
from formura_gb300.generator.manifest import compile_program
from formura_gb300.host import builtin_program


def _mm(program):
    src, cfg = builtin_program(program)
    return compile_program(src, decode_config(cfg))


@pytest.mark.parametrize("program,own,gpu", [("hllc3d", [35, 15, 0], [20, 15, 0]),
                                             ("hlld3d", [63, 27, 0], [36, 27, 0]),
                                             ("sod1d", [9, 3, 0], [6, 3, 0])])
def test_slopes_stored_instead_of_face_states(program, own, gpu):
    mm = _mm(program)
    assert [len(s.mid_out) for s in build_stages(mm.step)] == own
    assert [len(s.mid_out) for s in build_stages(gpu_step_program(mm).step)] == gpu
    # the program itself (the oracle's view) is unchanged
    assert [len(s.mid_out) for s in build_stages(mm.step)] == own


@pytest.mark.parametrize("program", ["gs2d", "heat3d"])
def test_single_stage_programs_unchanged(program):
    mm = _mm(program)
    assert gpu_step_program(mm) is mm


def test_adjoint_keeps_the_programs_own_arrays():
    mm = _mm("hllc3d")
    kp = emit_cuda(mm, "hllc3d", [], stage_adjoint=True)
    src = kp.source
    assert len(kp.mids) == 35
    assert "namespace fgb_gen_hllc3d_adj" in src
    assert "using AdjStages = fgb::StageTypes<" in src
    assert "using StageAdjoint = fgb_gen_hllc3d_adj::StageAdjointList;" in src
    own = re.search(r"namespace fgb_gen_hllc3d_adj \{.*?static constexpr int kMids = (\d+);", src, re.S)
    assert own and int(own.group(1)) == 50
    # one uniform table: the forward's starts with the adjoint's entries
    uni = [int(x) for x in re.findall(r"static constexpr int kUniforms = (\d+);", src)]
    assert len(uni) == 2 and uni[0] <= uni[1] == len(kp.uniform_exprs)
