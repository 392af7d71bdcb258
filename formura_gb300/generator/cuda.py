"""CUDA emission: turns a program's step graph (Manifest Machine) into the
device code that the hand-written sm_103a kernel templates of
``formura_gb300/csrc/fgb_templates.cuh`` are instantiated with.

Where the reference emits one OpenMP loop nest per manifest node over a
halo-padded buffer (``src/Formura/Generator/Templates.hs:426-487``), this
backend groups manifest nodes into *stages*.  A node joins the stage of a
dependency it reads only at cursor 0 (the value stays in registers), and opens
a later stage when it reads a dependency at a nonzero cursor (the value goes
through an HBM array).  Heat and Gray-Scott are one stage; HLLC/HLLD are
three.  Loads wrap periodically in-kernel instead of reading a halo buffer.

Arithmetic follows the reference's SSA chain one operation at a time, so the
FP64 form rounds exactly where the reference's C rounds:

* subexpressions that do not depend on the grid (``dt``, ``dx**2`` ...) are
  evaluated once on the host, each operation correctly rounded, which is what
  gcc's constant folding of the reference's literal chain gives;
* ``pow(x, 2)`` is ``x*x`` (gcc expands it the same way); ``sqrt`` is
  correctly rounded on both sides;
* a product by a literal power of two is exact, so ``a - 2*b`` may become one
  fused multiply-add without changing the result;
* division by a grid-independent value uses the reciprocal and one fused
  correction step (Markstein's theorem: with ``r = RN(1/c)``, ``q = RN(x*r)``,
  ``e = fma(-q, c, x)``, ``RN(q + e*r)`` is the correctly rounded ``x/c``);
  the policy selects it only after the GPU self-check in the tests.
"""
from __future__ import annotations

import math
import os
import struct
from dataclasses import dataclass, field
from decimal import Decimal, localcontext
from fractions import Fraction
from typing import Dict, List, Optional, Set, Tuple

import copy
import dataclasses

from .manifest import MMNode, MMProgram, MicroNode, calc_range, manifest_graph
from .translate import FormuraCompileError, Graph


# --------------------------------------------------------------------------
# correctly rounded evaluation of grid-independent values
# --------------------------------------------------------------------------
def _dec(x: float) -> Decimal:
    return Decimal(Fraction(x).numerator) / Decimal(Fraction(x).denominator)


def _dec_sin(x: Decimal) -> Decimal:
    with localcontext() as ctx:
        ctx.prec += 10
        two_pi = Decimal("6.283185307179586476925286766559005768394338798750211641949889184615632812572417997")
        x = x % two_pi
        term, s, k = x, x, 1
        while True:
            term = -term * x * x / ((2 * k) * (2 * k + 1))
            if abs(term) < Decimal(10) ** (-(ctx.prec + 5)):
                break
            s += term
            k += 1
    return +s


def external_value(f: str, x: float) -> float:
    """Correctly rounded libm function of a constant (what gcc folds to)."""
    if f == "sqrt":
        return math.sqrt(x)
    if f == "fabs":
        return abs(x)
    with localcontext() as ctx:
        ctx.prec = 60
        d = _dec(x)
        if f == "exp":
            return float(d.exp())
        if f == "log":
            return float(d.ln())
        if f == "sin":
            return float(_dec_sin(d))
        if f == "cos":
            return float(_dec_sin(d + Decimal("1.5707963267948966192313216916397514420985846996875529104874722961539082031431044993")))
    raise FormuraCompileError(f"external function {f} has no host evaluation")


def pow_value(a: float, b: float) -> float:
    if b == int(b) and abs(b) <= 64:
        n = int(b)
        if a == 0.0:
            return math.pow(a, b)
        v = Fraction(a) ** n
        return float(v)
    with localcontext() as ctx:
        ctx.prec = 60
        return float((_dec(b) * _dec(a).ln()).exp())


def fold(inst, vals) -> object:
    """Evaluate one micro instruction on constant operands (IEEE double)."""
    k = inst[0]
    if k == "imm":
        return float(inst[1])
    if k == "uniop":
        op, a = inst[1], vals[0]
        if op == "-":
            return -a
        if op == "+":
            return a
        if op.startswith("external-call/"):
            return external_value(op[len("external-call/"):], a)
        raise FormuraCompileError(f"unary operator {op}")
    if k == "binop":
        op, a, b = inst[1], vals[0], vals[1]
        if op == "+":
            return a + b
        if op == "-":
            return a - b
        if op == "*":
            return a * b
        if op == "/":
            return a / b if b != 0 else math.copysign(math.inf, a) * math.copysign(1, b)
        if op == "**":
            return pow_value(a, b)
        if op == "<":
            return a < b
        if op == ">":
            return a > b
        if op == "<=":
            return a <= b
        if op == ">=":
            return a >= b
        if op == "==":
            return a == b
        if op == "!=":
            return a != b
        if op == "&&":
            return bool(a) and bool(b)
        if op == "||":
            return bool(a) or bool(b)
        raise FormuraCompileError(f"binary operator {op}")
    if k == "triop":
        return vals[1] if vals[0] else vals[2]
    raise FormuraCompileError(f"cannot fold {k}")


def c_double(x: float) -> str:
    """Exact C literal for a double."""
    if x != x:
        return "(0.0/0.0)"
    if math.isinf(x):
        return "(1.0/0.0)" if x > 0 else "(-1.0/0.0)"
    return float.hex(x)


def is_pow2(x: float) -> bool:
    if x == 0 or not math.isfinite(x):
        return False
    m, _ = math.frexp(abs(x))
    return m == 0.5


# --------------------------------------------------------------------------
# program analysis
# --------------------------------------------------------------------------
CONFIG_NAMES_PREFIX = ("total_grid_",)


@dataclass
class Stage:
    index: int
    nodes: List[MMNode]
    writes_state: bool
    mid_out: List[int] = field(default_factory=list)   # manifest ids stored to HBM


@dataclass
class KernelProgram:
    name: str
    dim: int
    axes: List[str]
    fields: List[str]
    sleeve: int
    shift: int                   # output index = position + shift (periodic)
    max_reach: int               # largest |cursor| read from any array
    stages: List[Stage]
    mids: List[int]              # manifest ids stored to HBM, in array order
    uniform_exprs: List[tuple]   # table entries: ('node', key) evaluated by host
    runtime_params: List[str]
    source: str = ""             # generated CUDA


class _Analysis:
    """Classifies micro nodes of one program: grid-independent (uniform) or
    not, and whether a uniform value depends on the configuration."""

    def __init__(self, mm: MMProgram, runtime_params: List[str], graph: str = "step"):
        self.mm = mm
        self.g = {"step": mm.om.step_graph, "first_step": mm.om.first_step_graph,
                  "filter": mm.om.filter_graph}[graph]
        self.axes = mm.om.genv.axes
        names = {"d" + a for a in self.axes} | {"total_grid_" + a for a in self.axes}
        names |= set(runtime_params)
        self.param_names = names
        self._uni: Dict[int, bool] = {}
        self._cfg: Dict[int, bool] = {}

    def om_uniform(self, nid: int) -> bool:
        """An OM node is uniform when no grid load reaches it."""
        if nid in self._uni:
            return self._uni[nid]
        inst = self.g[nid].inst
        k = inst[0]
        if k == "imm":
            r = True
        elif k in ("uniop",):
            r = self.om_uniform(inst[2])
        elif k == "binop":
            r = self.om_uniform(inst[2]) and self.om_uniform(inst[3])
        elif k == "triop":
            r = all(self.om_uniform(x) for x in inst[2:5])
        elif k == "shift":
            r = self.om_uniform(inst[2])
        else:
            r = False
        self._uni[nid] = r
        return r

    def om_config_dependent(self, nid: int) -> bool:
        """A uniform node whose value changes with the numerical config or a
        runtime parameter (it reads ``dx``, ``total_grid_x`` ...)."""
        if nid in self._cfg:
            return self._cfg[nid]
        nd = self.g[nid]
        inst = nd.inst
        if inst[0] == "imm":
            r = nd.name in self.param_names
        elif inst[0] == "uniop":
            r = self.om_config_dependent(inst[2])
        elif inst[0] == "binop":
            r = self.om_config_dependent(inst[2]) or self.om_config_dependent(inst[3])
        elif inst[0] == "triop":
            r = any(self.om_config_dependent(x) for x in inst[2:5])
        elif inst[0] == "shift":
            r = self.om_config_dependent(inst[2])
        else:
            r = False
        self._cfg[nid] = r
        return r

    def om_value(self, nid: int, params: Optional[Dict[str, float]] = None):
        """Host value of a uniform OM node (each operation rounded once)."""
        nd = self.g[nid]
        inst = nd.inst
        if inst[0] == "imm":
            if params and nd.name in params:
                return float(params[nd.name])
            return float(inst[1])
        if inst[0] == "shift":
            return self.om_value(inst[2], params)
        if inst[0] == "uniop":
            return fold(inst[:2] + (None,), [self.om_value(inst[2], params)])
        if inst[0] == "binop":
            return fold(inst[:2] + (None, None), [self.om_value(inst[2], params),
                                                   self.om_value(inst[3], params)])
        if inst[0] == "triop":
            return fold(inst, [self.om_value(x, params) for x in inst[2:5]])
        raise FormuraCompileError("not a uniform node")


def build_stages(step: List[MMNode]) -> List[Stage]:
    """Group manifest nodes: reading a node at cursor 0 keeps it in the same
    stage; reading it at a nonzero cursor needs it in an earlier stage."""
    stage_of: Dict[int, int] = {}
    for node in step:
        st = 0
        for mn in node.micro:
            if mn.inst[0] == "loadcursor":
                dep = mn.inst[2]
                c = mn.inst[1]
                need = stage_of[dep] + (0 if all(x == 0 for x in c) else 1)
                st = max(st, need)
        stage_of[node.omid] = st
    # stores go last: they overwrite the state that earlier stages read
    last = max(stage_of.values())
    for node in step:
        if node.is_store:
            stage_of[node.omid] = last
    nst = last + 1
    stages = [Stage(i, [n for n in step if stage_of[n.omid] == i],
                    any(n.is_store and stage_of[n.omid] == i for n in step)) for i in range(nst)]
    # which manifest values must go through HBM
    for node in step:
        for mn in node.micro:
            if mn.inst[0] == "loadcursor":
                dep = mn.inst[2]
                if stage_of[dep] != stage_of[node.omid]:
                    s = stages[stage_of[dep]]
                    if dep not in s.mid_out:
                        s.mid_out.append(dep)
    for s in stages:
        s.mid_out.sort()
    return stages


# --------------------------------------------------------------------------
# emission
# --------------------------------------------------------------------------
_EXT = {"sqrt": "sqrt", "fabs": "fabs", "exp": "exp", "log": "log", "sin": "sin", "cos": "cos"}
_CMP = {"<", ">", "<=", ">=", "==", "!="}
# comparisons are policy calls: the bit-faithful FP64 policy evaluates them
# on the integer pipe
_CMP_NAME = {"<": "lt", ">": "gt", "<=": "le", ">=": "ge", "==": "eq", "!=": "ne"}

class _StageEmitter:
    """Emits one stage's SSA chain.  ``policy`` names the arithmetic policy
    of the operations (``M``, the kernel's, or ``D``, its derivative policy);
    with ``reciprocal`` a quotient by a grid value is formed as a product
    with the reciprocal, which then serves every later use of it."""

    def __init__(self, prog: "_ProgramEmitter", stage: Stage, policy: str = "M", reciprocal: bool = False,
                 div_uses: Optional[Dict[str, int]] = None):
        self.p = prog
        self.stage = stage
        self.P = policy
        self.reciprocal = reciprocal
        # quotients per grid denominator, from an earlier pass over the same
        # stage: a denominator with several gets one reciprocal (M::rcp) and
        # its quotients M::divr
        self.div_uses = div_uses or {}
        self.div_seen: Dict[str, int] = {}
        self.nr = 0
        self.lines: List[str] = []
        self.var: Dict[tuple, object] = {}     # key -> expression handle
        self.memo: Dict[tuple, tuple] = {}     # (expression, type) -> handle
        self.n = 0
        self.scaled: Dict[tuple, str] = {}     # materialised power-of-two products

    def fresh(self) -> str:
        self.n += 1
        return f"t{self.n}"

    def emit(self, text: str):
        self.lines.append("    " + text)

    # expression handles: ('v', name, ctype) or ('lit', float) or ('u', index)
    # or ('scaled', literal, handle) for an exact product by a power of two
    def as_T(self, h) -> str:
        if h[0] == "v":
            return h[1]
        if h[0] == "lit":
            return f"T({c_double(h[1])})"
        if h[0] == "u":
            return f"U[{self.p.table_index(h[1])}]"
        if h[0] == "scaled":
            return self.materialize(h)
        raise AssertionError(h)

    def materialize(self, h) -> str:
        cache = self.scaled
        key = (h[1], self.as_T(h[2]))
        if key not in cache:
            name = self.fresh()
            self.emit(f"const T {name} = {self.P}::mul(T({c_double(h[1])}), {key[1]});")
            cache[key] = name
        return cache[key]

    def uniform_handle(self, omid: int):
        an = self.p.an
        if an.om_config_dependent(omid):
            return ("u", ("node", omid))
        v = an.om_value(omid)
        if isinstance(v, bool):
            return ("lit", 1.0 if v else 0.0)
        return ("lit", v)

    def recip_handle(self, omid: int):
        an = self.p.an
        if an.om_config_dependent(omid):
            return ("u", ("recip", omid))
        return ("lit", 1.0 / an.om_value(omid))

    def node(self, node: MMNode):
        micro = node.micro
        for idx, mn in enumerate(micro):
            key = mn.key
            if key in self.var:
                continue
            h = self.micro(mn, micro, node)
            if h is not None:
                self.var[key] = h
        if node.omid in self.stage.mid_out:
            root = self.var[micro[-1].key]
            k = self.p.mids.index(node.omid)
            self.emit(f"a.template stm<{k}>({self.as_T(root)});")

    def operand(self, micro, i):
        return self.var[micro[i].key]

    def micro(self, mn: MicroNode, micro, node: MMNode):
        inst = mn.inst
        k = inst[0]
        an = self.p.an
        omid = mn.key[1]
        if k in ("imm", "uniop", "binop", "triop") and an.om_uniform(omid):
            return self.uniform_handle(omid)
        if k == "loadstatic":
            c = self.p.cursor3(inst[1])
            f = self.p.fields.index(inst[2])
            return self.bind(f"a.template ld<{f}, {c[0]}, {c[1]}, {c[2]}>()")
        if k == "loadcursor":
            dep = inst[2]
            c = self.p.cursor3(inst[1])
            kk = self.p.mids.index(dep)
            return self.bind(f"a.template ldm<{kk}, {c[0]}, {c[1]}, {c[2]}>()")
        if k == "loadindex":
            raise FormuraCompileError("index variables inside the step function are not supported "
                                      "by the GPU backend")
        if k == "store":
            f = self.p.fields.index(inst[1])
            self.emit(f"a.template st<{f}>({self.as_T(self.operand(micro, inst[2]))});")
            return None
        if k == "uniop":
            x = self.operand(micro, inst[2])
            op = inst[1]
            if op == "+":
                return x
            if op == "-":
                return self.bind(f"{self.P}::neg({self.as_T(x)})")
            f = op[len("external-call/"):]
            if f not in _EXT:
                raise FormuraCompileError(f"external function {f} is not available on the GPU")
            return self.bind(f"{self.P}::{_EXT[f]}({self.as_T(x)})")
        if k == "binop":
            op = inst[1]
            a = self.operand(micro, inst[2])
            b = self.operand(micro, inst[3])
            if op in _CMP:
                return self.bind(f"{self.P}::{_CMP_NAME[op]}({self.as_T(a)}, {self.as_T(b)})", "bool")
            if op in ("&&", "||"):
                return self.bind(f"({self.as_bool(a)} {op} {self.as_bool(b)})", "bool")
            if op == "*":
                for x, y in ((a, b), (b, a)):
                    if x[0] == "lit":
                        if x[1] == 1.0:
                            return y
                        if x[1] == -1.0:
                            return self.bind(f"{self.P}::neg({self.as_T(y)})")
                        if is_pow2(x[1]) and y[0] != "scaled":
                            return ("scaled", x[1], y)
                return self.bind(f"{self.P}::mul({self.as_T(a)}, {self.as_T(b)})")
            if op in ("+", "-"):
                if b[0] == "scaled":
                    c = b[1] if op == "+" else -b[1]
                    return self.bind(f"{self.P}::fma(T({c_double(c)}), {self.as_T(b[2])}, {self.as_T(a)}, fgb_ok)")
                if a[0] == "scaled":
                    rhs = self.as_T(b) if op == "+" else f"{self.P}::neg({self.as_T(b)})"
                    return self.bind(f"{self.P}::fma(T({c_double(a[1])}), {self.as_T(a[2])}, {rhs}, fgb_ok)")
                if op == "-" and a[0] == "lit" and a[1] == 1.0:
                    return self.bind(f"{self.P}::one_minus({self.as_T(b)})")
                fn = "add" if op == "+" else "sub"
                return self.bind(f"{self.P}::{fn}({self.as_T(a)}, {self.as_T(b)})")
            if op == "/":
                dep = micro[inst[3]].key[1]
                if an.om_uniform(dep):
                    if b[0] == "lit" and is_pow2(b[1]):
                        return self.bind(f"{self.P}::mul({self.as_T(a)}, T({c_double(1.0 / b[1])}))")
                    rc = self.recip_handle(dep)
                    if self.P == "M" and self.p.divisor_slots is not None:
                        if b[0] == "u":
                            self.p.divisor_slots.add(self.p.table_index(b[1]))
                        else:
                            self.p.divisor_slots = None
                    return self.bind(f"{self.P}::divu({self.as_T(a)}, {self.as_T(b)}, {self.as_T(rc)}, fgb_ok)")
                if self.reciprocal:
                    r = self.bind(f"{self.P}::div(T(1), {self.as_T(b)})")
                    return self.bind(f"{self.P}::mul({self.as_T(a)}, {self.as_T(r)})")
                den = self.as_T(b)
                self.div_seen[den] = self.div_seen.get(den, 0) + 1
                if self.div_uses.get(den, 0) >= 2:
                    y = self.bind(f"{self.P}::rcp({den})", prefix="r")
                    return self.bind(f"{self.P}::divr({self.as_T(a)}, {den}, {self.as_T(y)}, fgb_ok)")
                return self.bind(f"{self.P}::div({self.as_T(a)}, {den})")
            if op == "**":
                if b[0] == "lit" and b[1] == 2.0:
                    xa = self.as_T(a)
                    return self.bind(f"{self.P}::mul({xa}, {xa})")
                return self.bind(f"{self.P}::pow({self.as_T(a)}, {self.as_T(b)})")
            raise FormuraCompileError(f"operator {op} is not supported by the GPU backend")
        if k == "triop":
            c = self.operand(micro, inst[2])
            x = self.operand(micro, inst[3])
            y = self.operand(micro, inst[4])
            return self.bind(f"({self.as_bool(c)} ? {self.as_T(x)} : {self.as_T(y)})")
        raise FormuraCompileError(f"cannot emit {k}")

    def as_bool(self, h) -> str:
        if h[0] == "v" and h[2] == "bool":
            return h[1]
        if h[0] == "lit":
            return "true" if h[1] != 0.0 else "false"
        return f"({self.as_T(h)} != T(0))"

    def bind(self, expr: str, ctype: str = "T", prefix: Optional[str] = None):
        # value numbering: the same operation on the same operands is the same
        # value (every operation is deterministic), so it is computed once.
        # Reciprocals are named apart so that the other names do not depend
        # on whether a pass shares denominators.
        hit = self.memo.get((expr, ctype))
        if hit is not None:
            return hit
        if prefix is None:
            name = self.fresh()
        else:
            self.nr += 1
            name = f"{prefix}{self.nr}"
        self.emit(f"const {ctype} {name} = {expr};")
        h = ("v", name, ctype)
        self.memo[(expr, ctype)] = h
        return h


class _ProgramEmitter:
    def __init__(self, mm: MMProgram, name: str, runtime_params: List[str], graph: str = "step",
                 stage_adjoint: bool = False):
        self.mm = mm
        self.name = name
        self.graph = graph
        self.dim = mm.om.genv.dimension
        if self.dim > 3:
            raise FormuraCompileError("the GPU backend supports 1, 2 and 3 dimensions")
        self.fields = mm.fields
        self.an = _Analysis(mm, runtime_params, graph)
        self.runtime_params = list(runtime_params)
        cfg = mm.om.config
        self.mmg = {"step": mm.step, "first_step": mm.first_step, "filter": mm.filter}[graph]
        self.sleeve = {"step": cfg.sleeve, "first_step": cfg.sleeve0, "filter": cfg.filter_sleeve}[graph]
        if self.mmg is None:
            raise FormuraCompileError(f"the program has no {graph} function")
        self.stages = build_stages(self.mmg)
        self.mids = sorted({m for s in self.stages for m in s.mid_out})
        self.table: List[tuple] = []
        self.stage_adjoint = stage_adjoint
        self.adjoint_pairs: List[List[tuple]] = []
        # uniform-table slots the forward divides by (M::divu); None once a
        # divisor is a literal that is not a power of two
        self.divisor_slots: Optional[Set[int]] = set()
        rng = calc_range(self.mmg)
        s = self.sleeve
        stores = [n for n in self.mmg if n.is_store]
        offs = {rng[n.omid].offset() for n in stores}
        sizes = {rng[n.omid].size() for n in stores}
        if len(offs) != 1 or sizes != {2 * s}:
            raise FormuraCompileError(
                "the stores of this program cover a different extent than the sleeve; the "
                "reference's loop nest would write outside the grid")
        self.shift = 2 * s - offs.pop()
        reach = 0
        star = True
        for n in self.mmg:
            for mn in n.micro:
                if mn.inst[0] in ("loadstatic", "loadcursor"):
                    reach = max(reach, max(abs(x) for x in mn.inst[1]))
                    star = star and sum(1 for x in mn.inst[1] if x != 0) <= 1
        self.reach = reach
        # every load moves along at most one axis
        self.star = star

    def stage_reads(self) -> str:
        """Where each stage reads: the lowest and highest offset per axis of
        its state loads, and of its loads of the arrays of every earlier
        stage (lo > hi: no such load).  The fused multi-stage kernels size
        their shared-memory windows from these."""
        ns = len(self.stages)
        stage_of = {n.omid: st.index for st in self.stages for n in st.nodes}
        big = 1 << 20
        slo = [[big] * 3 for _ in range(ns)]
        shi = [[-big] * 3 for _ in range(ns)]
        rlo = [[[big] * 3 for _ in range(ns)] for _ in range(ns)]
        rhi = [[[-big] * 3 for _ in range(ns)] for _ in range(ns)]
        for st in self.stages:
            c = st.index
            for node in st.nodes:
                for mn in node.micro:
                    k = mn.inst[0]
                    if k == "loadstatic":
                        lo, hi = slo[c], shi[c]
                    elif k == "loadcursor" and stage_of[mn.inst[2]] != c:
                        lo, hi = rlo[c][stage_of[mn.inst[2]]], rhi[c][stage_of[mn.inst[2]]]
                    else:
                        continue
                    for a, x in enumerate(self.cursor3(mn.inst[1])):
                        lo[a] = min(lo[a], x)
                        hi[a] = max(hi[a], x)
        mid_stage = [stage_of[m] for m in self.mids] or [0]

        def arr(v):
            if isinstance(v, list):
                return "{" + ", ".join(arr(x) for x in v) + "}"
            return str(v)
        return (f"struct StageReads {{\n"
                f"  static constexpr int kMidStage[{len(mid_stage)}] = {arr(mid_stage)};\n"
                f"  static constexpr int kStateLo[{ns}][3] = {arr(slo)};\n"
                f"  static constexpr int kStateHi[{ns}][3] = {arr(shi)};\n"
                f"  static constexpr int kReadLo[{ns}][{ns}][3] = {arr(rlo)};\n"
                f"  static constexpr int kReadHi[{ns}][{ns}][3] = {arr(rhi)};\n"
                f"}};\n")

    def cursor3(self, c) -> List[int]:
        c = list(c)
        return [0] * (3 - len(c)) + c

    def table_index(self, entry) -> int:
        if entry not in self.table:
            self.table.append(entry)
        return self.table.index(entry)

    def emit(self, ns: Optional[str] = None, define: bool = True, stage_adjoint_type: Optional[str] = None,
             prog_extra: str = "") -> KernelProgram:
        """The program's device code in namespace `ns` (default
        fgb_gen_<name>), registered as a library program when `define`.
        `stage_adjoint_type` names a stage-adjoint list emitted elsewhere and
        `prog_extra` adds members to struct Prog."""
        ns = ns or f"fgb_gen_{self.name}"
        out = [f"// Device code generated by formura_gb300.generator.cuda for program '{self.name}'.",
               f"// Stencil expressions come from the program's step function; the kernel",
               f"// templates live in fgb_templates.cuh.",
               '#include "fgb_templates.cuh"', "",
               f"namespace {ns} {{", ""]
        stage_texts = []
        for st in self.stages:
            count = _StageEmitter(self, st)      # a pass that counts quotients per denominator
            for node in st.nodes:
                count.node(node)
            se = _StageEmitter(self, st, div_uses=count.div_seen)
            for node in st.nodes:
                se.node(node)
            body = "\n".join(se.lines)
            stage_texts.append(
                f"struct Stage{st.index} {{\n"
                f"  static constexpr int kIndex = {st.index};\n"
                f"  static constexpr bool kWritesState = {'true' if st.writes_state else 'false'};\n"

                f"  static constexpr int kMidOut = {len(st.mid_out)};\n"
                f"  template <class M, class A>\n"
                f"  static __device__ __forceinline__ bool run(const A& a, const typename M::U* __restrict__ U) {{\n"
                f"    using T = typename M::T;\n"
                f"    bool fgb_ok = true;\n"
                f"    (void)U;\n{body}\n    return fgb_ok;\n  }}\n}};\n")
        adj_src = None
        stage_adj = None
        if self.graph == "step" and len(self.stages) == 1 and not self.mids:
            from .adjoint import emit_adjoint
            try:
                adj_src, _ = emit_adjoint(self.mm, self.name, self)
            except FormuraCompileError:
                adj_src = None
        elif self.graph == "step" and self.stage_adjoint:
            from .adjoint import emit_stage_adjoints
            stage_adj, self.adjoint_pairs = emit_stage_adjoints(self)
        if adj_src:
            out.append(adj_src)
        if stage_adj:
            out.append(stage_adj)
        div_slots = sorted(self.divisor_slots) if self.divisor_slots is not None else []
        div_count = len(div_slots) if self.divisor_slots is not None else -1
        div_list = ", ".join(str(i) for i in div_slots) if div_slots else "0"
        out.append(self.stage_reads())
        sa = stage_adjoint_type or ('StageAdjointList' if stage_adj else 'void')
        out.append(f"struct Prog {{\n"
                   f"  using Adjoint = {'AdjointStep' if adj_src else 'void'};\n"
                   f"  using StageAdjoint = {sa};\n"
                   f"{prog_extra}"
                   f"  static constexpr int kDim = {self.dim};\n"
                   f"  static constexpr int kFields = {len(self.fields)};\n"
                   f"  static constexpr int kMids = {len(self.mids)};\n"
                   f"  static constexpr int kStages = {len(self.stages)};\n"
                   f"  static constexpr int kSleeve = {self.sleeve};\n"
                   f"  static constexpr int kShift = {self.shift};\n"
                   f"  static constexpr int kReach = {self.reach};\n"
                   f"  static constexpr bool kStar = {'true' if self.star else 'false'};\n"
                   f"  using Reads = StageReads;\n"
                   f"  static constexpr int kUniforms = {len(self.table)};\n"
                   f"  // uniform-table slots of the divisors (-1: a literal divisor)\n"
                   f"  static constexpr int kNumDivisors = {div_count};\n"
                   f"  static constexpr int kDivisors[{max(1, len(div_slots))}] = {{{div_list}}};\n"
                   f"}};\n")
        out += stage_texts
        out.append(f"}}  // namespace {ns}\n")
        if define:
            stage_list = ", ".join(f"{ns}::Stage{i}" for i in range(len(self.stages)))
            names = ", ".join(f'"{f}"' for f in self.fields)
            out.append(f"static const char* const fgb_fields_{self.name}[] = {{{names}}};")
            out.append(f"FGB_DEFINE_PROGRAM({self.name}, {ns}::Prog, fgb_fields_{self.name}, {stage_list})")
        return KernelProgram(self.name, self.dim, list(self.mm.om.genv.axes), list(self.fields),
                             self.sleeve, self.shift, self.reach, self.stages,
                             self.mids, list(self.table), self.runtime_params, "\n".join(out) + "\n")


def library_option(program: str, key: str, default=None):
    """A gpu_* option of a program shipped in formura_gb300/programs (the
    library's kernels were generated with it), or `default`."""
    from .config import decode_config
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "programs", program + ".yaml")
    if not os.path.exists(path):
        return default
    with open(path) as f:
        return decode_config(f.read()).gpu.get(key, default)


def store_shared_operands(g: Graph) -> Optional[Graph]:
    """The arrays the GPU step stores, chosen for HBM traffic.  Where two or
    more manifest nodes are each a state value plus or minus a constant times
    one shared non-manifest value X (MUSCL reconstruction: qL = q - s/2 and
    qR = q + s/2 from one limited slope s), X becomes the stored array and
    those nodes are evaluated at every point that reads them, from X and the
    state: one array instead of two or three, and one multiply-add per read.
    The operations and their order are the program's, so the results are
    the same bits.  None when no node fits."""
    shared: Dict[int, List[int]] = {}
    for i, nd in enumerate(g.nodes):
        inst = nd.inst
        if not nd.manifest or inst[0] != "binop" or inst[1] not in ("+", "-"):
            continue
        if g[inst[2]].inst[0] != "load":
            continue
        b = g[inst[3]]
        if b.manifest or b.inst[0] != "binop" or b.inst[1] != "*":
            continue
        x, y = b.inst[2], b.inst[3]
        xo = y if g[x].inst[0] == "imm" else (x if g[y].inst[0] == "imm" else None)
        if xo is None or g[xo].manifest or g[xo].inst[0] in ("imm", "load", "loadindex"):
            continue
        if g[xo].type != nd.type:
            continue
        shared.setdefault(xo, []).append(i)
    groups = {x: ns for x, ns in shared.items() if len(ns) >= 2}
    if not groups:
        return None
    g2 = Graph()
    g2.nodes = list(g.nodes)
    for x, ns in groups.items():
        g2.nodes[x] = dataclasses.replace(g.nodes[x], manifest=True)
        for i in ns:
            g2.nodes[i] = dataclasses.replace(g.nodes[i], manifest=False)
    return g2


def gpu_step_program(mm: MMProgram) -> MMProgram:
    """The program as the GPU step evaluates it: the same graph, with the
    stored arrays chosen by store_shared_operands."""
    g2 = store_shared_operands(mm.om.step_graph)
    if g2 is None:
        return mm
    om2 = dataclasses.replace(mm.om, step_graph=g2)
    return dataclasses.replace(mm, om=om2, step=manifest_graph(g2, mm.om.genv.dimension))


def _emit_with_own_adjoint(mm: MMProgram, mm2: MMProgram, name: str,
                           runtime_params: List[str]) -> Optional[KernelProgram]:
    """A program whose GPU step stores other arrays (mm2) than the program's
    own (mm) and that has a stage adjoint: the forward steps come from mm2,
    the adjoint and the forward stages that recompute its arrays from mm (the
    partial sums are generated for those arrays; generated for mm2's they
    would read the state at many more cursors).  Both share one uniform
    table: the forward's starts with the adjoint's entries.  None when the
    two have different stage counts."""
    adj = _ProgramEmitter(mm, name, runtime_params, "step", True)
    fwd = _ProgramEmitter(mm2, name, runtime_params, "step", False)
    if len(adj.stages) != len(fwd.stages):
        return None
    ans = f"fgb_gen_{name}_adj"
    adj_kp = adj.emit(ns=ans, define=False)
    fwd.table = list(adj.table)
    stages = ", ".join(f"{ans}::Stage{i}" for i in range(len(adj.stages)))
    extra = (f"  // the program's own forward stages, whose arrays the adjoint reads\n"
             f"  using AdjProg = {ans}::Prog;\n"
             f"  using AdjStages = fgb::StageTypes<{stages}>;\n")
    kp = fwd.emit(stage_adjoint_type=f"{ans}::StageAdjointList", prog_extra=extra)
    kp.source = adj_kp.source + "\n" + kp.source
    kp.graph = "step"
    return kp


def emit_cuda(mm: MMProgram, name: str, runtime_params: Optional[List[str]] = None,
              graph: str = "step", stage_adjoint: Optional[bool] = None) -> KernelProgram:
    """Device code of the step function (or of first_step / filter, which
    become library programs named <name>__first_step / <name>__filter).
    Multi-stage steps get an adjoint when `stage_adjoint` is set; by default
    when the library's program sets `gpu_adjoint: 1`."""
    if stage_adjoint is None:
        stage_adjoint = bool(library_option(name, "gpu_adjoint", 0))
    if graph == "step":
        mm2 = gpu_step_program(mm)
        if mm2 is not mm and stage_adjoint:
            kp = _emit_with_own_adjoint(mm, mm2, name, runtime_params or [])
            if kp is not None:
                return kp
        else:
            mm = mm2
    kp = _ProgramEmitter(mm, name if graph == "step" else f"{name}__{graph}",
                         runtime_params or [], graph, stage_adjoint and graph == "step").emit()
    kp.graph = graph
    return kp


def eval_utree(an: "_Analysis", tree, params=None) -> float:
    """Host value of a grid-independent expression tree: ('lit', x),
    ('node', omid), ('recip', omid) or (op, a[, b]) with op in + - * / neg."""
    k = tree[0]
    if k == "lit":
        return float(tree[1])
    if k == "node":
        return float(an.om_value(tree[1], params))
    if k == "recip":
        return 1.0 / float(an.om_value(tree[1], params))
    if k == "neg":
        return -eval_utree(an, tree[1], params)
    a = eval_utree(an, tree[1], params)
    b = eval_utree(an, tree[2], params)
    return {"+": a + b, "-": a - b, "*": a * b, "/": a / b}[k]


def uniform_table(mm: MMProgram, kp: KernelProgram, params: Optional[Dict[str, float]] = None) -> List[float]:
    """Host values of the runtime uniform table for one configuration."""
    an = _Analysis(mm, kp.runtime_params, getattr(kp, "graph", "step"))
    out = []
    for entry in kp.uniform_exprs:
        kind = entry[0]
        if kind == "node":
            out.append(float(an.om_value(entry[1], params)))
        elif kind == "recip":
            out.append(1.0 / float(an.om_value(entry[1], params)))
        elif kind == "expr":
            out.append(eval_utree(an, entry[1], params))
        else:
            raise FormuraCompileError(f"unknown uniform table entry {kind}")
    return out
