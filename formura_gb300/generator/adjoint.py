"""Adjoint (reverse-mode derivative) of a single-stage step function, emitted
as a stage functor for the kernel templates.

The forward step writes ``out[f][p + shift] = F_f(u at p + d for the cursors
d it reads)``.  Its transpose, applied to an adjoint state ``lam`` (the
derivative of a scalar loss with respect to ``out``), is

    lam_in[g][q] = sum over f and cursors d of field g:
                   lam[f][q - d + shift] * dF_f/du_g[d]  evaluated at p = q - d.

The partial derivatives come from reverse-mode differentiation of the
program's own SSA chain (seed 1 at each store).  Terms that do not depend
on the grid are carried symbolically and folded on the host into the
uniform table, so a linear stencil (heat) costs one multiply-add per cursor;
terms that do (the reaction terms of Gray-Scott) are evaluated at ``q - d``
from the forward state.  The reference has no adjoint; this is the
``Formura_Backward`` extension of the generated API, and the checkpointed
gradient of the runtime (``fgb_gradient_*``) calls this step.
"""
from __future__ import annotations

import re
from typing import Dict, List, Tuple

from .cuda import _ProgramEmitter, _StageEmitter, c_double
from .manifest import MMProgram
from .translate import FormuraCompileError

_CMP = {"<", ">", "<=", ">=", "==", "!=", "&&", "||"}


def _simplify(t):
    k = t[0]
    if k in ("lit", "node", "recip"):
        return t
    if k == "neg":
        a = _simplify(t[1])
        if a[0] == "lit":
            return ("lit", -a[1])
        return ("neg", a)
    a, b = _simplify(t[1]), _simplify(t[2])
    if a[0] == "lit" and b[0] == "lit":
        return ("lit", {"+": a[1] + b[1], "-": a[1] - b[1], "*": a[1] * b[1], "/": a[1] / b[1]}[k])
    if k == "*":
        if a == ("lit", 1.0):
            return b
        if b == ("lit", 1.0):
            return a
    if k == "/" and b == ("lit", 1.0):
        return a
    return (k, a, b)


class _OffsetEmitter(_StageEmitter):
    """Forward values of the step at cursor offset ``e`` from the thread's cell."""

    def __init__(self, prog, stage, shared_lines, memo, counter):
        super().__init__(prog, stage, policy="D", reciprocal=True)
        self.lines = shared_lines
        self.memo = memo
        self._counter = counter
        self.offset = (0, 0, 0)

    def fresh(self) -> str:
        self._counter[0] += 1
        return f"t{self._counter[0]}"

    def micro(self, mn, micro, node):
        inst = mn.inst
        if inst[0] == "loadstatic":
            c = self.p.cursor3(inst[1])
            c = [a + b for a, b in zip(c, self.offset)]
            f = self.p.fields.index(inst[2])
            return self.bind(f"a.template ld<{f}, {c[0]}, {c[1]}, {c[2]}>()")
        if inst[0] == "store":
            return None
        return super().micro(mn, micro, node)


class _Algebra:
    """Values of the reverse sweep: ('u', tree) grid-independent, or an
    emitted handle of the offset emitter."""

    def __init__(self, fe: _OffsetEmitter, pe: _ProgramEmitter):
        self.fe, self.pe = fe, pe

    def T(self, v) -> str:
        if v[0] == "u":
            t = _simplify(v[1])
            if t[0] == "lit":
                return f"T({c_double(t[1])})"
            return f"U[{self.pe.table_index(('expr', t))}]"
        return self.fe.as_T(v)

    def binop(self, k, a, b, fn):
        if a[0] == "u" and b[0] == "u":
            return ("u", _simplify((k, a[1], b[1])))
        if k == "*":
            for x, y in ((a, b), (b, a)):
                if x == ("u", ("lit", 1.0)):
                    return y
        if k == "/" and b[0] == "u":
            return self.fe.bind(f"D::mul({self.T(a)}, {self.T(('u', ('/', ('lit', 1.0), b[1])))})")
        return self.fe.bind(f"D::{fn}({self.T(a)}, {self.T(b)})")

    def add(self, a, b):
        return self.binop("+", a, b, "add")

    def sub(self, a, b):
        return self.binop("-", a, b, "sub")

    def mul(self, a, b):
        return self.binop("*", a, b, "mul")

    def div(self, a, b):
        return self.binop("/", a, b, "div")

    def over(self, a, b):
        """a / b for the derivative terms: through the reciprocal of b, which
        is bound once per denominator (both partials of a quotient and every
        later use share it), so a forward division costs one division in the
        reverse sweep rather than two."""
        if b[0] == "u":
            return self.div(a, b)
        return self.mul(a, self.fe.bind(f"D::div(T(1), {self.T(b)})"))

    def neg(self, a):
        if a[0] == "u":
            return ("u", _simplify(("neg", a[1])))
        return self.fe.bind(f"D::neg({self.T(a)})")


def emit_adjoint(mm: MMProgram, name: str, pe: _ProgramEmitter = None):
    """(CUDA source of ``struct AdjointStep``, program emitter holding its table).
    Pass the forward program's emitter so that both share one uniform table."""
    pe = pe or _ProgramEmitter(mm, name, [])
    if len(pe.stages) != 1 or pe.mids:
        raise FormuraCompileError("the generated adjoint covers single-stage programs")
    stage = pe.stages[0]
    fields = pe.fields
    shift = pe.shift
    an = pe.an
    lines: List[str] = []
    memo: Dict[tuple, tuple] = {}
    counter = [0]
    offsets = set()
    for node in stage.nodes:
        for mn in node.micro:
            if mn.inst[0] == "loadstatic":
                offsets.add(tuple(-x for x in pe.cursor3(mn.inst[1])))
    acc: Dict[int, List[str]] = {g: [] for g in range(len(fields))}

    for e in sorted(offsets):
        fe = _OffsetEmitter(pe, stage, lines, memo, counter)
        fe.offset = e
        alg = _Algebra(fe, pe)
        for node in stage.nodes:
            if not node.is_store:
                raise FormuraCompileError("single-stage programs store every manifest value")
            micro = node.micro
            fwd: Dict[int, tuple] = {}

            def value(i):
                """Forward value of micro node i at this offset (lazy)."""
                if i in fwd:
                    return fwd[i]
                mn = micro[i]
                if mn.inst[0] != "loadstatic" and an.om_uniform(mn.key[1]):
                    omid = mn.key[1]
                    v = ("u", ("node", omid)) if an.om_config_dependent(omid) else \
                        ("u", ("lit", float(an.om_value(omid))))
                else:
                    for j in range(i + 1):
                        if micro[j].key not in fe.var:
                            h = fe.micro(micro[j], micro, node)
                            if h is not None:
                                fe.var[micro[j].key] = h
                    v = fe.var[mn.key]
                fwd[i] = v
                return v

            fe.var = {}
            store = micro[-1]
            f = fields.index(store.inst[1])
            bar: Dict[int, List[tuple]] = {store.inst[2]: [("u", ("lit", 1.0))]}
            for i in range(len(micro) - 2, -1, -1):
                if i not in bar:
                    continue
                mn = micro[i]
                inst = mn.inst
                k = inst[0]
                total = bar[i][0]
                for t in bar[i][1:]:
                    total = alg.add(total, t)
                bar[i] = [total]
                if k in ("imm", "loadindex", "loadcursor", "loadstatic"):
                    continue
                if an.om_uniform(mn.key[1]):
                    continue
                Y = total

                def push(j, v):
                    # v is a thunk: derivative terms are built only for operands
                    # that depend on the grid
                    if micro[j].inst[0] == "loadstatic" or not an.om_uniform(micro[j].key[1]):
                        bar.setdefault(j, []).append(v())

                if k == "uniop":
                    op, a = inst[1], inst[2]
                    if op == "+":
                        push(a, lambda: Y)
                    elif op == "-":
                        push(a, lambda: alg.neg(Y))
                    else:
                        fn = op[len("external-call/"):]
                        x = alg.T(value(a))
                        y = alg.T(value(i))
                        d = {"sqrt": f"D::div(T(0.5), {y})", "exp": y, "log": f"D::div(T(1), {x})",
                             "sin": f"D::cos({x})", "cos": f"D::neg(D::sin({x}))",
                             "fabs": f"({x} < T(0) ? T(-1) : T(1))"}.get(fn)
                        if d is None:
                            raise FormuraCompileError(f"no derivative for {fn}")
                        push(a, lambda: alg.mul(Y, fe.bind(d)))
                elif k == "binop":
                    op, a, b = inst[1], inst[2], inst[3]
                    if op in _CMP:
                        continue
                    if op == "+":
                        push(a, lambda: Y)
                        push(b, lambda: Y)
                    elif op == "-":
                        push(a, lambda: Y)
                        push(b, lambda: alg.neg(Y))
                    elif op == "*":
                        push(a, lambda: alg.mul(Y, value(b)))
                        push(b, lambda: alg.mul(Y, value(a)))
                    elif op == "/":
                        push(a, lambda: alg.over(Y, value(b)))
                        if not an.om_uniform(micro[b].key[1]):
                            push(b, lambda: alg.neg(alg.over(alg.mul(Y, value(i)), value(b))))
                    elif op == "**":
                        A, B = alg.T(value(a)), alg.T(value(b))
                        push(a, lambda: alg.mul(Y, fe.bind(f"D::mul({B}, D::pow({A}, D::sub({B}, T(1))))")))
                        if not an.om_uniform(micro[b].key[1]):
                            push(b, lambda: alg.mul(Y, fe.bind(f"D::mul({alg.T(value(i))}, D::log({A}))")))
                    else:
                        raise FormuraCompileError(f"no derivative for {op}")
                elif k == "triop":
                    c, a, b = inst[2], inst[3], inst[4]
                    C = fe.as_bool(value(c))
                    push(a, lambda: fe.bind(f"({C} ? {alg.T(Y)} : T(0))"))
                    push(b, lambda: fe.bind(f"({C} ? T(0) : {alg.T(Y)})"))
            s3 = [x + shift if i >= 3 - pe.dim else x for i, x in enumerate(e)]
            lam = None
            for i, mn in enumerate(micro):
                if mn.inst[0] == "loadstatic" and i in bar:
                    c = tuple(pe.cursor3(mn.inst[1]))
                    if tuple(-x for x in c) == e:
                        if lam is None:
                            lam = fe.bind(f"a.template ldl<{f}, {s3[0]}, {s3[1]}, {s3[2]}>()")
                        g = fields.index(mn.inst[2])
                        acc[g].append(alg.T(alg.mul(lam, bar[i][0])))
    out = []
    for g in range(len(fields)):
        terms = acc[g]
        expr = terms[0] if terms else "T(0)"
        for t in terms[1:]:
            expr = f"D::add({expr}, {t})"
        out.append(f"    a.template stl<{g}>({expr});")
    body = "\n".join("    " + l.strip() for l in lines) + "\n" + "\n".join(out)
    return (f"struct AdjointStep {{\n"
            f"  template <class M, class A>\n"
            f"  static __device__ __forceinline__ bool run(const A& a, const typename M::U* __restrict__ U) {{\n"
            f"    using T = typename M::T;\n    using D = typename M::Deriv;\n    bool fgb_ok = true;\n"
            f"    (void)U;\n{body}\n    return fgb_ok;\n  }}\n}};\n"), pe


# ---------------------------------------------------------------------------
# multi-stage steps
# ---------------------------------------------------------------------------
def _as_alg(h):
    """Forward handle of the stage emitter in the form _Algebra expects."""
    if h[0] == "lit":
        return ("u", ("lit", float(h[1])))
    if h[0] == "u":
        return ("u", h[1])
    return h


_VAR = re.compile(r"\bt\d+\b")
_LDM = re.compile(r"a\.template ldm<(\d+),")


def _live_mids(lines: List[str]) -> set:
    """Forward arrays whose values a partial-sum kernel really uses: the
    ldm loads reachable from its stp lines through the SSA definitions (the
    rest is dead code the compiler drops)."""
    defs: Dict[str, str] = {}
    roots: List[str] = []
    for line in lines:
        text = line.strip()
        m = re.match(r"const \w+ (t\d+) = (.*);$", text)
        if m:
            defs[m.group(1)] = m.group(2)
        elif text.startswith("a.template stp<"):
            roots.append(text)
    live: set = set()
    todo = [v for r in roots for v in _VAR.findall(r)]
    mids: set = set()
    while todo:
        v = todo.pop()
        if v in live or v not in defs:
            continue
        live.add(v)
        expr = defs[v]
        mids.update(int(k) for k in _LDM.findall(expr))
        todo.extend(_VAR.findall(expr))
    return mids


def _stage_outputs(st) -> List[tuple]:
    """The outputs of a stage in emission order: ('s', node) for a store of
    the new state, ('m', node) for a manifest array kept in HBM."""
    out = []
    for node in st.nodes:
        if node.is_store:
            out.append(("s", node))
        if node.omid in st.mid_out:
            out.append(("m", node))
    return out


def _stage_is_linear(an, st) -> bool:
    """True when every output of the stage is a linear combination of its
    inputs with grid-independent coefficients: no product or quotient of two
    grid values, no function, power, comparison or selection on one.  The
    partial sums of such a stage are the adjoints of its outputs times
    constants, so they are cheaper to form where they are gathered than to
    store."""
    for node in st.nodes:
        micro = node.micro
        for mn in micro:
            inst = mn.inst
            k = inst[0]
            if k in ("imm", "loadstatic", "loadcursor", "loadindex", "store") or an.om_uniform(mn.key[1]):
                continue

            def grid(j):
                return not an.om_uniform(micro[j].key[1]) or micro[j].inst[0] in ("loadstatic", "loadcursor")

            if k == "uniop":
                if inst[1] not in ("+", "-"):
                    return False
            elif k == "binop":
                op, a, b = inst[1], inst[2], inst[3]
                if op in _CMP or op == "**":
                    return False
                if op == "*" and grid(a) and grid(b):
                    return False
                if op == "/" and grid(b):
                    return False
            elif k == "triop":
                if grid(inst[2]):
                    return False
            else:
                return False
    return True


# a partial-sum kernel holds the forward values of its outputs' backward
# slice in registers: stages larger than this many micro operations are cut
# into several kernels by output, so that none of them spills
_PARTIAL_MICRO_OPS = 1000


def emit_stage_adjoints(pe: _ProgramEmitter):
    """Adjoint of a step made of several stages (HLLC, HLLD), as partial-sum
    functors and one gather functor per stage.

    Stage s computes its outputs o (manifest arrays, or the new state) at p
    from its inputs x (state fields and earlier arrays) read at p + c.  With
    lam_o the adjoint of each output:

    * ``AdjStage<s>_<g>`` evaluates the stage forward at p, seeds the reverse
      sweep of its SSA chain with lam_o(p) for the outputs o of group g (lam
      of the new state is read at p + shift, where the forward wrote it) and
      adds, for every input read (x, c), lam_o(p) * do(p)/dx(p + c) to the
      partial sum P_(x,c,g)(p) of its own.  Large stages are cut into groups
      of outputs so that no kernel spills;
    * ``AdjGather<s>`` forms lam_x(q) = sum_(c,g) P_(x,c,g)(q - c) in a fixed order,
      storing it for the first stage (in reverse order) that reads x and
      adding to it for the others;
    * a stage whose outputs are linear in its inputs with grid-independent
      coefficients (``kDirect``) launches no partial-sum kernel: its gather
      evaluates the partial-sum functors at q - c itself, which reads the
      adjoints of the outputs instead of the (more numerous) stored sums.

    Stages run from last to first, after the forward arrays of the step were
    recomputed from u_n.  Nothing is atomic, so the result is deterministic.
    Returns (source, [pairs per stage])."""
    S = len(pe.stages)
    if S < 2:
        raise FormuraCompileError("single-stage programs use the one-pass adjoint")
    stage_of = {n.omid: s.index for s in pe.stages for n in s.nodes}
    fields = pe.fields
    an = pe.an
    shift3 = [pe.shift if i >= 3 - pe.dim else 0 for i in range(3)]
    pass1: Dict[int, str] = {}
    pair_lists: List[List[tuple]] = []
    needed_mids: set = set()          # forward arrays the partial sums read
    for st in pe.stages:
        texts: List[str] = []
        outs = _stage_outputs(st)
        nmicro = sum(len(n.micro) for n in st.nodes)
        ngroups = max(1, min(len(outs), -(-nmicro // _PARTIAL_MICRO_OPS)))
        per = -(-len(outs) // ngroups)
        groups = [outs[i:i + per] for i in range(0, len(outs), per)]
        pairs: List[tuple] = []           # (x, c, group) partial sums of the stage, in kernel order
        part_names: List[str] = []
        for gi, group in enumerate(groups):
            # the forward at p in the derivative policy, quotients through the
            # reciprocals the reverse sweep needs anyway; stores are no-ops and
            # unused values are dropped
            se = _StageEmitter(pe, st, policy="D", reciprocal=True)
            for node in st.nodes:
                se.node(node)
            defs: Dict[tuple, tuple] = {}
            order: List[tuple] = []
            for node in st.nodes:
                for idx, mn in enumerate(node.micro):
                    if mn.key not in defs:
                        defs[mn.key] = (node, idx)
                        order.append(mn.key)
            alg = _Algebra(se, pe)
            bar: Dict[tuple, List[tuple]] = {}
            for kind, node in group:
                if kind == "s":
                    store = node.micro[-1]
                    f = fields.index(store.inst[1])
                    lam = se.bind(f"a.template ldl<{f}, {shift3[0]}, {shift3[1]}, {shift3[2]}>()")
                    bar.setdefault(node.micro[store.inst[2]].key, []).append(lam)
                else:
                    k = pe.mids.index(node.omid)
                    lam = se.bind(f"a.template ldlm<{k}>()")
                    bar.setdefault(node.micro[-1].key, []).append(lam)
            touched: List[tuple] = []
            pair_val: Dict[tuple, tuple] = {}
            _reverse_sweep(se, alg, an, fields, pe, stage_of, st, defs, order, bar, touched, pair_val)
            for pair in touched:
                pairs.append(pair + (gi,))
                se.emit(f"a.template stp<{len(pairs) - 1}>({alg.T(pair_val[pair])});")
            needed_mids |= _live_mids(se.lines)
            body = "\n".join(se.lines)
            name = f"AdjStage{st.index}_{gi}"
            part_names.append(name)
            texts.append(f"struct {name} {{\n"
                         f"  template <class M, class A>\n"
                         f"  static __device__ __forceinline__ bool run(const A& a, const typename M::U* __restrict__ U) {{\n"
                         f"    using T = typename M::T;\n    using D = typename M::Deriv;\n    bool fgb_ok = true;\n"
                         f"    (void)U;\n{body}\n    return fgb_ok;\n  }}\n}};\n")
        pair_lists.append(pairs)
        direct = "true" if _stage_is_linear(an, st) else "false"
        texts.append(f"struct AdjStage{st.index} {{\n"
                     f"  static constexpr int kPairs = {len(pairs)};\n"
                     f"  static constexpr bool kDirect = {direct};\n"
                     f"  using Parts = fgb::AdjParts<{', '.join(part_names)}>;\n}};\n")
        pass1[st.index] = "\n".join(texts)
    # gathers, in the order the adjoint runs them (last stage first)
    written = set()
    gathers: Dict[int, str] = {}
    for st in reversed(pe.stages):
        pairs = pair_lists[st.index]
        targets: Dict[tuple, List[int]] = {}
        for j, p in enumerate(pairs):
            targets.setdefault(p[:2], []).append(j)
        lines = []
        for tgt in sorted(targets):
            terms = [f"a.template ldp<{j}, {-pairs[j][2][0]}, {-pairs[j][2][1]}, {-pairs[j][2][2]}>()"
                     for j in targets[tgt]]
            expr = terms[0]
            for t in terms[1:]:
                expr = f"M::add({expr}, {t})"
            first = "true" if tgt not in written else "false"
            written.add(tgt)
            fn = "accs" if tgt[0] == "s" else "accm"
            lines.append(f"    a.template {fn}<{tgt[1]}, {first}>({expr});")
        if st.index == 0:
            for g in range(len(fields)):
                if ("s", g) not in written:
                    lines.append(f"    a.template accs<{g}, true>(T(0));")
        gathers[st.index] = (f"struct AdjGather{st.index} {{\n"
                             f"  template <class M, class A>\n"
                             f"  static __device__ __forceinline__ bool run(const A& a, const typename M::U* __restrict__ U) {{\n"
                             f"    using T = typename M::T;\n    (void)U;\n" + "\n".join(lines) +
                             "\n    return true;\n  }\n};\n")
    # the stages an adjoint step recomputes: those whose arrays the partial
    # sums read, and the stages those depend on
    producer = {pe.mids.index(m): s.index for s in pe.stages for m in s.mid_out}
    recompute = [False] * S
    todo = sorted({producer[k] for k in needed_mids})
    while todo:
        s_ = todo.pop()
        if recompute[s_]:
            continue
        recompute[s_] = True
        for node in pe.stages[s_].nodes:
            for mn in node.micro:
                if mn.inst[0] == "loadcursor" and stage_of[mn.inst[2]] != s_:
                    todo.append(stage_of[mn.inst[2]])
    src = "\n".join(pass1[s] + gathers[s] for s in range(S))
    flags = ", ".join("true" if r else "false" for r in recompute)
    src += f"struct AdjointRecompute {{\n  static constexpr bool kStage[{S}] = {{{flags}}};\n}};\n"
    pairs_list = ", ".join(f"fgb::AdjointStagePair<AdjStage{s}, AdjGather{s}>" for s in range(S))
    src += f"using StageAdjointList = fgb::AdjointStages<AdjointRecompute, {pairs_list}>;\n"
    return src, pair_lists


def _reverse_sweep(se, alg, an, fields, pe, stage_of, st, defs, order, bar, touched, pair_val):
    """Reverse sweep of one stage's SSA chain from the seeds in `bar`:
    appends the (input array, cursor) pairs reached to `touched` and their
    summed adjoints to `pair_val`."""

    def value(key):
        return _as_alg(se.var[key])

    for key in reversed(order):
        if key not in bar:
            continue
        node, i = defs[key]
        micro = node.micro
        inst = micro[i].inst
        k = inst[0]
        total = bar[key][0]
        for t in bar[key][1:]:
            total = alg.add(total, t)
        if k == "loadstatic" or (k == "loadcursor" and stage_of[inst[2]] != st.index):
            kind = ("s", fields.index(inst[2])) if k == "loadstatic" else ("m", pe.mids.index(inst[2]))
            pair = kind + (tuple(pe.cursor3(inst[1])),)
            if pair in pair_val:
                pair_val[pair] = alg.add(pair_val[pair], total)
            else:
                touched.append(pair)
                pair_val[pair] = total
            continue
        if k in ("imm", "loadindex", "store", "loadcursor"):
            continue
        if an.om_uniform(key[1]):
            continue
        Y = total

        def opk(j, micro=micro):
            return micro[j].key

        def push(j, v, micro=micro):
            mj = micro[j]
            if mj.inst[0] in ("loadstatic", "loadcursor") or not an.om_uniform(mj.key[1]):
                bar.setdefault(mj.key, []).append(v())

        if k == "uniop":
            op, a = inst[1], inst[2]
            if op == "+":
                push(a, lambda: Y)
            elif op == "-":
                push(a, lambda: alg.neg(Y))
            else:
                fn = op[len("external-call/"):]
                x = alg.T(value(opk(a)))
                y = alg.T(value(key))
                d = {"sqrt": f"D::div(T(0.5), {y})", "exp": y, "log": f"D::div(T(1), {x})",
                     "sin": f"D::cos({x})", "cos": f"D::neg(D::sin({x}))",
                     "fabs": f"({x} < T(0) ? T(-1) : T(1))"}.get(fn)
                if d is None:
                    raise FormuraCompileError(f"no derivative for {fn}")
                push(a, lambda: alg.mul(Y, se.bind(d)))
        elif k == "binop":
            op, a, b = inst[1], inst[2], inst[3]
            if op in _CMP:
                continue
            if op == "+":
                push(a, lambda: Y)
                push(b, lambda: Y)
            elif op == "-":
                push(a, lambda: Y)
                push(b, lambda: alg.neg(Y))
            elif op == "*":
                push(a, lambda: alg.mul(Y, value(opk(b))))
                push(b, lambda: alg.mul(Y, value(opk(a))))
            elif op == "/":
                push(a, lambda: alg.over(Y, value(opk(b))))
                if not an.om_uniform(micro[b].key[1]) or micro[b].inst[0] in ("loadstatic", "loadcursor"):
                    push(b, lambda: alg.neg(alg.over(alg.mul(Y, value(key)), value(opk(b)))))
            elif op == "**":
                A, B = alg.T(value(opk(a))), alg.T(value(opk(b)))
                push(a, lambda: alg.mul(Y, se.bind(f"D::mul({B}, D::pow({A}, D::sub({B}, T(1))))")))
                if not an.om_uniform(micro[b].key[1]):
                    push(b, lambda: alg.mul(Y, se.bind(f"D::mul({alg.T(value(key))}, D::log({A}))")))
            else:
                raise FormuraCompileError(f"no derivative for {op}")
        elif k == "triop":
            c, a, b = inst[2], inst[3], inst[4]
            C = se.as_bool(value(opk(c)))
            push(a, lambda: se.bind(f"({C} ? {alg.T(Y)} : T(0))"))
            push(b, lambda: se.bind(f"({C} ? T(0) : {alg.T(Y)})"))
