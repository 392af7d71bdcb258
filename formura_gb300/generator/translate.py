"""Orthotope Machine (OM) translation: symbolic evaluation of a Formura
program into a dataflow graph over whole-grid values.

Restates ``src/Formura/OrthotopeMachine/Translate.hs`` for the language the
parser accepts:

* node insertion with sequential ids ``Translate.hs:135-153``;
* the type meet (``Type.hs:111-138``; ``Graph.hs:144-161``) and ``castVal``
  ``Translate.hs:166-172``;
* unary/binary/ternary operators, including function lifting, tuple
  broadcasting and composition ``.`` ``Translate.hs:184-269``
  (``TExpr.hs:22-31`` for the ternary broadcast);
* grid indexing with rational offsets: the integer part becomes a ``Shift``
  node, the fractional part stays in the grid type ``Translate.hs:287-313``;
* application, tuple projection by a constant ``Translate.hs:322-351``;
* lambdas resolve their free identifiers at definition time except inside
  ``let`` bindings, which are resolved at the call site
  ``Translate.hs:353-383``;
* bindings enter scope one by one, index variables become ``LoadIndex``
  nodes, declared types cast values, ``manifest`` marks nodes, ``extern``
  functions become external calls ``Translate.hs:453-527``;
* ``genGlobalFunction`` (``Load``/``Store``) ``Translate.hs:559-584``;
* ``calcSleeve`` with the lexicographic ``max`` of ``Vec`` ``Translate.hs:613-623``
  (``Vec.hs:63-64``);
* ``genOMProgram`` ``Translate.hs:625-686``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from fractions import Fraction
from typing import Dict, List, Optional, Tuple

from .config import InternalConfig, convert_config
from .syntax import COMPARISONS, ELEMENT_TYPES, Program


class FormuraCompileError(ValueError):
    pass


# --------------------------------------------------------------------------
# types
# --------------------------------------------------------------------------
TOP = ("top",)


def elem(name):
    return ("elem", name)


def meet(a, b):
    """``semiLatticeOfOMNodeType`` (``Graph.hs:147-161``)."""
    r = _meet_go(a, b)
    if r == TOP:
        return _meet_go(b, a)
    return r


def _meet_go(x, y):
    if x == y:
        return x
    if x[0] == "elem" and y[0] == "elem":
        ia = ELEMENT_TYPES.index(x[1]) if x[1] in ELEMENT_TYPES else 10 ** 9
        ib = ELEMENT_TYPES.index(y[1]) if y[1] in ELEMENT_TYPES else 10 ** 9
        m = max(ia, ib)
        return TOP if m >= len(ELEMENT_TYPES) else elem(ELEMENT_TYPES[m])
    if x[0] == "elem" and y[0] == "gridtype":
        d = meet(x, y[2])
        return TOP if d == TOP else ("gridtype", y[1], d)
    if x[0] == "gridtype" and y[0] == "gridtype":
        if tuple(x[1]) == tuple(y[1]):
            return ("gridtype", x[1], meet(x[2], y[2]))
        return TOP
    return TOP


def map_elem_type(f, t):
    if t[0] == "elem":
        return elem(f(t[1]))
    if t[0] == "gridtype":
        return ("gridtype", t[1], map_elem_type(f, t[2]))
    return t


def is_boolish(t):
    if t[0] == "elem":
        return t[1] == "bool"
    if t[0] == "gridtype":
        return is_boolish(t[2])
    return False


def elem_of(t):
    """Element type name of a node type (``toMicroType``)."""
    while t[0] == "gridtype":
        t = t[2]
    if t[0] != "elem":
        raise FormuraCompileError("Top type encountered while manifestation")
    return t[1]


# --------------------------------------------------------------------------
# graph
# --------------------------------------------------------------------------
@dataclass
class Node:
    inst: tuple          # ('imm', r) ('uniop', op, a) ('binop', op, a, b)
                         # ('triop', op, a, b, c) ('shift', vec, a) ('load', name)
                         # ('loadindex', axis) ('store', name, a)
    type: tuple
    manifest: bool = False
    name: Optional[str] = None   # source name annotation


class Graph:
    def __init__(self):
        self.nodes: List[Node] = []

    def insert(self, inst, typ) -> tuple:
        nid = len(self.nodes)
        self.nodes.append(Node(inst, typ))
        return ("node", nid, typ)

    def __getitem__(self, i) -> Node:
        return self.nodes[i]

    def __len__(self):
        return len(self.nodes)


# values: ('node', id, type) | ('tuple', [..]) | ('fun', lhs, body) | ('imm', r)
HOLDER = ("holder",)


@dataclass
class GlobalEnv:
    dimension: int
    axes: List[str]
    grid_struct_type_name: str
    grid_struct_instance_name: str
    comm_bases: List[List[int]]


def comm_bases_for(dim):
    """``Translate.hs:106-110``."""
    if dim == 1:
        return [[1]]
    if dim == 2:
        return [[1, 0], [0, 1], [1, 1]]
    if dim == 3:
        return [[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1], [0, 1, 1], [1, 1, 1]]
    raise FormuraCompileError("Not support")


def names_of_lhs(l):
    k = l[0]
    if k == "ident":
        return l
    if k in ("grid",):
        return names_of_lhs(l[2])
    if k == "vector":
        return names_of_lhs(l[2])
    if k == "tuple":
        return ("tuple", [names_of_lhs(x) for x in l[1]])
    raise FormuraCompileError(f"unexpected l-expression {l[0]}")


def tuple_contents(x):
    if x[0] == "tuple":
        out = []
        for y in x[1]:
            out.extend(tuple_contents(y))
        return out
    return [x]


def match_to_idents(names, v):
    if names[0] == "tuple":
        if v[0] == "tuple":
            if len(names[1]) != len(v[1]):
                raise FormuraCompileError("tuple length mismatch.")
            out = []
            for a, b in zip(names[1], v[1]):
                out.extend(match_to_idents(a, b))
            return out
        raise FormuraCompileError("the LHS expects a tuple, but RHS is not a tuple.")
    if names[0] == "ident":
        return [(names[1], v)]
    raise FormuraCompileError("no match (matchToIdents)")


def match_to_lhs(l, v):
    return match_to_idents(names_of_lhs(l), v)


def index_names_of_lhs(l, dim):
    if l[0] == "grid":
        return [n if n else None for (n, _k) in l[1]]
    return [None] * dim


def lexical_scope_holder(l):
    return {x[1]: HOLDER for x in tuple_contents(names_of_lhs(l))}


def value_type(v):
    """``typeOfVal`` / ``typeExprOf`` (``Translate.hs:157-162``)."""
    k = v[0]
    if k == "imm":
        return elem("Rational")
    if k == "node":
        return v[2]
    if k == "fun":
        return ("fun",)
    if k == "tuple":
        return ("tuple", [value_type(x) for x in v[1]])
    raise FormuraCompileError("no match (typeOfVal)")


class Translator:
    """One compiler run (``runCompilerRight``) producing one OM graph."""

    def __init__(self, prog: Program, env: GlobalEnv):
        self.prog = prog
        self.genv = env
        self.g = Graph()

    # -- helpers -------------------------------------------------------
    def insert(self, inst, typ):
        return self.g.insert(inst, typ)

    def cast_val(self, t1, v):
        t0 = value_type(v)
        if t1 == t0:
            return v
        if t1[0] == "elem" and t0[0] == "elem":
            return v
        if t1[0] == "gridtype" and t1[2][0] == "elem" and t0[0] == "elem" and v[0] == "node":
            return ("node", v[1], ("gridtype", t1[1], t1[2]))
        if t1[0] == "gridtype" and t0[0] == "gridtype" and tuple(t1[1]) == tuple(t0[1]):
            return v
        raise FormuraCompileError(f"cannot convert type {t0} to {t1}")

    # -- evaluation ----------------------------------------------------
    def gen(self, e, env):
        k = e[0]
        if k == "imm":
            return self.insert(("imm", e[1]), elem("Rational"))
        if k == "ident":
            if e[1] not in env:
                raise FormuraCompileError(f"undefined variable: {e[1]}")
            v = env[e[1]]
            if v is HOLDER:
                raise FormuraCompileError(f"unbound lexical variable: {e[1]}")
            return v
        if k in ("node", "fun"):
            return e
        if k == "tuple":
            return ("tuple", [self.gen(x, env) for x in e[1]])
        if k == "grid":
            return self.go_grid(e[1], self.gen(e[2], env))
        if k == "apply":
            f = self.gen(e[1], env)
            a = self.gen(e[2], env)
            return self.go_apply(f, a, env)
        if k == "lambda":
            scope = dict(env)
            scope.update(lexical_scope_holder(e[1]))
            return ("fun", e[1], self.resolve_lex(e[2], scope))
        if k == "let":
            return self.with_bindings(e[1], env, lambda env2: self.gen(e[2], env2))
        if k == "uniop":
            return self.go_uniop(e[1], self.gen(e[2], env))
        if k == "binop":
            a = self.gen(e[2], env)
            b = self.gen(e[3], env)
            return self.go_binop(e[1], a, b)
        if k == "triop":
            a = self.gen(e[2], env)
            b = self.gen(e[3], env)
            c = self.gen(e[4], env)
            return self.gen_triop(e[1], a, b, c)
        raise FormuraCompileError(f"cannot evaluate {k}")

    def resolve_lex(self, e, scope):
        k = e[0]
        if k == "ident":
            if e[1] not in scope:
                raise FormuraCompileError(
                    f"undefined variable: {e[1]}\nwhen resolving lexical binding.")
            v = scope[e[1]]
            return e if v is HOLDER else v
        if k == "lambda" or k == "fun":
            s2 = dict(scope)
            s2.update(lexical_scope_holder(e[1]))
            return ("fun", e[1], self.resolve_lex(e[2], s2))
        if k == "let":
            s2 = dict(scope)
            for st in e[1]:
                if st[0] == "subst":
                    s2.update(lexical_scope_holder(st[1]))
            return ("let", e[1], self.resolve_lex(e[2], s2))
        if k in ("imm", "node"):
            return e
        if k == "tuple":
            return ("tuple", [self.resolve_lex(x, scope) for x in e[1]])
        if k == "grid":
            return ("grid", e[1], self.resolve_lex(e[2], scope))
        if k == "apply":
            return ("apply", self.resolve_lex(e[1], scope), self.resolve_lex(e[2], scope))
        if k == "uniop":
            return ("uniop", e[1], self.resolve_lex(e[2], scope))
        if k == "binop":
            return ("binop", e[1], self.resolve_lex(e[2], scope), self.resolve_lex(e[3], scope))
        if k == "triop":
            return ("triop", e[1], self.resolve_lex(e[2], scope),
                    self.resolve_lex(e[3], scope), self.resolve_lex(e[4], scope))
        raise FormuraCompileError(f"cannot resolve {k}")

    def eval_to_imm(self, v):
        if v[0] == "imm":
            return v[1]
        if v[0] == "node":
            inst = self.g[v[1]].inst
            if inst[0] == "imm":
                return inst[1]
            raise FormuraCompileError("tuple applied to a computed (non-literal) index")
        return None

    def go_apply(self, f, a, env):
        if f[0] == "tuple":
            r = self.eval_to_imm(a)
            if r is None:
                raise FormuraCompileError("tuple applied to non-constant integer")
            if r.denominator != 1:
                raise FormuraCompileError("non-integer indexing in tuple access")
            n = int(r)
            if n < 0 or n >= len(f[1]):
                raise FormuraCompileError("tuple access out of bounds")
            return f[1][n]
        if f[0] == "fun":
            binds = dict(match_to_lhs(f[1], a))
            env2 = dict(env)
            env2.update(binds)
            return self.gen(f[2], env2)
        raise FormuraCompileError("unexpected combination of application")

    def go_uniop(self, op, v):
        if v[0] == "node":
            return self.insert(("uniop", op, v[1]), v[2])
        if v[0] == "fun":
            return ("fun", ("ident", "x"), ("uniop", op, ("apply", v, ("ident", "x"))))
        if v[0] == "tuple":
            return ("tuple", [self.go_uniop(op, x) for x in v[1]])
        raise FormuraCompileError("unexpected path in unary operator")

    def go_binop(self, op, a, b):
        if op == ".":
            return ("fun", ("ident", "x"), ("apply", a, ("apply", b, ("ident", "x"))))
        if a[0] == "node" and b[0] == "node":
            ct = meet(a[2], b[2])
            if ct == TOP:
                raise FormuraCompileError(
                    f"there is no common type that can accomodate both hand side: {a[2]} {op} {b[2]}")
            a2 = self.cast_val(ct, a)
            b2 = self.cast_val(ct, b)
            t = map_elem_type(lambda _: "bool", ct) if op in COMPARISONS else ct
            return self.insert(("binop", op, a2[1], b2[1]), t)
        x = ("ident", "x")
        if a[0] == "fun" and b[0] == "fun":
            return ("fun", x, ("binop", op, ("apply", a, x), ("apply", b, x)))
        if a[0] == "fun" and b[0] == "node":
            return ("fun", x, ("binop", op, ("apply", a, x), b))
        if a[0] == "node" and b[0] == "fun":
            return ("fun", x, ("binop", op, a, ("apply", b, x)))
        if a[0] == "tuple" and b[0] == "tuple":
            if len(a[1]) != len(b[1]):
                raise FormuraCompileError("tuple length mismatch.")
            return ("tuple", [self.go_binop(op, p, q) for p, q in zip(a[1], b[1])])
        if a[0] == "node" and b[0] == "tuple":
            return ("tuple", [self.go_binop(op, a, q) for q in b[1]])
        if a[0] == "tuple" and b[0] == "node":
            return ("tuple", [self.go_binop(op, p, b) for p in a[1]])
        raise FormuraCompileError(f"unexpected path in binary operator: {op}")

    def gen_triop(self, op, a, b, c):
        """Ternary operator over tuple trees with leaf broadcast (``TExpr.hs:22-31``)."""
        def go(x, y, z):
            trees = [t for t in (x, y, z) if t[0] == "tuple"]
            if not trees:
                return self.go_triop(op, x, y, z)
            n = len(trees[0][1])
            if any(len(t[1]) != n for t in trees):
                raise FormuraCompileError("Tuple length mismatch")
            pick = lambda t, i: t[1][i] if t[0] == "tuple" else t
            return ("tuple", [go(pick(x, i), pick(y, i), pick(z, i)) for i in range(n)])
        return go(a, b, c)

    def go_triop(self, op, a, b, c):
        if op == "ite" and a[0] == "node" and b[0] == "node" and c[0] == "node":
            if not is_boolish(a[2]):
                raise FormuraCompileError("the first argument of if-expr must be of type bool")
            bct = meet(b[2], c[2])
            if meet(a[2], bct) == TOP:
                raise FormuraCompileError(f"Type mismatch in if-then-else expr: {a[2]} {b[2]} {c[2]}")
            return self.insert(("triop", op, a[1], b[1], c[1]), bct)
        raise FormuraCompileError(f"unexpected path in trinary operator {op}")

    def go_grid(self, npks, v):
        if v[0] == "node":
            t = v[2]
            if t[0] == "elem":
                return v
            if t[0] == "gridtype":
                offs0 = list(t[1])
                patk = [k for (_n, k) in npks]
                n = max(len(offs0), len(patk))
                offs0 = (offs0 + [Fraction(0)] * n)[:n]
                patk = (patk + [Fraction(0)] * n)[:n]
                new_pos = [o - p for o, p in zip(offs0, patk)]
                int_off = [math.floor(x) for x in new_pos]
                new_off = [x - i for x, i in zip(new_pos, int_off)]
                typ1 = ("gridtype", new_off, t[2])
                if all(i == 0 for i in int_off):
                    return ("node", v[1], typ1)
                return self.insert(("shift", tuple(-i for i in int_off), v[1]), typ1)
            raise FormuraCompileError("no match")
        if v[0] == "tuple":
            return ("tuple", [self.go_grid(npks, x) for x in v[1]])
        raise FormuraCompileError(f"unexpected pattern in gen of grid: {v[0]}")

    # -- bindings ------------------------------------------------------
    def with_bindings(self, stmts, env, body):
        type_decls = [(st[3], st[2]) for st in stmts
                      if st[0] == "typedecl" and st[2] != TOP]
        substs = [(st[1], st[2]) for st in stmts if st[0] == "subst"]
        type_dict = {}
        for l, t in type_decls:
            for n, tt in match_to_lhs(l, t):
                type_dict[n] = tt
        mods: Dict[str, List[str]] = {}
        for st in stmts:
            if st[0] == "typedecl":
                for x in tuple_contents(names_of_lhs(st[3])):
                    mods.setdefault(x[1], []).extend(st[1])
        ext_funs = [l[1] for l, t in type_decls
                    if l[0] == "ident" and t == ("fun",) and "extern" in mods.get(l[1], [])]
        env = dict(env)
        for f in ext_funs:
            env[f] = ("fun", ("ident", "q"), ("uniop", "external-call/" + f, ("ident", "q")))
        for l0, rhs in substs:
            env_i = dict(env)
            for ax, name in enumerate(index_names_of_lhs(l0, self.genv.dimension)):
                if name is not None:
                    env_i[name] = self.insert(("loadindex", ax), elem("Rational"))
            v0 = self.gen(rhs, env_i)
            lvs = self.match_value_expr_to_lhs(l0, v0)
            for name0, v1 in lvs:
                v = self.cast_val(type_dict[name0], v1) if name0 in type_dict else v1
                self._annotate(v, name0, "manifest" in mods.get(name0, []))
                env[name0] = v
        return body(env)

    def _annotate(self, v, name0, manifest):
        if v[0] == "node":
            nd = self.g[v[1]]
            if nd.name is None:
                nd.name = name0
            if manifest:
                nd.manifest = True
                nd.name = name0
        elif v[0] == "tuple":
            for x in v[1]:
                self._annotate(x, name0, manifest)

    def match_value_expr_to_lhs(self, l, v):
        if l[0] == "grid":
            ivx = match_to_lhs(l[2], v)
            neg = [(n, -k) for (n, k) in l[1]]
            return [(i, self.go_grid(neg, x)) for i, x in ivx]
        return match_to_lhs(l, v)

    # -- global functions ----------------------------------------------
    def gen_global_function(self, global_stmts, input_type, output_pattern, fundef):
        """``genGlobalFunction`` (``Translate.hs:559-584``)."""
        if fundef[0] != "lambda":
            raise FormuraCompileError(
                "Identifier specified for function generation is not of function type.")
        l, r = fundef[1], fundef[2]

        def body(env):
            env2 = dict(env)
            for name1, t1 in match_to_lhs(l, input_type):
                if t1[0] not in ("elem", "gridtype"):
                    raise FormuraCompileError(
                        f"incompatible type `{t1}` encountered in conversion to node type.")
                env2[name1] = self.insert(("load", name1), t1)
            rv = self.gen(r, env2)
            for name1, rv1 in match_to_lhs(output_pattern, rv):
                if rv1[0] != "node":
                    raise FormuraCompileError(
                        "The return type of a global function must be a tuple of grids.")
                st = self.insert(("store", name1, rv1[1]), elem("void"))
                nd = self.g[st[1]]
                nd.manifest = True
                nd.name = name1 + "_next"
            return value_type(rv)

        return self.with_bindings(global_stmts, {}, body)


def calc_sleeve(g: Graph, dim: int) -> int:
    """``calcSleeve`` (``Translate.hs:613-623``).  ``max`` on ``Vec`` is the
    derived lexicographic order (``Vec.hs:63-64``)."""
    zero = None  # PureVec 0
    tbl: List[Optional[tuple]] = []

    def as_vec(v):
        return tuple([0] * dim) if v is None else v

    def vmax(a, b):
        if a is None and b is None:
            return None
        return max(as_vec(a), as_vec(b))

    for nd in g.nodes:
        inst = nd.inst
        k = inst[0]
        if k == "shift":
            prev = as_vec(tbl[inst[2]])
            tbl.append(tuple(d + p for d, p in zip(inst[1], prev)))
        elif k == "uniop":
            tbl.append(tbl[inst[2]])
        elif k == "binop":
            tbl.append(vmax(tbl[inst[2]], tbl[inst[3]]))
        elif k == "triop":
            tbl.append(vmax(vmax(tbl[inst[2]], tbl[inst[3]]), tbl[inst[4]]))
        else:
            tbl.append(zero)
    if not tbl:
        raise FormuraCompileError("empty graph")
    return max(max(as_vec(v)) for v in tbl)


@dataclass
class OMProgram:
    genv: GlobalEnv
    config: InternalConfig
    init_graph: Graph
    first_step_graph: Optional[Graph]
    filter_graph: Optional[Graph]
    step_graph: Graph
    state_signature: Dict[str, tuple]   # field name -> type, sorted by name
    step_lhs: tuple


def _lookup_toplevel(prog: Program, name: str, required=True):
    hits = [st[2] for st in prog.statements
            if st[0] == "subst" and st[1] == ("ident", name)]
    if not hits:
        if required:
            raise FormuraCompileError(f"Identifier `{name}` not found.")
        return None
    if len(hits) > 1:
        raise FormuraCompileError(f"Multiple declaration of identifier `{name}` found.")
    return hits[0]


def gen_om_program(prog: Program) -> OMProgram:
    """``genOMProgram`` (``Translate.hs:625-686``)."""
    genv = GlobalEnv(prog.dimension, prog.axes, prog.grid_struct_type_name,
                     prog.grid_struct_instance_name, comm_bases_for(prog.dimension))
    step_def = _lookup_toplevel(prog, "step")
    if step_def[0] != "lambda":
        raise FormuraCompileError("step is not a function")
    lhs_of_step = step_def[1]
    gb = prog.binding

    t_init = Translator(prog, genv)
    init_type = t_init.gen_global_function(gb, ("tuple", []), lhs_of_step,
                                           _lookup_toplevel(prog, "init"))

    def optional(name):
        d = _lookup_toplevel(prog, name, required=False)
        if d is None:
            return None
        t = Translator(prog, genv)
        ty = t.gen_global_function(gb, init_type, lhs_of_step, d)
        if ty != init_type:
            raise FormuraCompileError(
                f"the return type of {name} : {ty}\nmust match the return type of init : {init_type}")
        return t.g

    first_g = optional("first_step")
    filter_g = optional("filter")
    t_step = Translator(prog, genv)
    step_type = t_step.gen_global_function(gb, init_type, lhs_of_step, step_def)
    if step_type != init_type:
        raise FormuraCompileError(
            f"the return type of step : {step_type}\nmust match the return type of init : {init_type}")
    sig = dict(match_to_lhs(lhs_of_step, step_type))
    dim = prog.dimension
    s = calc_sleeve(t_step.g, dim)
    s0 = calc_sleeve(first_g, dim) if first_g is not None else None
    sf = calc_sleeve(filter_g, dim) if filter_g is not None else None
    cfg = convert_config(s, s0, sf, prog.nc)
    return OMProgram(genv, cfg, t_init.g, first_g, filter_g, t_step.g,
                     dict(sorted(sig.items())), lhs_of_step)
