"""Manifest Machine (MM): each manifest OM node becomes one instruction, a
micro-graph evaluated at one grid point.  Delayed (non-manifest) nodes are
inlined at every cursor they are read at; ``Shift`` becomes a cursor move;
reads of manifest nodes and of the state become cursored loads.

Restates ``src/Formura/OrthotopeMachine/Manifestation.hs``:
``insertMM``/``mapNodeID`` ``:85-113``, ``rhsCodeAt``/``rhsDelayedCodeAt``
``:116-152``, ``manifestG`` ``:170-207`` (``boundaryAnalysis`` ``:226-251``
is a no-op whose result is never used, so it is not restated).  Also
restates the per-node cursor range ``calcRange`` of
``src/Formura/Generator/Templates.hs:388-424``.

Micro instructions: ``('imm', r)``, ``('uniop', op, a)``, ``('binop', op, a, b)``,
``('triop', op, a, b, c)``, ``('loadcursor', cursor, omid)``,
``('loadstatic', cursor, field)``, ``('loadindex', axis)``, ``('store', name, a)``.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Tuple

from .translate import FormuraCompileError, Graph, OMProgram, elem_of


@dataclass
class MicroNode:
    inst: tuple
    type: str          # element type name
    key: tuple = ()    # (cursor, OM node id) this micro node evaluates


@dataclass
class MMNode:
    """One manifest node: its micro-graph (ordered by micro id) and OM type."""
    omid: int
    micro: List[MicroNode]
    om_type: tuple
    name: str

    @property
    def is_store(self) -> bool:
        return self.om_type == ("elem", "void")


class _Manifester:
    def __init__(self, g: Graph, manifest_set, dim: int):
        self.g = g
        self.is_m = manifest_set
        self.dim = dim

    def run(self, nid: int) -> List[MicroNode]:
        self.map: Dict[Tuple[tuple, int], int] = {}
        self.mm: Dict[int, MicroNode] = {}
        self.delayed(tuple([0] * self.dim), nid)
        return [self.mm[i] for i in range(len(self.mm))]

    def insert(self, c, i, inst):
        key = (c, i)
        j = self.map.get(key)
        if j is None:
            j = len(self.map)
            self.map[key] = j
        self.mm[j] = MicroNode(inst, elem_of(self.g[i].type), key)
        return j

    def code_at(self, c, nid):
        if nid in self.is_m:
            return self.insert(c, nid, ("loadcursor", c, nid))
        return self.delayed(c, nid)

    def delayed(self, c, nid):
        key = (c, nid)
        if key in self.map and self.map[key] in self.mm:
            return self.map[key]
        inst = self.g[nid].inst
        k = inst[0]
        if k == "imm":
            return self.insert(c, nid, inst)
        if k == "uniop":
            return self.insert(c, nid, ("uniop", inst[1], self.code_at(c, inst[2])))
        if k == "binop":
            a = self.code_at(c, inst[2])
            b = self.code_at(c, inst[3])
            return self.insert(c, nid, ("binop", inst[1], a, b))
        if k == "triop":
            a = self.code_at(c, inst[2])
            b = self.code_at(c, inst[3])
            cc = self.code_at(c, inst[4])
            return self.insert(c, nid, ("triop", inst[1], a, b, cc))
        if k == "shift":
            c2 = tuple(x + d for x, d in zip(c, inst[1]))
            return self.code_at(c2, inst[2])
        if k == "load":
            return self.insert(c, nid, ("loadstatic", c, inst[1]))
        if k == "loadindex":
            return self.insert(c, nid, inst)
        if k == "store":
            a = self.code_at(c, inst[2])
            return self.insert(c, nid, ("store", inst[1], a))
        raise FormuraCompileError(f"manifestation path unimplemented for keyword: {k}")


def manifest_graph(g: Graph, dim: int) -> List[MMNode]:
    """``manifestG``: one MM instruction per manifest node, ascending OM id."""
    mset = {i for i, nd in enumerate(g.nodes) if nd.manifest}
    m = _Manifester(g, mset, dim)
    out = []
    for nid in sorted(mset):
        micro = m.run(nid)
        nd = g[nid]
        out.append(MMNode(nid, micro, nd.type, nd.name or ""))
    return out


@dataclass
class Range:
    lower: int
    upper: int

    def size(self) -> int:
        return abs(self.lower) + abs(self.upper)

    def offset(self) -> int:
        return abs(self.lower)


def calc_range(mmg: List[MMNode]) -> Dict[int, Range]:
    """``calcRange`` (``Templates.hs:388-424``): per manifest node the union of
    its cursor ranges, isotropic over the axes (min/max over all components)."""
    tbl: Dict[int, Range] = {}
    for node in mmg:
        lo, hi = 0, 0
        for mn in node.micro:
            inst = mn.inst
            if inst[0] == "loadstatic":
                c = inst[1]
                lo, hi = min(lo, min(c)), max(hi, max(c))
            elif inst[0] == "loadcursor":
                c = inst[1]
                r = tbl[inst[2]]
                lo = min(lo, min(c) + r.lower)
                hi = max(hi, max(c) + r.upper)
        tbl[node.omid] = Range(lo, hi)
    return tbl


@dataclass
class MMProgram:
    om: OMProgram
    init: List[MMNode]
    first_step: List[MMNode] | None
    filter: List[MMNode] | None
    step: List[MMNode]

    @property
    def fields(self) -> List[str]:
        return list(self.om.state_signature.keys())


def gen_mm_program(om: OMProgram) -> MMProgram:
    dim = om.genv.dimension
    return MMProgram(
        om,
        manifest_graph(om.init_graph, dim),
        manifest_graph(om.first_step_graph, dim) if om.first_step_graph is not None else None,
        manifest_graph(om.filter_graph, dim) if om.filter_graph is not None else None,
        manifest_graph(om.step_graph, dim),
    )


def compile_program(src: str, nc) -> MMProgram:
    """Parse, translate and manifest a Formura program."""
    from .syntax import parse_program
    from .translate import gen_om_program
    return gen_mm_program(gen_om_program(parse_program(src, nc)))
