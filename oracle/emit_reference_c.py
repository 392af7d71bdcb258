"""ORACLE (test infrastructure only): emits the C file pair that Formura's own
code generator writes for a program, in its no-MPI form (1 rank).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, as the checker.  The GPU product never calls it.

The Haskell generator cannot be built here (it needs GHC/Stack/z3), so this
module restates its emission rules so that the generated C can be compiled
with gcc and run on the host:

* ``scaffold`` and section order ``src/Formura/Generator/Templates.hs:23-51``;
  header/body layout ``src/Formura/Generator/Encode.hs:11-27``; statement and
  declaration printing ``Encode.hs:44-93``;
* grid struct (SoA, fields in name order) ``Templates.hs:53-73``;
  ``Formura_Navi`` ``Templates.hs:75-115`` (no-MPI branch ``:100-104``);
* local buffers for NoBlocking and TemporalBlocking ``Templates.hs:125-172``;
  comm buffers ``Templates.hs:174-186``;
* ``to_pos_*`` ``Templates.hs:221-225``; ``Formura_Init`` ``:227-250``;
  ``Formura_First_Step``/``Formura_Filter`` ``:252-270``; ``Formura_Setup``
  ``:272-280``; ``Formura_Step`` ``:282-293``; ``Formura_Forward`` ``:295-334``;
  ``noBlocking`` ``:336-346``; ``updateWithTB`` ``:348-381``;
  ``Formura_Finalize`` ``:383-386``;
* the per-manifest-node loop nest ``mkKernel`` ``Templates.hs:426-487``;
* ``loop``/``copy``/``sendrecv``/``isendrecv``/``waitAndCopy`` (no-MPI:
  send buffer copied to receive buffer) ``src/Formura/Generator/Functions.hs:169-290``;
  ``mkIdent`` ``Functions.hs:195-209``; index formatting ``Functions.hs:211-245``.

Numbers are printed like Haskell's ``show :: Double -> String``.
"""
from __future__ import annotations

import math
import os
import sys
from decimal import Decimal
from fractions import Fraction
from typing import Dict, List, Optional, Sequence, Tuple

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from formura_gb300.generator.manifest import MMProgram, MMNode, calc_range  # noqa: E402


# A kernel whose manifest temporaries add up to more than this keeps them on
# the heap (see mk_kernel).
HEAP_TEMPORARY_BYTES = 512 << 20


# --------------------------------------------------------------------------
# printing helpers
# --------------------------------------------------------------------------
def hs_show_double(x: float) -> str:
    """Haskell ``show`` for ``Double`` (GHC ``showFloat``)."""
    if x != x:
        return "NaN"
    if math.isinf(x):
        return "Infinity" if x > 0 else "-Infinity"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    sign = "-" if x < 0 else ""
    t = Decimal(repr(abs(x))).normalize().as_tuple()
    digits = "".join(str(d) for d in t.digits)
    e = len(digits) + t.exponent        # x = 0.d1d2.. * 10^e
    if 0.1 <= abs(x) < 1e7:
        if e <= 0:
            return sign + "0." + "0" * (-e) + digits
        if e >= len(digits):
            return sign + digits + "0" * (e - len(digits)) + ".0"
        return sign + digits[:e] + "." + digits[e:]
    mant = digits[0] + "." + (digits[1:] if len(digits) > 1 else "0")
    return sign + mant + "e" + str(e - 1)


def fmt_int(x: int) -> str:
    """``formatInt`` (``Functions.hs:211-212``)."""
    return "" if x == 0 else ("%+d" % x)


def idx_str(parts: Sequence[str]) -> str:
    return "".join("[" + p + "]" for p in parts)


# --------------------------------------------------------------------------
# variables
# --------------------------------------------------------------------------
class Var:
    """A C variable: ``kind`` is 'soa' (struct of arrays), 'soaptr' (pointer to
    such a struct) or 'aos' (array of structs)."""

    def __init__(self, name, kind, size, fields):
        self.name, self.kind, self.size, self.fields = name, kind, list(size), list(fields)

    def ident(self, f: str, idx: Sequence[str]) -> str:
        if self.kind == "soa":
            return f"{self.name}.{f}{idx_str(idx)}"
        if self.kind == "soaptr":
            return f"{self.name}->{f}{idx_str(idx)}"
        return f"{self.name}{idx_str(idx)}.{f}"

    def ref(self) -> str:
        return self.name if self.kind in ("aos", "soaptr") else "&" + self.name


class Emitter:
    def __init__(self, mm: MMProgram, header_name: str):
        self.mm = mm
        self.om = mm.om
        self.cfg = mm.om.config
        self.dim = mm.om.genv.dimension
        self.axes = mm.om.genv.axes
        self.fields = mm.fields
        self.N = list(self.cfg.grid_per_node)
        self.header_name = header_name
        self.omp = self.cfg.with_omp > 0
        if self.cfg.mpi_shape is not None and any(m != 1 for m in self.cfg.mpi_shape):
            raise ValueError("the oracle restates the 1-rank (no-MPI) form only")
        self.h_lines: List[str] = []
        self.local_types: List[str] = []
        self.local_vars: List[str] = []
        self.global_vars: List[str] = []
        self.local_funcs: List[str] = []
        self.global_funcs: List[str] = []
        self.global_protos: List[str] = []
        self.gs_type = mm.om.genv.grid_struct_type_name
        self.gs_name = mm.om.genv.grid_struct_instance_name
        self.gdata = Var(self.gs_name, "soa", self.N, self.fields)

    # -- structure -----------------------------------------------------
    def struct_def(self, name, size, scalar=False) -> str:
        body = "".join(f"double {f}{'' if scalar else idx_str(map(str, size))};\n"
                       for f in self.fields)
        return "typedef struct {\n" + body + "} " + name + ";"

    def sleeves(self) -> List[int]:
        """``getSleeves`` (``Functions.hs:51-60``)."""
        s = self.cfg.sleeve
        out = [s * self.cfg.blocking.nt] if self.cfg.blocking.temporal else [s]
        if self.cfg.sleeve0 is not None:
            out.append(self.cfg.sleeve0)
        if self.cfg.filter_sleeve is not None:
            out.append(self.cfg.filter_sleeve)
        return sorted(set(out))

    def loop(self, size, body_fn, names=None) -> List[str]:
        """``loop`` (``Functions.hs:169-174``) with the OpenMP pragma."""
        d = len(size)
        names = names or ["i%d" % (k + 1) for k in range(d)]
        out = []
        if self.omp:
            out.append("#pragma omp parallel for" + (f" collapse({d})" if d > 1 else ""))
        out.extend(self.loop_with([(n, 0, s) for n, s in zip(names, size)], body_fn(names)))
        return out

    @staticmethod
    def loop_with(idx, body: List[str]) -> List[str]:
        """``Loop`` printing (``Encode.hs:91``)."""
        text = "\n".join(body) + "\n"
        for n, lo, hi in reversed(idx):
            text = f"for(int {n} = {lo}; {n} < {hi}; {n} += 1) {{\n{text}}}\n"
        return [text.rstrip("\n")]

    def copy(self, src: Var, tgt: Var, src_off, tgt_off) -> List[str]:
        """``copy`` (``Functions.hs:250-256``)."""
        size = [min(a, b) for a, b in zip(src.size, tgt.size)]

        def body(names):
            so = [n + o for n, o in zip(names, src_off)]
            to = [n + o for n, o in zip(names, tgt_off)]
            return [f"{tgt.ident(f, to)} = {src.ident(f, so)};" for f in src.fields if f in tgt.fields]
        return self.loop(size, body)

    # -- kernels -------------------------------------------------------
    def mk_kernel(self, mmg: List[MMNode], sleeve: int, buff: Var, rslt: Var) -> List[str]:
        """``mkKernel`` (``Templates.hs:426-487``)."""
        out_size = rslt.size
        in_size = [s + 2 * sleeve for s in out_size]
        rng = calc_range(mmg)
        lines = []
        tmps = [n for n in mmg if not n.is_store]
        total = sum(math.prod(s - rng[n.omid].size() for s in in_size) * 8 for n in tmps)
        for n in tmps:
            if n.om_type[0] != "gridtype":
                raise ValueError("manifest scalar values are not supported by the reference emitter")
            ds = rng[n.omid].size()
            dims = [s - ds for s in in_size]
            if total <= HEAP_TEMPORARY_BYTES:
                lines.append(f"static double formura_mn{n.omid}{idx_str(map(str, dims))};")
            else:
                # Same array, same indexing, allocated once on first use: a
                # static array this large cannot be addressed from code in a
                # shared object (x86-64 and aarch64 reach +-2 / 4 GB of
                # PC-relative data), and aarch64 has no medium code model.
                v = f"formura_mn{n.omid}"
                lines.append(f"static double (*{v}){idx_str(map(str, dims[1:]))} = 0;")
                lines.append(f"if (!{v}) {{ {v} = calloc({dims[0]}, sizeof *{v}); if (!{v}) abort(); }}")
        for n in mmg:
            r = rng[n.omid]
            size = [s - r.size() for s in in_size]
            micro = list(n.micro)
            if not n.is_store:
                micro.append(("mnstore", len(micro) - 1))

            def body(names, micro=micro, r=r, n=n):
                stmts = []
                for mid, mn in enumerate(micro):
                    if isinstance(mn, tuple):       # inserted store to the temp array
                        stmts.append(f"formura_mn{n.omid}{idx_str(names)} = a{mn[1]};")
                        continue
                    inst = mn.inst
                    k = inst[0]
                    if k == "store":
                        stmts.append(f"{rslt.ident(inst[1], names)} = a{inst[2]};")
                        continue
                    ctype = {"Rational": "double", "double": "double", "float": "float",
                             "int": "int"}.get(mn.type, mn.type)
                    if k == "loadstatic":
                        ix = [nm + fmt_int(c + r.offset()) for nm, c in zip(names, inst[1])]
                        rhs = buff.ident(inst[2], ix)
                    elif k == "loadcursor":
                        ro = rng[inst[2]]
                        ix = [nm + fmt_int(c + r.offset() - ro.offset()) for nm, c in zip(names, inst[1])]
                        rhs = f"formura_mn{inst[2]}{idx_str(ix)}"
                    elif k == "imm":
                        rhs = hs_show_double(float(inst[1]))
                    elif k == "uniop":
                        op = inst[1]
                        if op.startswith("external-call/"):
                            rhs = f"{op[len('external-call/'):]}(a{inst[2]})"
                        else:
                            rhs = f"{op}a{inst[2]}"
                    elif k == "binop":
                        if inst[1] == "**":
                            rhs = f"pow(a{inst[2]},a{inst[3]})"
                        else:
                            rhs = f"a{inst[2]}{inst[1]}a{inst[3]}"
                    elif k == "triop":
                        rhs = f"a{inst[2]}?a{inst[3]}:a{inst[4]}"
                    elif k == "loadindex":
                        ax = inst[1]
                        rhs = f"{names[ax]}+n.offset_{self.axes[ax]}+block_offset_{ax + 1}"
                    else:
                        raise ValueError(f"Unimplemented for keyword: {k}")
                    stmts.append(f"{ctype} a{mid} = {rhs};")
                return stmts
            lines.extend(self.loop(size, body))
        return lines

    # -- sections ------------------------------------------------------
    def navi_fields(self) -> List[Tuple[str, str, str]]:
        """``mkNavi`` (``Templates.hs:81-115``), no-MPI branch."""
        cfg = self.cfg
        out = [("time_step", "int", "0")]
        out += [("lower_" + a, "int", "0") for a in self.axes]
        out += [("upper_" + a, "int", str(l)) for a, l in zip(self.axes, self.N)]
        out += [("space_interval_" + a, "double", hs_show_double(v))
                for a, v in zip(self.axes, cfg.space_interval)]
        out += [("my_rank", "int", "0")]
        out += [("offset_" + a, "int", "0") for a in self.axes]
        out += [("length_" + a, "double", hs_show_double(float(l)))
                for a, l in zip(self.axes, cfg.length_per_node)]
        out += [("total_grid_" + a, "int", str(l)) for a, l in zip(self.axes, self.N)]
        return out

    def func(self, rtype, name, args, body: List[str], is_global):
        text = f"{rtype} {name}(" + ",".join(f"{t} {n}" for t, n in args) + ") {\n" + \
               "".join(b + "\n" for b in body) + "}"
        (self.global_funcs if is_global else self.local_funcs).append(text)
        if is_global:
            self.global_protos.append(f"{rtype} {name}(" + ",".join(t for t, _ in args) + ");")

    def emit(self) -> Tuple[str, str]:
        cfg = self.cfg
        d = self.dim
        s = cfg.sleeve
        bt = cfg.blocking
        block_args = [("int", f"block_offset_{i + 1}") for i in range(d)]

        # header
        hdr = ["#pragma once", "#include <stdio.h>", "#include <stdlib.h>",
               "#include <stdbool.h>", "#include <math.h>"]
        if self.omp:
            hdr.append("#include <omp.h>")
        hdr.append(f"#define Ns {s}")
        hdr += [f"#define L{i + 1} {v}" for i, v in enumerate(self.N)]
        hdr.append(self.struct_def(self.gs_type, self.N))
        navi = self.navi_fields()
        hdr.append("typedef struct {\n" + "".join(f"{t} {n};\n" for n, t, _ in navi) + "} Formura_Navi;")
        self.global_vars.append(f"{self.gs_type} {self.gs_name};")

        # local buffers
        if not bt.temporal:
            ms = max(self.sleeves())
            self.local_types.append(self.struct_def("Formura_Buff", [n + 2 * ms for n in self.N]))
            self.local_vars.append("static Formura_Buff buff;")
            buff_v = Var("buff", "soa", [n + 2 * ms for n in self.N], self.fields)
            step_in, step_out = buff_v, self.gdata
            first_in = filt_in = buff_v
        else:
            gpb, bpn, nt = bt.grid_per_block, bt.block_per_node, bt.nt
            self.local_types.append(self.struct_def("Formura_Buff", [g + 2 * s for g in gpb]))
            self.local_types.append(self.struct_def("Formura_Rslt", gpb))
            self.local_vars.append("static Formura_Buff buff;")
            self.local_vars.append("static Formura_Rslt rslt;")
            ms = max(self.sleeves())
            tf_size = [n + 2 * ms for n in self.N]
            self.local_types.append(self.struct_def("Formura_Tmp_Floor", tf_size))
            self.local_vars.append("static Formura_Tmp_Floor tmp_floor;")
            walls = []
            for i in range(d):
                flag = [j == i for j in range(d)]
                bs = [m for m, b in zip(bpn, flag) if not b]
                gs = [2 * s if b else g + 2 * s for g, b in zip(gpb, flag)]
                wsize = bs + [nt] + gs
                self.local_types.append(self.struct_def(f"Formura_Tmp_Wall_{i + 1}", wsize))
                self.local_vars.append(f"static Formura_Tmp_Wall_{i + 1} tmp_wall_{i + 1};")
                walls.append((flag, gs, Var(f"tmp_wall_{i + 1}", "soa", wsize, self.fields)))
            buff_v = Var("buff", "soa", [g + 2 * s for g in gpb], self.fields)
            rslt_v = Var("rslt", "soa", gpb, self.fields)
            tmp_floor = Var("tmp_floor", "soa", tf_size, self.fields)
            step_in, step_out = buff_v, rslt_v
            first_in = filt_in = tmp_floor

        # comm buffers (no MPI: send buffer is copied to the receive buffer)
        self.local_types.append(self.struct_def("Formura_Comm_Buff", self.N, scalar=True))
        bases = self.om.genv.comm_bases
        comm = {}
        for sl in self.sleeves():
            for b in bases:
                r = "_".join("p1" if x == 1 else "0" for x in b)
                r2 = "_".join("m1" if x == 1 else "0" for x in b)
                size = [2 * sl if x == 1 else n for x, n in zip(b, self.N)]
                self.local_vars.append(f"static Formura_Comm_Buff send_buf{sl}_{r}{idx_str(map(str, size))};")
                self.local_vars.append(f"static Formura_Comm_Buff recv_buf{sl}_{r2}{idx_str(map(str, size))};")
                comm[(sl, tuple(b))] = (Var(f"send_buf{sl}_{r}", "aos", size, self.fields),
                                        Var(f"recv_buf{sl}_{r2}", "aos", size, self.fields))

        def isendrecv(src: Var, sl: int) -> List[str]:
            out = []
            for b in bases:
                sb, rb = comm[(sl, tuple(b))]
                out += self.copy(src, sb, [fmt_int(n - 2 * sl) if x == 1 else "" for x, n in zip(b, self.N)],
                                 [""] * d)
                out += self.copy(sb, rb, [""] * d, [""] * d)
            return out

        def wait_and_copy(tgt: Var, sl: int) -> List[str]:
            out = []
            for b in bases:
                _, rb = comm[(sl, tuple(b))]
                out += self.copy(rb, tgt, [""] * d, ["" if x == 1 else fmt_int(2 * sl) for x in b])
            return out

        def no_blocking(buff: Var, rslt: Var, sl: int, kernel: str) -> List[str]:
            out = isendrecv(self.gdata, sl)
            out += wait_and_copy(buff, sl)
            out += self.copy(self.gdata, buff, [""] * d, [fmt_int(2 * sl)] * d)
            out.append(f"{kernel}({buff.ref()},{rslt.ref()},*n" + ",0" * d + ");")
            for a in self.axes:
                out.append(f"n->offset_{a} = (n->offset_{a} - {sl} + n->total_grid_{a})%n->total_grid_{a};")
            return out

        # utility functions
        for a in self.axes:
            self.func("double", f"to_pos_{a}", [("int", "i"), ("Formura_Navi", "n")],
                      [f"return n.space_interval_{a}*((i+n.offset_{a})%n.total_grid_{a});"], True)

        # Formura_Setup
        self.func("void", "Formura_Setup", [("Formura_Navi", "n")] + block_args,
                  self.mk_kernel(self.mm.init, 0,
                                 Var(self.gs_name, "soa", self.N, self.fields),
                                 Var(self.gs_name, "soa", self.N, self.fields)), False)

        def kernel_fn(name, graph, sl, bin_: Var, bout: Var):
            bp = Var("buff", "soaptr", bin_.size, self.fields)
            rp = Var("rslt", "soaptr", bout.size, self.fields)
            btype = {"buff": "Formura_Buff", "rslt": "Formura_Rslt", "tmp_floor": "Formura_Tmp_Floor"}.get(
                bin_.name, self.gs_type)
            rtype = {"buff": "Formura_Buff", "rslt": "Formura_Rslt"}.get(bout.name, self.gs_type)
            self.func("void", name, [(btype + " *", "buff"), (rtype + " *", "rslt"), ("Formura_Navi", "n")]
                      + block_args, self.mk_kernel(graph, sl, bp, rp), False)

        if self.mm.first_step is not None:
            kernel_fn("Formura_First_Step_Kernel", self.mm.first_step, cfg.sleeve0, first_in, self.gdata)
            self.func("void", "Formura_First_Step", [("Formura_Navi *", "n")],
                      no_blocking(first_in, self.gdata, cfg.sleeve0, "Formura_First_Step_Kernel"), False)
        if self.mm.filter is not None:
            kernel_fn("Formura_Filter_Kernel", self.mm.filter, cfg.filter_sleeve, filt_in, self.gdata)
            self.func("void", "Formura_Filter", [("Formura_Navi *", "n")],
                      no_blocking(filt_in, self.gdata, cfg.filter_sleeve, "Formura_Filter_Kernel"), False)

        # Formura_Init
        init_body = [f"n->{f} = {v};" for f, _, v in navi]
        init_body.append("Formura_Setup(*n" + ",0" * d + ");")
        if self.mm.first_step is not None:
            init_body.append("Formura_First_Step(n);")
        self.func("void", "Formura_Init", [("int *", "argc"), ("char ***", "argv"), ("Formura_Navi *", "n")],
                  init_body, True)

        # Formura_Step
        kernel_fn("Formura_Step", self.mm.step, s, step_in, step_out)

        # Formura_Forward
        fwd: List[str] = []
        filt = []
        if self.mm.filter is not None:
            filt = [f"if (n->time_step % {cfg.filter_interval} == 0) {{", "Formura_Filter(n);", "}"]
        if not bt.temporal:
            fwd += no_blocking(step_in, step_out, s, "Formura_Step")
            fwd += filt
            fwd.append("n->time_step += 1;")
        else:
            gpb, bpn, nt = bt.grid_per_block, bt.block_per_node, bt.nt
            fwd += self.copy(self.gdata, tmp_floor, [""] * d, [fmt_int(2 * s * nt)] * d)
            fwd += isendrecv(self.gdata, s * nt)
            b0 = [(0, m - 1 - (2 * s * nt) // g) for g, m in zip(gpb, bpn)]
            bs = [[((m - 1 - (2 * s * nt) // g) if i == j else 0,
                    (m - 1 - (2 * s * nt) // g) if i > j else m)
                   for g, m, i in zip(gpb, bpn, range(1, d + 1))] for j in range(1, d + 1)]

            def update(boundary):
                jn = [f"j{i + 1}" for i in range(d)]
                floor_off = [f"+{g * (m - 1)}-{g}*{j}" for g, m, j in zip(gpb, bpn, jn)]
                body: List[str] = []
                body += self.copy(tmp_floor, rslt_v, floor_off, [""] * d)
                sub: List[str] = []
                sub += self.copy(rslt_v, buff_v, [""] * d, [""] * d)
                for flag, gs, wall in walls:
                    idx0 = [j for j, b in zip(jn, flag) if not b] + ["it"]

                    def wbody(names, flag=flag, wall=wall, idx0=idx0):
                        bix = [nm + fmt_int(g if b else 0) for nm, g, b in zip(names, gpb, flag)]
                        return [f"{buff_v.ident(f, bix)} = {wall.ident(f, idx0 + list(names))};"
                                for f in self.fields]
                    sub += self.loop(gs, wbody)
                sub.append(f"Formura_Step({buff_v.ref()},{rslt_v.ref()},*n," + ",".join(floor_off) + ");")
                for flag, gs, wall in walls:
                    idx0 = [j for j, b in zip(jn, flag) if not b] + ["it"]

                    def wbody2(names, wall=wall, idx0=idx0):
                        return [f"{wall.ident(f, idx0 + list(names))} = {buff_v.ident(f, names)};"
                                for f in self.fields]
                    sub += self.loop(gs, wbody2)
                body += self.loop_with([("it", 0, nt)], sub)
                body += self.copy(rslt_v, tmp_floor, [""] * d, floor_off)
                return self.loop_with([(j, lo, hi) for j, (lo, hi) in zip(jn, boundary)], body)

            fwd += update(b0)
            fwd += wait_and_copy(tmp_floor, s * nt)
            for b in bs:
                fwd += update(b)
            fwd += self.copy(tmp_floor, self.gdata, [""] * d, [""] * d)
            for a in self.axes:
                fwd.append(f"n->offset_{a} = (n->offset_{a} - {s * nt} + n->total_grid_{a})%n->total_grid_{a};")
            fwd += filt
            fwd.append(f"n->time_step += {nt};")
        self.func("void", "Formura_Forward", [("Formura_Navi *", "n")], fwd, True)
        self.func("void", "Formura_Finalize", [], [], True)

        h = hdr + [f"extern {self.gs_type} {self.gs_name};"] + self.global_protos
        c = [f'#include "{self.header_name}"'] + self.local_types + self.local_vars + \
            self.global_vars + self.local_funcs + self.global_funcs
        return "\n".join(h) + "\n", "\n".join(c) + "\n"


def emit_reference_c(mm: MMProgram, header_name: str) -> Tuple[str, str]:
    """Return (header text, C text) of the reference generator's output."""
    return Emitter(mm, header_name).emit()
