"""Emission of the drop-in C pair (``X.h``/``X.c``) for the GB300 backend.

The header is the reference generator's header, symbol for symbol and byte
layout for layout (``src/Formura/Generator/Templates.hs:23-115``,
``Encode.hs:11-20``), so existing driver programs (``main.c``) compile and
link unchanged.  The body keeps ``formura_data`` and ``Formura_Navi`` on the
host; ``Formura_Init`` evaluates the init function on the host like
``Formura_Setup`` (``Templates.hs:272-280``, loop nest rules of
``mkKernel`` ``Templates.hs:426-487``) and opens the device grid;
``Formura_Forward`` uploads ``formura_data``, advances the time loop on the
GPU and downloads the result, then updates ``offset_*`` and ``time_step``
like the reference (``Templates.hs:300-334, 346``).

Backend options come from ``gpu_*`` keys of the numerical config:
``gpu_precision`` (f64, f64fast, f32, f16), ``gpu_steps_per_forward``
(default: ``temporal_blocking_interval`` when temporal blocking is
configured, else 1, i.e. the reference's step count per call) and
``gpu_field_scales`` (FP16 storage), ``gpu_host_sync`` (``eager``: upload and
download formura_data on every call; ``lazy``: copy only when the driver
touches it, by page protection) and ``gpu_autotune`` (0 turns off the
choice of the temporal-blocking kernel at ``Formura_Init``; results do not
depend on it except with FP16 storage).
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

from .cuda import KernelProgram, c_double, emit_cuda, uniform_table
from .manifest import MMNode, MMProgram, calc_range
from .translate import FormuraCompileError

PRECISIONS = {"f64": 0, "f64fast": 1, "f32": 2, "f16": 3}


def _show(x: float) -> str:
    return repr(float(x))


def steps_per_forward(mm: MMProgram) -> int:
    cfg = mm.om.config
    v = cfg.gpu.get("gpu_steps_per_forward")
    if v is not None:
        n = int(v)
        if n < 1:
            raise FormuraCompileError("gpu_steps_per_forward must be positive")
        return n
    return cfg.blocking.nt if cfg.blocking.temporal else 1


def precision_of(mm: MMProgram) -> int:
    v = str(mm.om.config.gpu.get("gpu_precision", "f64"))
    if v not in PRECISIONS:
        raise FormuraCompileError(f"gpu_precision must be one of {sorted(PRECISIONS)}")
    return PRECISIONS[v]


def _setup_nest(mm: MMProgram) -> List[str]:
    """Host loop nest of the init function, evaluated into formura_data."""
    axes = mm.om.genv.axes
    N = list(mm.om.config.grid_per_node)
    gs = mm.om.genv.grid_struct_instance_name
    rng = calc_range(mm.init)
    lines = []
    for node in mm.init:
        if not node.is_store:
            raise FormuraCompileError("manifest values inside init are not supported by the GPU backend")
        r = rng[node.omid]
        if r.size() != 0:
            raise FormuraCompileError("init must not read shifted values")
        names = [f"i{k + 1}" for k in range(len(N))]
        body = []
        for mid, mn in enumerate(node.micro):
            inst = mn.inst
            k = inst[0]
            if k == "store":
                body.append(f"{gs}.{inst[1]}" + "".join(f"[{n}]" for n in names) + f" = a{inst[2]};")
                continue
            ctype = {"Rational": "double", "double": "double", "float": "float", "int": "int"}.get(mn.type, mn.type)
            if k == "imm":
                rhs = c_double(float(inst[1]))
            elif k == "loadindex":
                ax = inst[1]
                rhs = f"{names[ax]}+n.offset_{axes[ax]}"
            elif k == "uniop":
                op = inst[1]
                rhs = (f"{op[len('external-call/'):]}(a{inst[2]})" if op.startswith("external-call/")
                       else f"{op}a{inst[2]}")
            elif k == "binop":
                rhs = (f"pow(a{inst[2]},a{inst[3]})" if inst[1] == "**"
                       else f"a{inst[2]}{inst[1]}a{inst[3]}")
            elif k == "triop":
                rhs = f"a{inst[2]}?a{inst[3]}:a{inst[4]}"
            else:
                raise FormuraCompileError(f"init cannot use {k}")
            body.append(f"{ctype} a{mid} = {rhs};")
        text = "\n".join(body) + "\n"
        for nm, n in reversed(list(zip(names, N))):
            text = f"for(int {nm} = 0; {nm} < {n}; {nm} += 1) {{\n{text}}}\n"
        lines.append(text.rstrip("\n"))
    return lines


def emit_dropin(mm: MMProgram, program: str, header_name: str,
                params: Optional[Dict[str, float]] = None,
                runtime_params: Optional[List[str]] = None) -> Tuple[str, str]:
    """Return (X.h, X.c) for the GB300 backend; ``program`` is the name of
    the program compiled into libformura_gb300."""
    cfg = mm.om.config
    if cfg.mpi_shape is not None and any(m != 1 for m in cfg.mpi_shape):
        raise FormuraCompileError("the GPU backend runs one rank per process (mpi_shape must be all 1)")
    kp = emit_cuda(mm, program, runtime_params or [])
    U = uniform_table(mm, kp, params)
    subs = {}
    for graph in ("first_step", "filter"):
        if getattr(mm, graph) is not None:
            kps = emit_cuda(mm, program, runtime_params or [], graph)
            subs[graph] = uniform_table(mm, kps, params)
    axes = mm.om.genv.axes
    N = list(cfg.grid_per_node)
    dim = len(N)
    fields = mm.fields
    gst, gsn = mm.om.genv.grid_struct_type_name, mm.om.genv.grid_struct_instance_name
    s = cfg.sleeve
    nt = steps_per_forward(mm)
    prec = precision_of(mm)

    def show_double(x: float) -> str:
        return repr(float(x))

    navi = [("time_step", "int", "0")]
    navi += [("lower_" + a, "int", "0") for a in axes]
    navi += [("upper_" + a, "int", str(n)) for a, n in zip(axes, N)]
    navi += [("space_interval_" + a, "double", show_double(v)) for a, v in zip(axes, cfg.space_interval)]
    navi += [("my_rank", "int", "0")]
    navi += [("offset_" + a, "int", "0") for a in axes]
    navi += [("length_" + a, "double", show_double(float(l))) for a, l in zip(axes, cfg.length_per_node)]
    navi += [("total_grid_" + a, "int", str(n)) for a, n in zip(axes, N)]

    h = ["#pragma once", "#include <stdio.h>", "#include <stdlib.h>", "#include <stdbool.h>",
         "#include <math.h>"]
    if cfg.with_omp > 0:
        h.append("#include <omp.h>")
    h.append(f"#define Ns {s}")
    h += [f"#define L{i + 1} {v}" for i, v in enumerate(N)]
    h.append("typedef struct {\n" + "".join(f"double {f}" + "".join(f"[{n}]" for n in N) + ";\n"
                                            for f in fields) + f"}} {gst};")
    h.append("typedef struct {\n" + "".join(f"{t} {nm};\n" for nm, t, _ in navi) + "} Formura_Navi;")
    h.append(f"extern {gst} {gsn};")
    h += [f"double to_pos_{a}(int,Formura_Navi);" for a in axes]
    h += ["void Formura_Init(int *,char ***,Formura_Navi *);", "void Formura_Forward(Formura_Navi *);",
          "void Formura_Finalize();"]

    scales = cfg.gpu.get("gpu_field_scales")
    sync = str(cfg.gpu.get("gpu_host_sync", "eager"))
    if sync not in ("eager", "lazy"):
        raise FormuraCompileError("gpu_host_sync must be eager or lazy")
    lazy = sync == "lazy"
    if lazy:
        # formura_data in its own page-aligned, page-padded block (64 KiB
        # covers 4 KiB and 64 KiB pages), so that protecting it protects
        # nothing else
        storage = [f"#define FORMURA_GB300_PAGE 65536",
                   f"static union {{ {gst} s; char pad[(sizeof({gst}) + FORMURA_GB300_PAGE - 1)"
                   f" / FORMURA_GB300_PAGE * FORMURA_GB300_PAGE]; }} formura_gb300_storage"
                   f" __attribute__((aligned(FORMURA_GB300_PAGE)));",
                   f'extern {gst} {gsn} __attribute__((alias("formura_gb300_storage")));']
    else:
        storage = [f"{gst} {gsn};"]
    c = [f'#include "{header_name}"', '#include "formura_gb300.h"'] + storage + [
         "static fgb_grid* formura_gb300_grid = 0;",
         f"static const double formura_gb300_uniforms[{max(1, len(U))}] = {{"
         + ", ".join(c_double(x) for x in U) + ("" if U else "0.0") + "};",
         "static void formura_gb300_check(int rc, const char* what) {",
         "  if (rc != 0) {",
         '    fprintf(stderr, "formura_gb300: %s failed: %s\\n", what, fgb_last_error());',
         "    exit(1);",
         "  }",
         "}"]
    for a in axes:
        c.append(f"double to_pos_{a}(int i,Formura_Navi n) {{\n"
                 f"return n.space_interval_{a}*((i+n.offset_{a})%n.total_grid_{a});\n}}")
    c.append("static void Formura_Setup(Formura_Navi n) {")
    c += _setup_nest(mm)
    c.append("}")
    shape = ", ".join(str(n) for n in N)
    c.append("void Formura_Init(int *argc,char ***argv,Formura_Navi *n) {")
    c.append("(void)argc; (void)argv;")
    c += [f"n->{nm} = {v};" for nm, _, v in navi]
    c.append("Formura_Setup(*n);")
    c.append(f"static const int shape[{dim}] = {{{shape}}};")
    c.append(f'formura_gb300_check(fgb_open("{program}", shape, {dim}, {prec}, formura_gb300_uniforms, '
             f'{len(U)}, &formura_gb300_grid), "fgb_open");')
    if prec == 3:
        sc = scales if isinstance(scales, list) else [1.0] * len(fields)
        if len(sc) != len(fields):
            raise FormuraCompileError("gpu_field_scales needs one scale per field")
        c.append(f"static const float scales[{len(fields)}] = {{" + ", ".join(f"{float(x)!r}f" for x in sc) + "};")
        c.append(f'formura_gb300_check(fgb_set_scales(formura_gb300_grid, scales, {len(fields)}), "fgb_set_scales");')
    tune = cfg.gpu.get("gpu_autotune", 1)
    if int(tune):
        c.append(f'formura_gb300_check(fgb_autotune(formura_gb300_grid, {max(8, 2 * nt) if nt < 64 else 64}, 0), "fgb_autotune");')
    for graph, Ug in subs.items():
        c.append(f"static const double formura_gb300_{graph}_uniforms[{max(1, len(Ug))}] = {{"
                 + ", ".join(c_double(x) for x in Ug) + ("" if Ug else "0.0") + "};")
        c.append(f'formura_gb300_check(fgb_attach(formura_gb300_grid, "{graph}", formura_gb300_{graph}_uniforms, '
                 f'{len(Ug)}), "fgb_attach");')
    if "first_step" in subs:
        # Formura_First_Step (Templates.hs:250, 252-260): once, rolled by its sleeve
        c.append(f'formura_gb300_check(fgb_upload(formura_gb300_grid, (const double*)&{gsn}), "fgb_upload");')
        c.append('formura_gb300_check(fgb_apply(formura_gb300_grid, "first_step"), "fgb_apply");')
        c.append(f'formura_gb300_check(fgb_download(formura_gb300_grid, (double*)&{gsn}), "fgb_download");')
        for a in axes:
            c.append(f"n->offset_{a} = (n->offset_{a} - {cfg.sleeve0} + n->total_grid_{a})%n->total_grid_{a};")
    if lazy:
        c.append('formura_gb300_check(fgb_lazy_attach(formura_gb300_grid, &formura_gb300_storage, '
                 'sizeof(formura_gb300_storage)), "fgb_lazy_attach");')
    else:
        c.append(f"fgb_host_register(&{gsn}, sizeof({gsn}));")
    c.append("}")
    # one reference Formura_Forward call advances g steps (Templates.hs:300-334);
    # a call here advances nt = k*g steps and keeps the reference's per-call
    # offset, filter and time_step updates for each of the k sub-calls
    g = cfg.blocking.nt if cfg.blocking.temporal else 1
    if nt % g != 0:
        raise FormuraCompileError(f"gpu_steps_per_forward must be a multiple of {g}")
    k = nt // g

    def offsets(amount):
        return [f"n->offset_{a} = (n->offset_{a} - {amount} + n->total_grid_{a})%n->total_grid_{a};" for a in axes]

    c.append("void Formura_Forward(Formura_Navi *n) {")
    if lazy:
        fwd = lambda steps: f'formura_gb300_check(fgb_lazy_forward(formura_gb300_grid, {steps}), "fgb_lazy_forward");'
    else:
        c.append(f'formura_gb300_check(fgb_upload(formura_gb300_grid, (const double*)&{gsn}), "fgb_upload");')
        fwd = lambda steps: f'formura_gb300_check(fgb_forward(formura_gb300_grid, {steps}), "fgb_forward");'
    if "filter" in subs:
        c.append(f"for (int c = 0; c < {k}; ++c) {{")
        c.append(fwd(g))
        c += offsets(s * g)
        c.append(f"if (n->time_step % {cfg.filter_interval} == 0) {{")
        c.append('formura_gb300_check(fgb_apply(formura_gb300_grid, "filter"), "fgb_apply");')
        c += offsets(cfg.filter_sleeve)
        c.append("}")
        c.append(f"n->time_step += {g};")
        c.append("}")
    else:
        c.append(fwd(nt))
        c.append(f"for (int c = 0; c < {k}; ++c) {{")
        c += offsets(s * g)
        c.append(f"n->time_step += {g};")
        c.append("}")
    if not lazy:
        c.append(f'formura_gb300_check(fgb_download(formura_gb300_grid, (double*)&{gsn}), "fgb_download");')
    c.append("}")
    c.append("void Formura_Finalize() {")
    if lazy:
        c.append("if (formura_gb300_grid) { fgb_lazy_detach(formura_gb300_grid); fgb_close(formura_gb300_grid); "
                 "formura_gb300_grid = 0; }")
    else:
        c.append(f"if (formura_gb300_grid) {{ fgb_host_unregister(&{gsn}); fgb_close(formura_gb300_grid); "
                 f"formura_gb300_grid = 0; }}")
    c.append("}")
    return "\n".join(h) + "\n", "\n".join(c) + "\n"
