"""Command line of the generator, mirroring the reference's ``formura``
executable (``app/formura.hs:26-94``, options ``CommandLineOption.hs:33-51``):

    python -m formura_gb300.generator.cli [-o X.c] [--nc X.yaml] [-v] X.fmr

writes ``X.c`` and ``X.h`` for the GB300 backend (the header is the
reference's header; the body calls libformura_gb300) and prints the files
it generated, like ``Generator.hs:36``.  The numerical config defaults to
the ``.fmr`` file's name with ``.yaml`` (the reference's default name is
``X.yaml`` too).  ``--program`` names the library program whose kernels the
body uses (default: the file's base name).  ``-v`` prints the manifest
structure: sleeve, stages, manifest nodes.

``--lib`` also builds ``lib<program>_gb300.so`` beside the C file: the
GB300 library with this program's kernels (``build_program_library``), for
programs that are not shipped with the package.  The program name is then
the file's base name made into a C identifier (``3d_hllc`` becomes
``p3d_hllc``).  A driver links it like the reference's generated C::

    gcc main.c X.c -L<dir> -l<program>_gb300 -Wl,-rpath,<dir> -lm
"""
from __future__ import annotations

import argparse
import os
import sys
from typing import List, Optional

from .config import ConfigError, read_config
from .cuda import emit_cuda
from .dropin import emit_dropin
from .manifest import calc_range, gen_mm_program
from .syntax import FormuraSyntaxError, parse_program
from .translate import FormuraCompileError, gen_om_program


def main(argv: Optional[List[str]] = None) -> int:
    ap = argparse.ArgumentParser(prog="formura-gb300", description="Formura code generator, GB300 backend")
    ap.add_argument("source", help="the .fmr program")
    ap.add_argument("-o", "--output", help="output C file (default: <source>.c)")
    ap.add_argument("--nc", help="numerical config YAML (default: <source>.yaml)")
    ap.add_argument("--program", help="library program providing the kernels (default: source base name)")
    ap.add_argument("--lib", action="store_true",
                    help="also build lib<program>_gb300.so with this program's kernels")
    ap.add_argument("-v", "--verbose", action="store_true")
    args = ap.parse_args(argv)

    base = os.path.splitext(args.source)[0]
    cpath = args.output or base + ".c"
    hpath = os.path.splitext(cpath)[0] + ".h"
    ncpath = args.nc or base + ".yaml"
    from .. import build as B
    program = args.program or (B.program_identifier(os.path.basename(base)) if args.lib
                               else os.path.basename(base))
    try:
        nc = read_config(ncpath)
        with open(args.source) as f:
            fmr_src = f.read()
        with open(ncpath) as f:
            yaml_text = f.read()
        prog = parse_program(fmr_src, nc)
        om = gen_om_program(prog)
        mm = gen_mm_program(om)
        if args.lib:
            rp = B.runtime_params(yaml_text)
        else:
            rp = B.library_runtime_params(program) if os.path.exists(
                os.path.join(B.PROGRAMS, program + ".yaml")) else []
        if args.verbose:
            kp = emit_cuda(mm, program, rp)
            rng = calc_range(mm.step)
            print(f"fields: {mm.fields}")
            print(f"sleeve: {om.config.sleeve}  roll per step: {kp.shift}")
            print(f"manifest nodes: {len(mm.step)}")
            for n in mm.step:
                r = rng[n.omid]
                print(f"  #{n.omid} {n.name or '(anonymous)'}  range ({r.lower},{r.upper})  "
                      f"{len(n.micro)} micro ops")
            print(f"stages: {[len(s.nodes) for s in kp.stages]}  HBM intermediates: {len(kp.mids)}")
        h, c = emit_dropin(mm, program, os.path.basename(hpath), None, rp)
    except (ConfigError, FormuraSyntaxError, FormuraCompileError, OSError) as e:
        print(f"formura-gb300: {e}", file=sys.stderr)
        return 1
    with open(hpath, "w") as f:
        f.write(h)
    with open(cpath, "w") as f:
        f.write(c)
    print("Generate:")
    print("  " + cpath)
    print("  " + hpath)
    if args.lib:
        out = os.path.join(os.path.dirname(os.path.abspath(cpath)), f"lib{program}_gb300.so")
        try:
            B.build_program_library(program, fmr_src, yaml_text, out)
        except (RuntimeError, ValueError, FormuraCompileError) as e:
            print(f"formura-gb300: {e}", file=sys.stderr)
            return 1
        print("  " + out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
