"""ORACLE (test infrastructure only): builds the reference generator's C output
for a program (see ``emit_reference_c.py``) into a shared object and drives it
through the generated C API, the way an example ``main.c`` does
(``examples/pearson2/main.c:39-56``): ``Formura_Init``, direct writes and
reads of ``formura_data`` (the user's init/output hook), ``Formura_Forward``.

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module.

Build recipe: ``gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared``.  Every
floating-point operation of the generated SSA chain is then rounded once, on
x86_64 and on aarch64 alike (``-ffp-contract=off`` stops FMA contraction,
which aarch64 gcc does by default; the reference Makefiles' ``-ffast-math``
is left out because it lets the compiler reassociate).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import sys
from typing import Dict, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(_HERE))

from formura_gb300.generator.config import decode_config  # noqa: E402
from formura_gb300.generator.manifest import compile_program  # noqa: E402
from oracle.emit_reference_c import Emitter  # noqa: E402

CFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11",
          "-Wno-unused-variable", "-Wno-unused-but-set-variable"]
BUILD_DIR = os.environ.get("FORMURA_ORACLE_BUILD", os.path.join(_HERE, "_build"))


class ReferenceProgram:
    """One program's generated C, compiled and loaded."""

    def __init__(self, fmr_src: str, yaml_text: str, name: str = "prog",
                 build_dir: Optional[str] = None, extra_cflags=()):
        self.mm = compile_program(fmr_src, decode_config(yaml_text))
        em = Emitter(self.mm, f"{name}.h")
        self.navi_spec = em.navi_fields()
        h, c = em.emit()
        key = hashlib.sha1((h + c + " ".join(CFLAGS + list(extra_cflags))).encode()).hexdigest()[:12]
        d = os.path.join(build_dir or BUILD_DIR, f"{name}_{key}")
        os.makedirs(d, exist_ok=True)
        so = os.path.join(d, f"lib{name}.so")
        if not os.path.exists(so):
            with open(os.path.join(d, f"{name}.h"), "w") as f:
                f.write(h)
            with open(os.path.join(d, f"{name}.c"), "w") as f:
                f.write(c)
            tmp = so + f".tmp{os.getpid()}"
            cmd = ["gcc", *CFLAGS, *extra_cflags, os.path.join(d, f"{name}.c"), "-o", tmp, "-lm"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
            os.replace(tmp, so)
        self.dir = d
        self.so_path = so
        self.lib = ctypes.CDLL(so)
        self.fields = self.mm.fields
        self.shape = tuple(self.mm.om.config.grid_per_node)
        n = int(np.prod(self.shape))
        self._data = (ctypes.c_double * (n * len(self.fields))).in_dll(
            self.lib, self.mm.om.genv.grid_struct_instance_name)
        self._arr = np.ctypeslib.as_array(self._data).reshape((len(self.fields),) + self.shape)

        cmap = {"int": ctypes.c_int, "double": ctypes.c_double}
        self.Navi = type("Formura_Navi", (ctypes.Structure,),
                         {"_fields_": [(nm, cmap[t]) for nm, t, _ in self.navi_spec]})
        self.navi = self.Navi()
        self.lib.Formura_Init.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(self.Navi)]
        self.lib.Formura_Forward.argtypes = [ctypes.POINTER(self.Navi)]
        for a in self.mm.om.genv.axes:
            fn = getattr(self.lib, f"to_pos_{a}")
            fn.argtypes = [ctypes.c_int, self.Navi]
            fn.restype = ctypes.c_double

    # -- the generated C API --------------------------------------------
    def init(self):
        self.lib.Formura_Init(None, None, ctypes.byref(self.navi))
        return self.navi_dict()

    def forward(self, calls: int = 1):
        for _ in range(calls):
            self.lib.Formura_Forward(ctypes.byref(self.navi))
        return self.navi_dict()

    def finalize(self):
        self.lib.Formura_Finalize()

    def navi_dict(self) -> Dict[str, float]:
        return {nm: getattr(self.navi, nm) for nm, _, _ in self.navi_spec}

    def to_pos(self, axis: str, i: int) -> float:
        return getattr(self.lib, f"to_pos_{axis}")(i, self.navi)

    # -- formura_data hook ----------------------------------------------
    def get(self, field: str) -> np.ndarray:
        return self._arr[self.fields.index(field)].copy()

    def set(self, field: str, value: np.ndarray):
        self._arr[self.fields.index(field)][...] = value

    def state(self) -> Dict[str, np.ndarray]:
        return {f: self.get(f) for f in self.fields}
