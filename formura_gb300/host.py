"""Host side of the GB300 backend, in Python.

* :class:`Library` binds the C ABI of ``libformura_gb300.so``
  (``include/formura_gb300.h``) with ctypes.
* :class:`Grid` is one device-resident grid (``fgb_open``/``fgb_forward``/...).
* :class:`FormuraProgram` is the drop-in: it generates the program's C pair
  with the GB300 backend (``generator/dropin.py``), compiles it against the
  library and exposes the generated API the way a Formura driver uses it
  (``Formura_Init``, ``Formura_Forward``, ``formura_data``, ``to_pos_*``;
  ``src/Formura/Generator/Templates.hs:221-334``).

Nothing here falls back to the CPU: if the CUDA library cannot be loaded,
every entry point raises.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import build as _build
from .generator.config import decode_config
from .generator.cuda import emit_cuda, uniform_table
from .generator.dropin import PRECISIONS, emit_dropin, steps_per_forward
from .generator.manifest import compile_program

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


class FgbError(RuntimeError):
    pass


class Library:
    _inst: Optional["Library"] = None

    def __init__(self, path: Optional[str] = None):
        path = path or _build.LIB
        if not os.path.exists(path):
            raise FgbError(f"{path} is missing: run formura_gb300.build.build() first "
                           "(the GB300 backend has no CPU fallback)")
        self.path = path
        self.lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
        L = self.lib
        L.fgb_last_error.restype = ctypes.c_char_p
        L.fgb_program_name.restype = ctypes.c_char_p
        L.fgb_program_field.restype = ctypes.c_char_p
        L.fgb_program_field.argtypes = [ctypes.c_char_p, ctypes.c_int]
        L.fgb_program_query.argtypes = [ctypes.c_char_p] + [ctypes.POINTER(ctypes.c_int)] * 5
        L.fgb_open.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        L.fgb_close.argtypes = [ctypes.c_void_p]
        L.fgb_upload.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.fgb_download.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.fgb_forward.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.fgb_synchronize.argtypes = [ctypes.c_void_p]
        L.fgb_stream.argtypes = [ctypes.c_void_p]
        L.fgb_stream.restype = ctypes.c_void_p
        L.fgb_state_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
        L.fgb_launch_count.argtypes = [ctypes.c_void_p]
        L.fgb_launch_count.restype = ctypes.c_int64
        L.fgb_set_scales.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_int]
        L.fgb_variant_count.argtypes = [ctypes.c_void_p]
        L.fgb_variant_info.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3
        L.fgb_set_variant.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.fgb_variant.argtypes = [ctypes.c_void_p]
        L.fgb_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.fgb_backward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.fgb_gradient_forward.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.fgb_gradient_backward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.fgb_gradient_backward_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.fgb_gradient_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
        L.fgb_adjoint_steps.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.fgb_totals.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int]

    @classmethod
    def get(cls) -> "Library":
        if cls._inst is None:
            cls._inst = Library()
        return cls._inst

    def check(self, rc: int, what: str):
        if rc != 0:
            raise FgbError(f"{what}: {self.lib.fgb_last_error().decode()} (code {rc})")

    def programs(self) -> List[str]:
        return [self.lib.fgb_program_name(i).decode() for i in range(self.lib.fgb_program_count())]

    def query(self, program: str) -> Dict[str, int]:
        vals = [ctypes.c_int() for _ in range(5)]
        self.check(self.lib.fgb_program_query(program.encode(), *[ctypes.byref(v) for v in vals]), "query")
        return dict(zip(["dim", "nfields", "nuniforms", "sleeve", "shift"], [v.value for v in vals]))

    def fields(self, program: str) -> List[str]:
        """The program's state fields in formura_data order."""
        n = self.query(program)["nfields"]
        return [self.lib.fgb_program_field(program.encode(), i).decode() for i in range(n)]


class Grid:
    """One device-resident grid of a program compiled into the library."""

    def __init__(self, program: str, shape: Sequence[int], precision: str, uniforms: Sequence[float],
                 scales: Optional[Sequence[float]] = None, lib: Optional[Library] = None):
        self.L = lib or Library.get()
        self.program = program
        self.shape = tuple(int(x) for x in shape)
        self.precision = precision
        info = self.L.query(program)
        self.nfields = info["nfields"]
        self.shift = info["shift"]
        u = (ctypes.c_double * max(1, len(uniforms)))(*uniforms)
        shp = (ctypes.c_int * len(self.shape))(*self.shape)
        h = ctypes.c_void_p()
        self.L.check(self.L.lib.fgb_open(program.encode(), shp, len(self.shape), PRECISIONS[precision], u,
                                         len(uniforms), ctypes.byref(h)), "fgb_open")
        self.h = h
        if scales is not None:
            sc = (ctypes.c_float * self.nfields)(*scales)
            self.L.check(self.L.lib.fgb_set_scales(self.h, sc, self.nfields), "fgb_set_scales")

    def close(self):
        if self.h:
            self.L.lib.fgb_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, state: np.ndarray):
        a = np.ascontiguousarray(state, dtype=np.float64)
        assert a.size == self.nfields * int(np.prod(self.shape))
        self.L.check(self.L.lib.fgb_upload(self.h, a.ctypes.data), "fgb_upload")

    def download(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.nfields,) + self.shape, np.float64)
        self.L.check(self.L.lib.fgb_download(self.h, out.ctypes.data), "fgb_download")
        return out

    def forward(self, nsteps: int):
        self.L.check(self.L.lib.fgb_forward(self.h, int(nsteps)), "fgb_forward")

    def synchronize(self):
        self.L.check(self.L.lib.fgb_synchronize(self.h), "fgb_synchronize")

    def variants(self) -> List[Dict[str, int]]:
        out = []
        for i in range(self.L.lib.fgb_variant_count(self.h)):
            v = [ctypes.c_int() for _ in range(3)]
            self.L.check(self.L.lib.fgb_variant_info(self.h, i, *[ctypes.byref(x) for x in v]), "variant_info")
            out.append({"index": i, "tile_x": v[0].value, "tile_y": v[1].value, "steps": v[2].value})
        return out

    def set_variant(self, index: int):
        self.L.check(self.L.lib.fgb_set_variant(self.h, int(index)), "fgb_set_variant")

    @property
    def variant(self) -> int:
        return self.L.lib.fgb_variant(self.h)

    def autotune(self, trial_steps: int = 32) -> int:
        c = ctypes.c_int()
        self.L.check(self.L.lib.fgb_autotune(self.h, int(trial_steps), ctypes.byref(c)), "fgb_autotune")
        return c.value

    def totals(self) -> np.ndarray:
        """FP64 sum of each field of the current state."""
        out = (ctypes.c_double * self.nfields)()
        self.L.check(self.L.lib.fgb_totals(self.h, out, self.nfields), "fgb_totals")
        return np.array(out[:])

    # -- reverse mode -----------------------------------------------------
    def backward(self, lam_next: np.ndarray) -> np.ndarray:
        """One adjoint step at the current state: (dF/du)^T lam_next."""
        a = np.ascontiguousarray(lam_next, dtype=np.float64)
        out = np.empty((self.nfields,) + self.shape, np.float64)
        self.L.check(self.L.lib.fgb_backward(self.h, a.ctypes.data, out.ctypes.data), "fgb_backward")
        return out

    def adjoint_steps(self, nsteps: int):
        self.L.check(self.L.lib.fgb_adjoint_steps(self.h, int(nsteps)), "fgb_adjoint_steps")

    def gradient_forward(self, nsteps: int, snapshots: int):
        self.L.check(self.L.lib.fgb_gradient_forward(self.h, int(nsteps), int(snapshots)), "fgb_gradient_forward")

    def gradient_backward(self, seed: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(seed, dtype=np.float64)
        out = np.empty((self.nfields,) + self.shape, np.float64)
        self.L.check(self.L.lib.fgb_gradient_backward(self.h, a.ctypes.data, out.ctypes.data),
                     "fgb_gradient_backward")
        return out

    def gradient_stats(self):
        f, a = ctypes.c_int64(), ctypes.c_int64()
        self.L.check(self.L.lib.fgb_gradient_stats(self.h, ctypes.byref(f), ctypes.byref(a)), "fgb_gradient_stats")
        return {"forward_steps": f.value, "adjoint_steps": a.value}

    def gradient(self, u0: np.ndarray, nsteps: int, snapshots: int, seed_fn):
        """(u_T, dJ/du_0) for a loss J(u_T) whose derivative seed_fn(u_T) gives."""
        self.upload(u0)
        self.gradient_forward(nsteps, snapshots)
        uT = self.download()
        return uT, self.gradient_backward(seed_fn(uT))

    @property
    def stream(self) -> int:
        return self.L.lib.fgb_stream(self.h)

    @property
    def launches(self) -> int:
        return self.L.lib.fgb_launch_count(self.h)

    def state_pointers(self) -> List[int]:
        p = (ctypes.c_void_p * self.nfields)()
        self.L.check(self.L.lib.fgb_state_device(self.h, p, self.nfields), "fgb_state_device")
        return [int(x) for x in p]


class Batch:
    """An ensemble of independent 2D grids of one program (fgb_batch_*)."""

    def __init__(self, program: str, shapes: Sequence[Sequence[int]], precision: str,
                 uniforms: Sequence[Sequence[float]], lib: Optional[Library] = None):
        self.L = lib or Library.get()
        L = self.L.lib
        L.fgb_batch_open.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        for fn in ("fgb_batch_close", "fgb_batch_synchronize", "fgb_batch_variant_count", "fgb_batch_variant"):
            getattr(L, fn).argtypes = [ctypes.c_void_p]
        L.fgb_batch_upload.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.fgb_batch_download.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.fgb_batch_forward.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.fgb_batch_set_variant.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.fgb_batch_variant_info.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3
        L.fgb_batch_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.fgb_batch_stream.argtypes = [ctypes.c_void_p]
        L.fgb_batch_stream.restype = ctypes.c_void_p
        L.fgb_batch_launch_count.argtypes = [ctypes.c_void_p]
        L.fgb_batch_launch_count.restype = ctypes.c_int64
        self.shapes = [tuple(int(x) for x in sh) for sh in shapes]
        self.nfields = self.L.query(program)["nfields"]
        nu = len(uniforms[0]) if len(uniforms) else 0
        flat = [float(x) for u in uniforms for x in u]
        shp = (ctypes.c_int * (2 * len(self.shapes)))(*[x for sh in self.shapes for x in sh])
        u = (ctypes.c_double * max(1, len(flat)))(*flat)
        h = ctypes.c_void_p()
        self.L.check(L.fgb_batch_open(program.encode(), len(self.shapes), shp, PRECISIONS[precision], u, nu,
                                      ctypes.byref(h)), "fgb_batch_open")
        self.h = h

    def close(self):
        if self.h:
            self.L.lib.fgb_batch_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, i: int, state: np.ndarray):
        a = np.ascontiguousarray(state, dtype=np.float64)
        self.L.check(self.L.lib.fgb_batch_upload(self.h, i, a.ctypes.data), "fgb_batch_upload")

    def download(self, i: int) -> np.ndarray:
        out = np.empty((self.nfields,) + self.shapes[i], np.float64)
        self.L.check(self.L.lib.fgb_batch_download(self.h, i, out.ctypes.data), "fgb_batch_download")
        return out

    def forward(self, nsteps: int):
        self.L.check(self.L.lib.fgb_batch_forward(self.h, int(nsteps)), "fgb_batch_forward")

    def synchronize(self):
        self.L.check(self.L.lib.fgb_batch_synchronize(self.h), "fgb_batch_synchronize")

    def variants(self):
        out = []
        for i in range(self.L.lib.fgb_batch_variant_count(self.h)):
            v = [ctypes.c_int() for _ in range(3)]
            self.L.check(self.L.lib.fgb_batch_variant_info(self.h, i, *[ctypes.byref(x) for x in v]), "info")
            out.append({"index": i, "tile_x": v[0].value, "tile_y": v[1].value, "steps": v[2].value})
        return out

    def set_variant(self, i: int):
        self.L.check(self.L.lib.fgb_batch_set_variant(self.h, int(i)), "fgb_batch_set_variant")

    @property
    def variant(self) -> int:
        return self.L.lib.fgb_batch_variant(self.h)

    def autotune(self, trial_steps: int = 32) -> int:
        c = ctypes.c_int()
        self.L.check(self.L.lib.fgb_batch_autotune(self.h, int(trial_steps), ctypes.byref(c)), "fgb_batch_autotune")
        return c.value

    @property
    def stream(self) -> int:
        return self.L.lib.fgb_batch_stream(self.h)

    @property
    def launches(self) -> int:
        return self.L.lib.fgb_batch_launch_count(self.h)


def program_uniforms(fmr_src: str, yaml_text: str, program: str,
                     params: Optional[Dict[str, float]] = None, runtime_params: Optional[Sequence[str]] = None):
    """(compiled MM program, uniform table) of a library program for one
    config; `params` overrides the runtime parameters (e.g. F, kappa)."""
    mm = compile_program(fmr_src, decode_config(yaml_text))
    if runtime_params is None:
        runtime_params = _build.library_runtime_params(program)
    kp = emit_cuda(mm, program, list(runtime_params))
    return mm, uniform_table(mm, kp, params)


def builtin_program(name: str):
    """Source and config of a program shipped with the library."""
    return _build.program_sources(name)


class FormuraProgram:
    """The generated C API of one program, running on the GB300 backend."""

    def __init__(self, fmr_src: str, yaml_text: str, program: str, name: Optional[str] = None,
                 params: Optional[Dict[str, float]] = None, runtime_params: Optional[Sequence[str]] = None,
                 build_dir: Optional[str] = None):
        lib = Library.get()
        self.mm = compile_program(fmr_src, decode_config(yaml_text))
        name = name or program
        if runtime_params is None:
            runtime_params = _build.library_runtime_params(program)
        h, c = emit_dropin(self.mm, program, f"{name}.h", params, list(runtime_params))
        key = hashlib.sha1((h + c + lib.path).encode()).hexdigest()[:12]
        d = os.path.join(build_dir or os.path.join(_build.BUILD, "dropin"), f"{name}_{key}")
        os.makedirs(d, exist_ok=True)
        so = os.path.join(d, f"lib{name}_gpu.so")
        if not os.path.exists(so):
            with open(os.path.join(d, f"{name}.h"), "w") as f:
                f.write(h)
            with open(os.path.join(d, f"{name}.c"), "w") as f:
                f.write(c)
            tmp = so + f".tmp{os.getpid()}"
            libdir = os.path.dirname(lib.path)
            cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off",
                   "-I", os.path.join(ROOT, "include"), os.path.join(d, f"{name}.c"), "-o", tmp,
                   "-L", libdir, "-lformura_gb300", f"-Wl,-rpath,{libdir}", "-lm"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise FgbError("drop-in build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
            os.replace(tmp, so)
        self.so_path = so
        self.lib = ctypes.CDLL(so)
        self.fields = self.mm.fields
        self.shape = tuple(self.mm.om.config.grid_per_node)
        self.steps_per_forward = steps_per_forward(self.mm)
        n = int(np.prod(self.shape))
        self._data = (ctypes.c_double * (n * len(self.fields))).in_dll(
            self.lib, self.mm.om.genv.grid_struct_instance_name)
        self._arr = np.ctypeslib.as_array(self._data).reshape((len(self.fields),) + self.shape)
        axes = self.mm.om.genv.axes
        spec = [("time_step", ctypes.c_int)]
        spec += [("lower_" + a, ctypes.c_int) for a in axes] + [("upper_" + a, ctypes.c_int) for a in axes]
        spec += [("space_interval_" + a, ctypes.c_double) for a in axes] + [("my_rank", ctypes.c_int)]
        spec += [("offset_" + a, ctypes.c_int) for a in axes] + [("length_" + a, ctypes.c_double) for a in axes]
        spec += [("total_grid_" + a, ctypes.c_int) for a in axes]
        self.navi_names = [nm for nm, _ in spec]
        self.Navi = type("Formura_Navi", (ctypes.Structure,), {"_fields_": spec})
        self.navi = self.Navi()
        self.lib.Formura_Init.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(self.Navi)]
        self.lib.Formura_Forward.argtypes = [ctypes.POINTER(self.Navi)]
        for a in axes:
            fn = getattr(self.lib, f"to_pos_{a}")
            fn.argtypes = [ctypes.c_int, self.Navi]
            fn.restype = ctypes.c_double

    def init(self):
        self.lib.Formura_Init(None, None, ctypes.byref(self.navi))
        return self.navi_dict()

    def forward(self, calls: int = 1):
        for _ in range(calls):
            self.lib.Formura_Forward(ctypes.byref(self.navi))
        return self.navi_dict()

    def finalize(self):
        self.lib.Formura_Finalize()

    def navi_dict(self):
        return {nm: getattr(self.navi, nm) for nm in self.navi_names}

    def to_pos(self, axis: str, i: int) -> float:
        return getattr(self.lib, f"to_pos_{axis}")(i, self.navi)

    def get(self, field: str) -> np.ndarray:
        return self._arr[self.fields.index(field)].copy()

    def set(self, field: str, value: np.ndarray):
        self._arr[self.fields.index(field)][...] = value

    def state(self):
        return {f: self.get(f) for f in self.fields}
