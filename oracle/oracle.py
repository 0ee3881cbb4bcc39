"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Runs the C restatement in ewf_oracle.c on an ``elanfmt_gb300.inputs.Model``.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import this module; the
product never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from elanfmt_gb300 import fields as F
from elanfmt_gb300.inputs import separable_weights

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libewf_oracle.so")


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("model", C.c_int32),
                ("src_order", C.c_int32), ("bc1_rows", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
                ("c66", C.c_double), ("bx", C.c_double), ("by", C.c_double), ("bz", C.c_double),
                ("vdamp", C.c_double), ("c44", C.c_double), ("c55", C.c_double), ("damping", C.c_int32),
                ("no_bc1", C.c_int32), ("smu", C.c_double)]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        from . import build as _build

        _build.build_oracle()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        for suf in ("f32", "f64"):
            fn = getattr(lib, f"orc_run_{suf}")
            fn.restype = C.c_int
            fn.argtypes = [C.POINTER(Grid), P, P, P, P, P, C.c_int32, P, P, P, C.c_int32, C.c_int32, P, P,
                           C.c_int32, C.c_int32, C.c_int32]
        lib.orc_num_threads.restype = C.c_int
        _lib = lib
    return _lib


def num_threads() -> int:
    return load().orc_num_threads()


def _ptrs(arrs) -> C.Array:
    arr = (C.c_void_p * len(arrs))()
    for q, a in enumerate(arrs):
        arr[q] = None if a is None else a.ctypes.data
    return arr


def bc1_rows(m) -> int:
    return min(m.nx, m.ny + max(0, m.over_y), m.ny)


class State:
    """The 9 state fields (+ compensation) and traces of one oracle run."""

    def __init__(self, m, dtype):
        self.dtype = dtype
        self.f = [np.zeros(F.shape(q, m.nx, m.ny, m.nz), dtype) for q in F.STATE]
        self.comp = None
        nrec = 0 if m.receivers is None else len(m.receivers)
        self.traces = np.zeros((nrec, m.nt), np.float64)
        self.it = 0


class Runner:
    """Model arrays converted once to the run's precision; ``step`` times only the C loop."""

    def __init__(self, m, precision: int = F.PREC_F32, state: State | None = None):
        self.lib = load()
        self.m = m
        self.dtype = dtype = np.float64 if precision == F.PREC_F64 else np.float32
        if state is None:
            state = State(m, dtype)
            if precision == F.PREC_F32_KAHAN:
                state.comp = [np.zeros(F.shape(q, m.nx, m.ny, m.nz), dtype) for q in (F.F_VX, F.F_VY, F.F_VZ)]
        self.state = state
        self.grid = Grid(m.nx, m.ny, m.nz, m.model, m.src_order, bc1_rows(m), m.dx, m.dy, m.dz, m.dt, m.c66, m.bx,
                         m.by, m.bz, getattr(m, "vdamp", 0.0), getattr(m, "c44", 0.0), getattr(m, "c55", 0.0),
                         m.damping, int(getattr(m, "free_surface", F.FS_BC1) == F.FS_NONE),
                         float(getattr(m, "surface_mu", 0.0)))
        cv = lambda a: np.ascontiguousarray(a, dtype=dtype)  # noqa: E731
        if m.model == F.MODEL_ISO:
            self.mats = [cv(m.materials[F.M_C11]), cv(m.materials[F.M_C12])]
            keys = F.PERCOMP_WEIGHTS if m.damping == F.DAMP_PERCOMP else (F.D_WX, F.D_WY, F.D_WZ)
            self.w = [cv(m.damping_arrays[k]) for k in keys]
            self.W = None
        else:
            # orthorhombic slots; the 9 km scheme leaves C22, C33, C13, C23 empty
            self.mats = [cv(m.materials[k]) if k in m.materials else None for k in F.ORTHO_MATERIALS]
            self.w = None
            if F.D_W3D in m.damping_arrays:
                self.W = cv(m.damping_arrays[F.D_W3D])
            else:
                self.W = separable_weights(m.damping_arrays[F.D_WX], m.damping_arrays[F.D_WY],
                                           m.damping_arrays[F.D_WZ], dtype)
        self.src = np.ascontiguousarray(m.sources if m.sources is not None else np.zeros((0, 4)), np.int32)
        self.coef = np.ascontiguousarray(m.source_coef if m.source_coef is not None else np.zeros(0), np.float64)
        self.stf = np.ascontiguousarray(m.stf if m.stf is not None else np.zeros(m.nt), np.float64)
        self.rec = np.ascontiguousarray(m.receivers if m.receivers is not None else np.zeros((0, 4)), np.int32)
        self.fn = self.lib.orc_run_f64 if dtype == np.float64 else self.lib.orc_run_f32
        self.fp = _ptrs(state.f)
        self.cp = _ptrs(state.comp) if state.comp is not None else None
        self.mp = _ptrs(self.mats)
        self.wp = _ptrs(self.w) if self.w is not None else None

    def step(self, nsteps: int) -> State:
        s = self.state
        st = self.fn(C.byref(self.grid), self.fp, self.cp, self.mp, self.wp,
                     None if self.W is None else self.W.ctypes.data, len(self.coef), self.src.ctypes.data,
                     self.coef.ctypes.data, self.stf.ctypes.data, len(self.stf), len(self.rec), self.rec.ctypes.data,
                     s.traces.ctypes.data, self.m.nt, s.it, nsteps)
        if st != 0:
            raise RuntimeError(f"oracle run failed with status {st}")
        s.it += nsteps
        return s


def run(m, nsteps: int, precision: int = F.PREC_F32, state: State | None = None) -> State:
    """Advances `state` (new, zeroed, if None) by nsteps with the oracle."""
    return Runner(m, precision, state).step(nsteps)
