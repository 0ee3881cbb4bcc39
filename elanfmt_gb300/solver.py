"""Python binding of libewfd.so (ctypes) and the host-side mirror of the reference's run.

The reference's interface for this path is an executable plus a file contract
(FastWaveED_GPU3D_v1.cu:390-559): inputs read from fixed-name files, the time loop, outputs
written as raw arrays.  ``Solver`` exposes the same steps over the C ABI -- set inputs, run,
read seismograms and snapshots -- and ``run_legacy`` is the executable's whole flow.  Errors are
raised as ``EwfError`` carrying the C status code; there is no CPU fallback: without the CUDA
library (or a GPU) every call fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import fields as F

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libewfd.so")


class EwfError(RuntimeError):
    def __init__(self, status: int, where: str, message: str = ""):
        self.status = status
        super().__init__(f"{where}: {F.STATUS.get(status, status)} ({message})")


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("nt", C.c_int32),
        ("model", C.c_int32), ("precision", C.c_int32), ("damping", C.c_int32), ("src_order", C.c_int32),
        ("over_y", C.c_int32), ("nout", C.c_int32), ("kchunk", C.c_int32), ("graph_steps", C.c_int32),
        ("check_finite", C.c_int32), ("fused", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
        ("c66", C.c_double), ("c44", C.c_double), ("c55", C.c_double),
        ("bx", C.c_double), ("by", C.c_double), ("bz", C.c_double),
        ("vdamp", C.c_double),
        ("workdir", C.c_char_p),
        ("free_surface", C.c_int32), ("reserved", C.c_int32), ("surface_mu", C.c_double),
    ]


# every symbol the header declares, with its ctypes signature
SIGNATURES = {
    "ewf_abi_version": (C.c_int, []),
    "ewf_strerror": (C.c_char_p, [C.c_int]),
    "ewf_last_error": (C.c_char_p, []),
    "ewf_params_default": (None, [C.POINTER(Params)]),
    "ewf_legacy_params": (C.c_int, [C.POINTER(Params)]),
    "ewf_create": (C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "ewf_destroy": (None, [C.c_void_p]),
    "ewf_get_params": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
    "ewf_load_legacy_inputs": (C.c_int, [C.c_void_p]),
    "ewf_set_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t, C.c_int32]),
    "ewf_get_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t, C.c_int32]),
    "ewf_field_size": (C.c_size_t, [C.c_void_p, C.c_int32]),
    "ewf_set_stf": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "ewf_set_moment_tensor": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "ewf_set_sources": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "ewf_set_receivers": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "ewf_receiver_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_reset": (C.c_int, [C.c_void_p]),
    "ewf_run": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_get_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_get_seismograms": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "ewf_last_run_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ewf_time_kernels": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "ewf_launches_per_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_write_legacy_outputs": (C.c_int, [C.c_void_p]),
    "ewf_write_snapshot": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_write_snapshot_async": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_snapshot_wait": (C.c_int, [C.c_void_p]),
    "ewf_pack_field_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p, C.c_int32,
                                         C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "ewf_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "ewf_set_wave": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_get_wave": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_set_tile": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_set_onepass": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_get_onepass": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_staged_test_hold": (C.c_int, [C.c_int32, C.c_int32]),
    "ewf_set_dependent_launch": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_set_l2_prefetch": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_get_l2_prefetch": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_get_dependent_launch": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_get_tile": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_wave_hold": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_batch_create": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "ewf_batch_destroy": (None, [C.c_void_p]),
    "ewf_batch_set_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t, C.c_int32]),
    "ewf_batch_set_stf": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    "ewf_batch_set_sources": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "ewf_batch_set_moment_tensor": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_int32,
                                              C.c_int32, C.c_int32]),
    "ewf_batch_set_receivers": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "ewf_batch_reset": (C.c_int, [C.c_void_p]),
    "ewf_batch_run": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_batch_last_run_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ewf_batch_get_seismograms": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t]),
    "ewf_batch_get_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t,
                                      C.c_int32]),
    "ewf_batch_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "ewf_batch_set_tile": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_batch_get_tile": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_batch_set_l2_prefetch": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_batch_set_launch": (C.c_int, [C.c_void_p, C.c_int32]),
    "ewf_batch_get_launch": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_batch_get_l2_prefetch": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ewf_mlp_gemm": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                               C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "ewf_mlp_status": (C.c_int, []),
    "ewf_sosfilt": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_int64]),
    "ewf_sosfilt_device": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]),
    "ewf_mlp_test_hold": (C.c_int, [C.c_int32, C.c_int32]),
    "ewf_mlp_transpose": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "ewf_mlp_gelu_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "ewf_mlp_bias_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "ewf_mlp_mse_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_float, C.c_void_p, C.c_int32,
                                   C.c_void_p]),
    "ewf_mlp_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_float,
                               C.c_float, C.c_float, C.c_float, C.c_int32, C.c_float, C.c_void_p]),
    "ewf_mlp_combine": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                  C.c_void_p]),
    "ewf_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ewf_restore": (C.c_int, [C.c_void_p, C.c_char_p]),
}

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads libewfd.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is not built: run elanfmt_gb300.build.build() (needs nvcc)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _check(st: int, where: str) -> None:
    if st != 0:
        msg = load_library().ewf_last_error()
        raise EwfError(st, where, msg.decode(errors="replace") if msg else "")


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def default_params() -> Params:
    p = Params()
    load_library().ewf_params_default(C.byref(p))
    return p


class Solver:
    """One simulation on the current CUDA device (a libewfd handle)."""

    def __init__(self, params: Params):
        lib = load_library()
        self._lib = lib
        self._workdir = params.workdir  # keep the bytes alive
        self.params = params
        h = C.c_void_p()
        _check(lib.ewf_create(C.byref(params), C.byref(h)), "ewf_create")
        self._h = h
        self.nrec = 0

    # -- construction --------------------------------------------------------------------
    @classmethod
    def from_model(cls, m, precision: int = F.PREC_F32, kchunk: int = 0, graph_steps: int = 0,
                   check_finite: bool = True, damping: int | None = None, nout: int = 0,
                   fused: int | None = None, workdir: str | None = None) -> "Solver":
        """`fused`: the step form, F.STEP_SPLIT (default), F.STEP_FUSED or F.STEP_WAVE."""
        p = default_params()
        p.nx, p.ny, p.nz, p.nt = m.nx, m.ny, m.nz, m.nt
        p.model, p.precision = m.model, precision
        p.damping = m.damping if damping is None else damping
        p.src_order, p.over_y, p.nout = m.src_order, m.over_y, nout
        p.kchunk, p.graph_steps, p.check_finite = kchunk, graph_steps, int(check_finite)
        p.dx, p.dy, p.dz, p.dt = m.dx, m.dy, m.dz, m.dt
        p.c66, p.bx, p.by, p.bz = m.c66, m.bx, m.by, m.bz
        p.c44, p.c55 = getattr(m, "c44", 0.0), getattr(m, "c55", 0.0)
        p.vdamp = getattr(m, "vdamp", 0.0)
        p.free_surface = getattr(m, "free_surface", F.FS_BC1)
        p.surface_mu = getattr(m, "surface_mu", 0.0)
        if fused is not None:
            p.fused = int(fused)
        if workdir is not None:
            p.workdir = os.fsencode(workdir)
        s = cls(p)
        try:
            s.set_model(m)
        except Exception:
            s.close()
            raise
        return s

    @classmethod
    def legacy(cls, workdir: str, nx: int, ny: int, nz: int, model: int = F.MODEL_ISO, nt: int = 0,
               precision: int = F.PREC_F32, over_y: int = 0, check_finite: bool = True) -> "Solver":
        """The reference executable's set-up: parameters from pa*.dat, inputs from workdir."""
        p = default_params()
        p.nx, p.ny, p.nz, p.nt = nx, ny, nz, nt
        p.model, p.precision = model, precision
        p.damping = F.DAMP_PML1D if model == F.MODEL_ISO else F.DAMP_W3D
        p.src_order = F.SRC_BEFORE_BC1 if model == F.MODEL_ISO else F.SRC_AFTER_BC1
        p.over_y, p.check_finite = over_y, int(check_finite)
        p.workdir = os.fsencode(workdir)
        _check(load_library().ewf_legacy_params(C.byref(p)), "ewf_legacy_params")
        s = cls(p)
        try:
            _check(s._lib.ewf_load_legacy_inputs(s._h), "ewf_load_legacy_inputs")
            s.nrec = s.receiver_count()
        except Exception:
            s.close()
            raise
        return s

    def receiver_count(self) -> int:
        n = C.c_int32()
        _check(self._lib.ewf_receiver_count(self._h, C.byref(n)), "ewf_receiver_count")
        return n.value

    def set_model(self, m) -> None:
        for fid, arr in m.materials.items():
            self.set_field(fid, arr)
        for fid, arr in m.damping_arrays.items():
            self.set_field(fid, arr)
        if m.stf is not None:
            self.set_stf(m.stf)
        if m.sources is not None:
            self.set_sources(m.sources, m.source_coef)
        if m.receivers is not None:
            self.set_receivers(m.receivers)

    # -- inputs ----------------------------------------------------------------------------
    def set_field(self, fid: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        if a.dtype not in (np.float32, np.float64):
            a = a.astype(np.float32)
        _check(self._lib.ewf_set_field(self._h, fid, _ptr(a), a.size, a.itemsize), f"ewf_set_field({fid})")

    def set_field_ptr(self, fid: int, ptr: int, n: int, itemsize: int) -> None:
        """set_field from a raw host pointer (e.g. pinned memory owned by the caller)."""
        _check(self._lib.ewf_set_field(self._h, fid, C.c_void_p(ptr), n, itemsize), f"ewf_set_field({fid})")

    def set_stf(self, stf: np.ndarray) -> None:
        a = np.ascontiguousarray(stf, dtype=np.float64)
        _check(self._lib.ewf_set_stf(self._h, _ptr(a), a.size), "ewf_set_stf")

    def set_sources(self, entries: np.ndarray, coef: np.ndarray) -> None:
        e = np.ascontiguousarray(entries, dtype=np.int32)
        c = np.ascontiguousarray(coef, dtype=np.float64)
        _check(self._lib.ewf_set_sources(self._h, len(c), _ptr(e), _ptr(c)), "ewf_set_sources")

    def set_moment_tensor(self, mt, xs: int, ys: int, zs: int, stencil: int) -> None:
        a = np.ascontiguousarray(mt, dtype=np.float64)
        _check(self._lib.ewf_set_moment_tensor(self._h, _ptr(a), xs, ys, zs, stencil), "ewf_set_moment_tensor")

    def set_receivers(self, rec: np.ndarray) -> None:
        r = np.ascontiguousarray(rec, dtype=np.int32).reshape(-1, 4)
        _check(self._lib.ewf_set_receivers(self._h, len(r), _ptr(r)), "ewf_set_receivers")
        self.nrec = len(r)

    # -- running -----------------------------------------------------------------------------
    def run(self, nsteps: int) -> float:
        """Advances nsteps; returns the device time of the call in ms."""
        _check(self._lib.ewf_run(self._h, int(nsteps)), "ewf_run")
        return self.last_run_ms()

    def reset(self) -> None:
        _check(self._lib.ewf_reset(self._h), "ewf_reset")

    def step(self) -> int:
        it = C.c_int32()
        _check(self._lib.ewf_get_step(self._h, C.byref(it)), "ewf_get_step")
        return it.value

    def time_kernels(self, nsteps: int) -> dict:
        """Advances nsteps launching kernels one by one between CUDA events; average ms per launch."""
        out = (C.c_double * 4)()
        _check(self._lib.ewf_time_kernels(self._h, int(nsteps), out), "ewf_time_kernels")
        return dict(zip(("stress", "inject", "velocity", "record"), list(out)))

    def autotune(self, nsteps: int = 30) -> int:
        """Picks the fastest z-chunk (and, for the two-kernel step, tile height) by timing `nsteps`
        steps per candidate; resets the state.  Returns the z-chunk."""
        k = C.c_int32()
        _check(self._lib.ewf_autotune(self._h, int(nsteps), C.byref(k)), "ewf_autotune")
        return k.value

    def set_tile(self, tile_y: int) -> None:
        """Two-kernel step: CTA tile height in rows of 32 columns (results do not depend on it)."""
        _check(self._lib.ewf_set_tile(self._h, int(tile_y)), "ewf_set_tile")

    def tile(self) -> int:
        ty = C.c_int32()
        _check(self._lib.ewf_get_tile(self._h, C.byref(ty)), "ewf_get_tile")
        return ty.value

    def set_onepass(self, kernel: int) -> None:
        """One-pass step: its kernel, F.ONEPASS_TILE (default), F.ONEPASS_BAND4 / F.ONEPASS_BAND8 or
        F.ONEPASS_STAGED.  Results do not depend on it."""
        _check(self._lib.ewf_set_onepass(self._h, int(kernel)), "ewf_set_onepass")

    def onepass(self) -> int:
        v = C.c_int32()
        _check(self._lib.ewf_get_onepass(self._h, C.byref(v)), "ewf_get_onepass")
        return v.value

    def set_l2_prefetch(self, planes: int) -> None:
        """Two-kernel step: L2 prefetch distance of the velocity kernel (0 = off; results do not depend on it)."""
        _check(self._lib.ewf_set_l2_prefetch(self._h, int(planes)), "ewf_set_l2_prefetch")

    def l2_prefetch(self) -> int:
        v = C.c_int32()
        _check(self._lib.ewf_get_l2_prefetch(self._h, C.byref(v)), "ewf_get_l2_prefetch")
        return v.value

    def set_dependent_launch(self, on: bool) -> None:
        """Two-kernel step: programmatic dependent launches (default on; results do not depend on it)."""
        _check(self._lib.ewf_set_dependent_launch(self._h, int(bool(on))), "ewf_set_dependent_launch")

    def dependent_launch(self) -> bool:
        v = C.c_int32()
        _check(self._lib.ewf_get_dependent_launch(self._h, C.byref(v)), "ewf_get_dependent_launch")
        return bool(v.value)

    def set_wave(self, lag_pct: int) -> None:
        """Wavefront step: lag of the velocity items behind the stress items, percent of the resident
        CTAs (the autotuner sets it; results do not depend on it)."""
        _check(self._lib.ewf_set_wave(self._h, int(lag_pct)), "ewf_set_wave")

    def wave_hold(self, item: int) -> None:
        """Diagnostic: stress item `item` never publishes its done flag (-1: normal operation)."""
        _check(self._lib.ewf_wave_hold(self._h, int(item)), "ewf_wave_hold")

    def wave_lag(self) -> int:
        lag = C.c_int32()
        _check(self._lib.ewf_get_wave(self._h, C.byref(lag)), "ewf_get_wave")
        return lag.value

    def launches_per_step(self) -> int:
        n = C.c_int32()
        _check(self._lib.ewf_launches_per_step(self._h, C.byref(n)), "ewf_launches_per_step")
        return n.value

    def last_run_ms(self) -> float:
        ms = C.c_double()
        _check(self._lib.ewf_last_run_ms(self._h, C.byref(ms)), "ewf_last_run_ms")
        return ms.value

    # -- outputs -----------------------------------------------------------------------------
    def field(self, fid: int, dtype=np.float32) -> np.ndarray:
        shp = F.shape(fid, self.params.nx, self.params.ny, self.params.nz, self.params.damping)
        out = np.empty(shp, dtype=dtype)
        _check(self._lib.ewf_get_field(self._h, fid, _ptr(out), out.size, out.itemsize), f"ewf_get_field({fid})")
        return out

    def seismograms(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.nrec, self.params.nt), dtype=np.float64)
        _check(self._lib.ewf_get_seismograms(self._h, _ptr(out), out.size), "ewf_get_seismograms")
        return out

    def write_legacy_outputs(self) -> None:
        _check(self._lib.ewf_write_legacy_outputs(self._h), "ewf_write_legacy_outputs")

    def write_snapshot(self, isave: int, wait: bool = True) -> None:
        """Vx, Vy, Vz to <isave>_0_V?.res in the work directory; wait=False queues the write and
        returns at once (ewf_write_snapshot_async; see snapshot_wait)."""
        if wait:
            _check(self._lib.ewf_write_snapshot(self._h, isave), "ewf_write_snapshot")
        else:
            _check(self._lib.ewf_write_snapshot_async(self._h, isave), "ewf_write_snapshot_async")

    def snapshot_wait(self) -> None:
        _check(self._lib.ewf_snapshot_wait(self._h), "ewf_snapshot_wait")

    def checkpoint(self, path: str) -> None:
        _check(self._lib.ewf_checkpoint(self._h, os.fsencode(path)), "ewf_checkpoint")

    def restore(self, path: str) -> None:
        _check(self._lib.ewf_restore(self._h, os.fsencode(path)), "ewf_restore")

    # -- lifetime ----------------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.ewf_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_legacy(workdir: str, nx: int, ny: int, nz: int, model: int = F.MODEL_ISO, nt: int = 0,
               precision: int = F.PREC_F32, autotune: int = 0) -> float:
    """The reference executable end to end: read inputs from workdir, run all nt steps, write
    0_infos.inf and 0_0_*.res.  Returns the device time in ms.  autotune > 0: the library's
    autotuner first times launch shapes over that many steps (outputs unchanged), as
    ``ewfd --autotune``."""
    with Solver.legacy(workdir, nx, ny, nz, model=model, nt=nt, precision=precision) as s:
        if autotune > 0:
            s.autotune(autotune)
        ms = s.run(s.params.nt)
        s.write_legacy_outputs()
    return ms


def params_for(m, precision: int = F.PREC_F32, kchunk: int = 0) -> Params:
    p = default_params()
    p.nx, p.ny, p.nz, p.nt = m.nx, m.ny, m.nz, m.nt
    p.model, p.precision, p.damping, p.src_order, p.over_y = m.model, precision, m.damping, m.src_order, m.over_y
    p.kchunk = kchunk
    p.dx, p.dy, p.dz, p.dt = m.dx, m.dy, m.dz, m.dt
    p.c66, p.bx, p.by, p.bz = m.c66, m.bx, m.by, m.bz
    p.c44, p.c55 = getattr(m, "c44", 0.0), getattr(m, "c55", 0.0)
    p.vdamp = getattr(m, "vdamp", 0.0)
    return p


class Batch:
    """Several problems x right-hand sides advanced together (ewf_batch_*).

    ``problems`` is a list of (Model, list of (sources, coef) per RHS); every problem's receivers
    are recorded for each of its RHS."""

    def __init__(self, problems, kchunk: int = 0):
        lib = load_library()
        self._lib = lib
        self.models = [m for m, _ in problems]
        self.nrhs = [len(r) for _, r in problems]
        n = len(problems)
        arr = (Params * n)(*[params_for(m, kchunk=kchunk) for m in self.models])
        rhs = (C.c_int32 * n)(*self.nrhs)
        h = C.c_void_p()
        _check(lib.ewf_batch_create(n, arr, rhs, C.byref(h)), "ewf_batch_create")
        self._h = h
        self.nt = self.models[0].nt
        try:
            for pid, (m, rl) in enumerate(problems):
                for fid, a in list(m.materials.items()) + list(m.damping_arrays.items()):
                    a = np.ascontiguousarray(a)
                    _check(lib.ewf_batch_set_field(h, pid, fid, _ptr(a), a.size, a.itemsize), "ewf_batch_set_field")
                stf = np.ascontiguousarray(m.stf, np.float64)
                _check(lib.ewf_batch_set_stf(h, pid, _ptr(stf), stf.size), "ewf_batch_set_stf")
                for r, (ent, coef) in enumerate(rl):
                    e = np.ascontiguousarray(ent, np.int32)
                    c = np.ascontiguousarray(coef, np.float64)
                    _check(lib.ewf_batch_set_sources(h, pid, r, len(c), _ptr(e), _ptr(c)), "ewf_batch_set_sources")
                if m.receivers is not None:
                    rec = np.ascontiguousarray(m.receivers, np.int32)
                    _check(lib.ewf_batch_set_receivers(h, pid, len(rec), _ptr(rec)), "ewf_batch_set_receivers")
        except Exception:
            self.close()
            raise

    def run(self, nsteps: int) -> float:
        _check(self._lib.ewf_batch_run(self._h, int(nsteps)), "ewf_batch_run")
        ms = C.c_double()
        _check(self._lib.ewf_batch_last_run_ms(self._h, C.byref(ms)), "ewf_batch_last_run_ms")
        return ms.value

    def reset(self) -> None:
        _check(self._lib.ewf_batch_reset(self._h), "ewf_batch_reset")

    def autotune(self, nsteps: int = 20) -> int:
        k = C.c_int32()
        _check(self._lib.ewf_batch_autotune(self._h, int(nsteps), C.byref(k)), "ewf_batch_autotune")
        return k.value

    def set_tile(self, tile_y: int) -> None:
        """CTA tile height of the batch's launches (4, 8 or 16 rows of 32 columns)."""
        _check(self._lib.ewf_batch_set_tile(self._h, int(tile_y)), "ewf_batch_set_tile")

    def tile(self) -> int:
        ty = C.c_int32()
        _check(self._lib.ewf_batch_get_tile(self._h, C.byref(ty)), "ewf_batch_get_tile")
        return ty.value

    def set_launch(self, own: int) -> None:
        """Single-RHS problems: 0 = one persistent launch per model family, 1 = launches of their own
        on parallel branches (results do not depend on it)."""
        _check(self._lib.ewf_batch_set_launch(self._h, int(own)), "ewf_batch_set_launch")

    def launch(self) -> int:
        v = C.c_int32()
        _check(self._lib.ewf_batch_get_launch(self._h, C.byref(v)), "ewf_batch_get_launch")
        return v.value

    def set_l2_prefetch(self, planes: int) -> None:
        """Multi-RHS problems: L2 prefetch distance of their velocity kernel (0 = off; results do not depend on it)."""
        _check(self._lib.ewf_batch_set_l2_prefetch(self._h, int(planes)), "ewf_batch_set_l2_prefetch")

    def l2_prefetch(self) -> int:
        v = C.c_int32()
        _check(self._lib.ewf_batch_get_l2_prefetch(self._h, C.byref(v)), "ewf_batch_get_l2_prefetch")
        return v.value

    def seismograms(self, prob: int, rhs: int) -> np.ndarray:
        m = self.models[prob]
        n = 0 if m.receivers is None else len(m.receivers)
        out = np.empty((n, self.nt), np.float64)
        _check(self._lib.ewf_batch_get_seismograms(self._h, prob, rhs, _ptr(out), out.size), "ewf_batch_get_seismograms")
        return out

    def field(self, prob: int, rhs: int, fid: int) -> np.ndarray:
        m = self.models[prob]
        out = np.empty(F.shape(fid, m.nx, m.ny, m.nz), np.float32)
        _check(self._lib.ewf_batch_get_field(self._h, prob, rhs, fid, _ptr(out), out.size, 4), "ewf_batch_get_field")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.ewf_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
