"""Replays the reference's time loop with the reference's own kernels (TEST INFRASTRUCTURE ONLY).

The kernels come from oracle/_ref/*.cubin, compiled unmodified from the reference sources by
oracle/build.py; oracle/refkernels.c loads a cubin and launches by name.  This module owns the
host side the reference's main() would have (FastWaveED_GPU3D_v1.cu:390-559,
FastWaveED_GPU3D_v1_9kmst_ANISO.cu:391-608): allocation, the launch geometry
(block (32,2,8), grid covering 64*NB cells per axis, :26-31, 88-89), and the loop order
  isotropic:     compute_StressPrf, BC1, update_Qxft                    (OK4:485-505)
  orthorhombic:  compute_StressOrtho, BC1, source, update_VelocityFromStress (ANISO:519-555)
  9 km / 16 km:  compute_StressPrf, BC1, source, update_Qxft            (9kmst.cu:463-477)
  DC_Earthquake: compute_StressPrf, BC1, source, update_Qxft            (FastWaveED_GPU3D_v1.cu:473-483)
  diff_BC2_OK3, diff_BC_OK2: compute_StressPrf (source inside), update_Qxft -- no BC1 (:473-483, :450-460)
  FULL:          compute_StressPrf, BC1, source, update_Qxft            (FastBiot_GPU3D_v1.cu:441-451)
with our receivers gathered from V after each step (a read-only gather; the reference's own
hard-coded `record` cells are left as they are).

Allocation differs from the reference in one way: every array carries a zeroed guard of one
plane on both sides.  The isotropic stress kernel reads Vx/Vy/Vz at i-1, j-1 and k-1 with no
guard (FastWaveED_GPU3D_v1.cu:323-329); at the grid's low edges those reads fall up to one plane
before the array (e.g. Vy[ix-1 + ...] = Vy[-1] at the origin).  In the reference run they read
whatever memory precedes the allocation; here they read the guard, so no access leaves an
allocation.  The values only reach shear-stress cells the velocity update never reads back.

Requires torch with CUDA (device memory) and the built librefkernels.so.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from elanfmt_gb300 import fields as F
from elanfmt_gb300.inputs import separable_weights

HERE = os.path.dirname(os.path.abspath(__file__))
REFK = os.path.join(HERE, "librefkernels.so")

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        from . import build as _build

        _build.build_refkernels()
        L = C.CDLL(REFK)
        L.refk_error.restype = C.c_char_p
        L.refk_init.argtypes = [C.c_int]
        L.refk_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        L.refk_unload.argtypes = [C.c_void_p]
        L.refk_function.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]
        L.refk_launch.argtypes = [C.c_void_p] + [C.c_uint] * 6 + [C.c_void_p]
        _lib = L
    return _lib


def _ck(st: int, what: str) -> None:
    if st != 0:
        raise RuntimeError(f"{what}: {lib().refk_error().decode(errors='replace')}")


# reference schemes selected by Model.meta["scheme"] rather than by model and damping alone
SCHEMES = ("ok3", "ok2", "full")


def cubin(model: int, variant: str, vdamp: float = 0.0, damping: int = -1, scheme: str | None = None) -> str:
    if scheme in SCHEMES:
        name = scheme
    elif model == F.MODEL_ISO and damping == F.DAMP_PERCOMP:
        name = "dcq"
    else:
        name = {F.MODEL_ISO: "ok4", F.MODEL_ORTHO: "aniso"}.get(model, "iso16km" if vdamp else "iso9km")
    return os.path.join(HERE, "_ref", f"{name}_{variant}.cubin")


def available(model: int = F.MODEL_ISO, variant: str = "exact", vdamp: float = 0.0, damping: int = -1,
              scheme: str | None = None) -> bool:
    return os.path.exists(cubin(model, variant, vdamp, damping, scheme))


def trace_errors(ours: np.ndarray, ref: np.ndarray) -> dict:
    """Relative L2 error of each trace of `ours` against `ref` (traces x samples).  Traces whose
    reference is identically zero are counted apart: `ours` must be zero there too."""
    ours = np.asarray(ours, np.float64)
    ref = np.asarray(ref, np.float64)
    assert ours.shape == ref.shape, (ours.shape, ref.shape)
    rel, zero_mismatch = [], 0
    for a, b in zip(ours, ref):
        nb = float(np.linalg.norm(b))
        if nb == 0.0:
            zero_mismatch += int(np.linalg.norm(a) != 0.0)
            continue
        rel.append(float(np.linalg.norm(a - b)) / nb)
    rel = np.array(rel) if rel else np.zeros(1)
    return {"max_rel_l2": float(rel.max()), "median_rel_l2": float(np.median(rel)),
            "p90_rel_l2": float(np.percentile(rel, 90)), "traces": int(len(ref)), "zero_mismatch": zero_mismatch}


class _Args:
    """Kernel argument vector: ('p', ptr) | ('f', float32) | ('i', int32)."""

    def __init__(self, spec):
        self.objs = []
        for kind, v in spec:
            if kind == "p":
                self.objs.append(C.c_void_p(int(v)))
            elif kind == "f":
                self.objs.append(C.c_float(float(v)))
            else:
                self.objs.append(C.c_int32(int(v)))
        self.argv = (C.c_void_p * len(self.objs))(*[C.cast(C.pointer(o), C.c_void_p) for o in self.objs])

    def set_int(self, pos: int, v: int) -> None:
        self.objs[pos].value = int(v)


class RefRunner:
    """Reference kernels on one Model (iso: OK4 stencil + before-BC1 order; ortho: the ANISO
    stencil with ANISO's built-in tensor, after-BC1 order, 3-D weights)."""

    def __init__(self, m, variant: str = "exact", device: int = 0):
        import torch

        self.torch = torch
        self.m = m
        self.dev = torch.device("cuda", device)
        torch.cuda.init()
        torch.zeros(1, device=self.dev)
        _ck(lib().refk_init(device), "refk_init")
        mod = C.c_void_p()
        self.scheme = (getattr(m, "meta", None) or {}).get("scheme")
        _ck(lib().refk_load(os.fsencode(cubin(m.model, variant, getattr(m, "vdamp", 0.0), m.damping, self.scheme)),
                            C.byref(mod)), "refk_load")
        self.mod = mod
        nx, ny, nz = m.nx, m.ny, m.nz
        self.pad = (nx + 2) * (ny + 2) + 64
        self._bufs = []
        self.nbx = math.ceil(nx / 64)
        self.nby = math.ceil(ny / 64)
        self.nbz = math.ceil(nz / 64)
        if nx > ny and 64 * self.nby > ny:
            raise ValueError("reference BC1 with nx > ny writes past row ny (a race): use nx <= ny or ny % 64 == 0")
        self.grid = (2 * self.nbx, 32 * self.nby, 8 * self.nbz)
        self.block = (32, 2, 8)
        self.f = [self._alloc(F.shape(q, nx, ny, nz)) for q in F.STATE]
        self.dummy = self._alloc((1024,))
        self.rec_dummy = [self._alloc((m.nt,)) for _ in range(4)]
        self.src = self._upload(np.asarray(m.stf[: m.nt], np.float32)) if m.stf is not None else self._alloc((m.nt,))
        nrec = 0 if m.receivers is None else len(m.receivers)
        self.traces = np.zeros((nrec, m.nt), np.float64)
        # receivers grouped by field: one index_select per field and step into a device trace
        # buffer, copied to the host when a run() ends
        self._dtraces = torch.zeros((nrec, m.nt), dtype=torch.float64, device=self.dev) if nrec else None
        self._rec_groups = []
        if nrec:
            by_comp = {}
            for r, (i, j, k, c) in enumerate(m.receivers):
                ez, ey, ex = F.shape(int(c), nx, ny, nz)
                by_comp.setdefault(int(c), []).append((r, int(i) + ex * (int(j) + ey * int(k))))
            for c, lst in sorted(by_comp.items()):
                rows = torch.tensor([r for r, _ in lst], device=self.dev)
                offs = torch.tensor([o for _, o in lst], device=self.dev)
                self._rec_groups.append((c, rows, offs))
        self.it = 0
        self._setup_kernels()

    # -- memory ---------------------------------------------------------------------------------
    def _alloc(self, shape):
        n = int(np.prod(shape))
        t = self.torch.zeros(n + 2 * self.pad, dtype=self.torch.float32, device=self.dev)
        self._bufs.append(t)
        view = t[self.pad: self.pad + n]
        return view

    def _upload(self, arr):
        a = np.ascontiguousarray(arr, np.float32).ravel()
        v = self._alloc(a.shape)
        v.copy_(self.torch.from_numpy(a))
        return v

    @staticmethod
    def _p(t) -> int:
        return t.data_ptr()

    def _fn(self, prefix: str):
        f = C.c_void_p()
        _ck(lib().refk_function(self.mod, prefix.encode(), C.byref(f)), prefix)
        return f

    # -- kernels --------------------------------------------------------------------------------
    def _check_sources(self, stencil: int):
        m = self.m
        if m.sources is None or len(m.sources) == 0:
            raise ValueError("the reference kernels always inject: the model needs a source")
        ent = np.asarray(m.sources)
        xs, ys, zs = int(ent[0, 1]) - 1, int(ent[0, 2]) - 1, int(ent[0, 3]) - 1
        want, coef = F.mt_entries(np.zeros(6), xs, ys, zs, stencil)
        if not np.array_equal(want, ent):
            raise ValueError("sources must be the reference's moment-tensor stencil")
        return xs, ys, zs

    def _setup_kernels(self):
        m = self.m
        P = self._p
        f = self.f
        nx, ny, nz = m.nx, m.ny, m.nz
        d = self.dummy
        self.bc1 = True
        if self.scheme in SCHEMES:
            self._setup_diff_bc()
        elif m.model == F.MODEL_ISO and m.damping == F.DAMP_PERCOMP:
            if m.src_order != F.SRC_AFTER_BC1:
                raise ValueError("DC_Earthquake reference = after-BC1 injection")
            xs, ys, zs = self._check_sources(1)
            coef = tuple(float(np.float32(v)) for v in self._mt_tuple())
            if coef != F.DCQ_LEGACY_MT:
                raise ValueError("the DC_Earthquake reference hard-codes its source: use fields.DCQ_LEGACY_MT")
            c11 = self._upload(m.materials[F.M_C11])
            c12 = self._upload(m.materials[F.M_C12])
            # every weight field at its full extent (its driver writes them so), which keeps the
            # kernels' edge-pitch reads of the shear weights inside the arrays
            wx, wy, wz, wxy, wxz, wyz = (self._upload(m.damping_arrays[k]) for k in F.PERCOMP_WEIGHTS)
            # compute_StressPrf(Prf, 6 stresses, Vx, Vy, Vz, Qxft, Qyft, Qzft, c11u_het, c12u_het,
            # weights_x/y/z/xy/xz/yz, dx, dy, dz, dt, c11u c22u c33u c12u c13u c23u c44u c55u c66u,
            # alpha1-3, M1, nx, ny, nz) (FastWaveED_GPU3D_v1.cu:298)
            self.k_stress = self._fn("_Z17compute_StressPrf")
            self.a_stress = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 3
                + [("p", P(x)) for x in (c11, c12, wx, wy, wz, wxy, wxz, wyz)]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 6
                + [("f", m.c44), ("f", m.c55), ("f", m.c66)] + [("f", 0.0)] * 4
                + [("i", nx), ("i", ny), ("i", nz)])
            self.it_pos_stress = None
            self.k_src = self._fn("_Z6source")
            self.a_src = _Args(
                [("p", P(d))] * 4 + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1)] + [("p", P(d))] * 2
                + [("p", P(self.src))] + [("f", m.dx), ("f", m.dy), ("f", m.dz)] + [("f", 0.0)] * 6
                + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", xs), ("i", ys), ("i", zs), ("i", 2)]
                + [("f", m.dt)])
            self.it_pos_src = 15 + 9 + 3
            # update_Qxft(Prf, 6 stresses, Vx, Vy, Vz, Qxft..Qzold (6), vrhox11het, weights_x/y/z,
            # dx, dy, dz, dt, eta_k1-3, vrho_x/y/z_11, 6 unused, nx, ny, nz, chi) (:328)
            self.k_vel = self._fn("_Z11update_Qxft")
            self.a_vel = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 7
                + [("p", P(x)) for x in (wx, wy, wz)]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 3
                + [("f", m.bx), ("f", m.by), ("f", m.bz)] + [("f", 0.0)] * 6
                + [("i", nx), ("i", ny), ("i", nz), ("f", 0.5)])
            self.it_pos_vel = None
        elif m.model == F.MODEL_ISO:
            if m.src_order != F.SRC_BEFORE_BC1 or m.damping != F.DAMP_PML1D:
                raise ValueError("isotropic reference = before-BC1 injection and 1-D PML")
            xs, ys, zs = self._check_sources(0)
            mt = {int(c): float(v) for (c, *_), v in zip(m.sources, m.source_coef)}
            c11 = self._upload(m.materials[F.M_C11])
            c12 = self._upload(m.materials[F.M_C12])
            wx, wy, wz = (self._upload(m.damping_arrays[k]) for k in (F.D_WX, F.D_WY, F.D_WZ))
            R = self.rec_dummy
            self.k_stress = self._fn("_Z17compute_StressPrf")
            self.a_stress = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 3
                + [("p", P(c11)), ("p", P(c12)), ("p", P(wx)), ("p", P(wy)), ("p", P(wz))]
                + [("p", P(r)) for r in R] + [("p", P(self.src))]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 8 + [("f", m.c66)]
                + [("f", 0.0)] * 4
                + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", xs), ("i", ys), ("i", zs), ("i", 2)]
                + [("f", mt[F.F_SXX]), ("f", mt[F.F_SYY]), ("f", mt[F.F_SZZ]), ("f", mt[F.F_SXY]),
                   ("f", mt[F.F_SXZ]), ("f", mt[F.F_SYZ])])
            self.it_pos_stress = 23 + 17 + 3
            self.k_vel = self._fn("_Z11update_Qxft")
            self.a_vel = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 7
                + [("p", P(wx)), ("p", P(wy)), ("p", P(wz))] + [("p", P(r)) for r in R]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt), ("f", 0.0), ("f", 0.0), ("f", 0.0),
                   ("f", m.bx), ("f", m.by), ("f", m.bz)] + [("f", 0.0)] * 6
                + [("i", nx), ("i", ny), ("i", nz), ("f", 0.5), ("i", 0)])
            self.it_pos_vel = 24 + 16 + 3 + 1
            self.k_src = None
        elif m.model == F.MODEL_ISO_HET:
            if m.src_order != F.SRC_AFTER_BC1:
                raise ValueError("9 km / 16 km reference = after-BC1 injection")
            xs, ys, zs = self._check_sources(1)
            vd = getattr(m, "vdamp", 0.0)
            if vd and vd != F.VDAMP_16KM:
                raise ValueError("the 16 km reference hard-codes its damping: use fields.VDAMP_16KM")
            coef = tuple(float(np.float32(v)) for v in self._mt_tuple())
            if coef != (F.ISO16KM_LEGACY_MT if vd else F.ANISO_LEGACY_MT):
                raise ValueError("the 9 km / 16 km references hard-code their tensors")
            c11, c12, mxy, mxz, myz, BX, BY, BZ = (self._upload(m.materials[k]) for k in F.ISOHET_MATERIALS)
            if F.D_W3D in m.damping_arrays:
                W = self._upload(m.damping_arrays[F.D_W3D])
            else:
                W = self._upload(separable_weights(m.damping_arrays[F.D_WX], m.damping_arrays[F.D_WY],
                                                   m.damping_arrays[F.D_WZ]))
            # compute_StressPrf(Prf, 6 stresses, Vx, Vy, Vz, Qxft, Qyft, Qzft, c11u_het, c12u_het,
            # c44u_hetxy/xz/yz, weights, dx, dy, dz, dt, 13 unused scalars, nx, ny, nz) (9kmst.cu:287)
            self.k_stress = self._fn("_Z17compute_StressPrf")
            self.a_stress = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 3
                + [("p", P(x)) for x in (c11, c12, mxy, mxz, myz, W)]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 13
                + [("i", nx), ("i", ny), ("i", nz)])
            self.it_pos_stress = None
            self.k_src = self._fn("_Z6source")
            self.a_src = _Args(
                [("p", P(d))] * 4 + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1)] + [("p", P(d))] * 2
                + [("p", P(self.src))] + [("f", m.dx), ("f", m.dy), ("f", m.dz)] + [("f", 0.0)] * 6
                + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", xs), ("i", ys), ("i", zs), ("i", 2)]
                + [("f", m.dt)])
            self.it_pos_src = 15 + 9 + 3
            # update_Qxft(Prf, 6 stresses, Vx, Vy, Vz, Qxft..Qzold (6), vrho x/y/z, weights, dx, dy,
            # dz, dt, 12 unused scalars, nx, ny, nz, chi) (9kmst.cu:333)
            self.k_vel = self._fn("_Z11update_Qxft")
            self.a_vel = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 6
                + [("p", P(x)) for x in (BX, BY, BZ, W)]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 12
                + [("i", nx), ("i", ny), ("i", nz), ("f", 0.5)])
            self.it_pos_vel = None
        else:
            if m.src_order != F.SRC_AFTER_BC1:
                raise ValueError("orthorhombic reference = after-BC1 injection")
            xs, ys, zs = self._check_sources(1)
            coef = tuple(float(np.float32(v)) for v in self._mt_tuple())
            if coef != F.ANISO_LEGACY_MT:
                raise ValueError("the orthorhombic reference hard-codes its tensor: use fields.ANISO_LEGACY_MT")
            mats = [self._upload(m.materials[k]) for k in F.ORTHO_MATERIALS]
            if F.D_W3D in m.damping_arrays:
                W = self._upload(m.damping_arrays[F.D_W3D])
            else:
                W = self._upload(separable_weights(m.damping_arrays[F.D_WX], m.damping_arrays[F.D_WY],
                                                   m.damping_arrays[F.D_WZ]))
            C11, C22, C33, C12, C13, C23, C66, C55, C44, BX, BY, BZ = mats
            self.k_stress = self._fn("_Z19compute_StressOrtho")
            self.a_stress = _Args(
                [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)]
                + [("p", P(x)) for x in (C11, C22, C33, C12, C13, C23, C66, C55, C44, W)]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt), ("i", nx), ("i", ny), ("i", nz)])
            self.it_pos_stress = None
            self.k_src = self._fn("_Z6source")
            self.a_src = _Args(
                [("p", P(d))] * 4 + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1)] + [("p", P(d))] * 2
                + [("p", P(self.src))] + [("f", m.dx), ("f", m.dy), ("f", m.dz)] + [("f", 0.0)] * 6
                + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", xs), ("i", ys), ("i", zs), ("i", 2)]
                + [("f", m.dt)])
            self.it_pos_src = 15 + 9 + 3
            self.k_vel = self._fn("_Z25update_VelocityFromStress")
            self.a_vel = _Args(
                [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(x)) for x in (BX, BY, BZ, W)]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt), ("i", nx), ("i", ny), ("i", nz)])
            self.it_pos_vel = None
        self.k_bc1 = self._fn("_Z3BC1")
        self.a_bc1 = _Args(
            [("p", P(d))] * 4 + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 2
            + [("p", P(self.rec_dummy[0]))] + [("f", m.dx), ("f", m.dy), ("f", m.dz)] + [("f", 0.0)] * 6
            + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", 0), ("i", 0), ("i", 0), ("i", 2)] + [("f", m.dt)])
        self.it_pos_bc1 = 16 + 9 + 3

    def _setup_diff_bc(self):
        """The isotropic variants of the DC_Earthquake FULL family: their sources are built in
        (sigma_yz += 0.8 Src at (xs+2, ys+2, zs+1), sigma_xz += 1.0 Src at (xs+3, ys+3, zs+1))."""
        m, P, f, d = self.m, self._p, self.f, self.dummy
        nx, ny, nz = m.nx, m.ny, m.nz
        xs, ys, zs = self._check_sources(0)
        coef = tuple(float(np.float32(v)) for v in self._mt_tuple())
        if coef != (0.0, 0.0, 0.0, 0.0, 1.0, float(np.float32(0.8))):
            raise ValueError("the diff_BC / FULL references hard-code their source: xz 1.0, yz 0.8")
        c11 = self._upload(m.materials[F.M_C11])
        c12 = self._upload(m.materials[F.M_C12])
        it_src = []
        if self.scheme == "ok3":
            # OK4's kernels without the tensor arguments; no BC1 launch (FastWaveED_GPU3D_v1.cu:473-483)
            if m.model != F.MODEL_ISO or m.damping != F.DAMP_PML1D:
                raise ValueError("the diff_BC2_OK3 reference: isotropic model, 1-D PML")
            wx, wy, wz = (self._upload(m.damping_arrays[k]) for k in (F.D_WX, F.D_WY, F.D_WZ))
            R = self.rec_dummy
            self.k_stress = self._fn("_Z17compute_StressPrf")
            self.a_stress = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 3
                + [("p", P(c11)), ("p", P(c12)), ("p", P(wx)), ("p", P(wy)), ("p", P(wz))]
                + [("p", P(r)) for r in R] + [("p", P(self.src))]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 8 + [("f", m.c66)]
                + [("f", 0.0)] * 4 + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", xs), ("i", ys), ("i", zs), ("i", 2)])
            self.it_pos_stress = 23 + 17 + 3
            self.k_vel = self._fn("_Z11update_Qxft")
            self.a_vel = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 7
                + [("p", P(wx)), ("p", P(wy)), ("p", P(wz))] + [("p", P(r)) for r in R]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt), ("f", 0.0), ("f", 0.0), ("f", 0.0),
                   ("f", m.bx), ("f", m.by), ("f", m.bz)] + [("f", 0.0)] * 6
                + [("i", nx), ("i", ny), ("i", nz), ("f", 0.5), ("i", 0)])
            self.it_pos_vel = 24 + 16 + 3 + 1
            self.k_src = None
            self.bc1 = False
            return
        # ok2 / full: c11/c12 cell fields, one 3-D weight field, scalar shear moduli and buoyancy
        # (the product's 9 km scheme with constant edge-modulus and buoyancy fields)
        if m.model != F.MODEL_ISO_HET or F.D_W3D not in m.damping_arrays:
            raise ValueError("the diff_BC_OK2 / FULL references: the 9 km scheme's form with 3-D weights")
        W = self._upload(m.damping_arrays[F.D_W3D])
        c44, c55, c66 = (float(np.asarray(m.materials[k]).flat[-1]) for k in (F.M_C44YZ, F.M_C55XZ, F.M_C66XY))
        bx, by, bz = (float(np.asarray(m.materials[k]).flat[-1]) for k in (F.M_BX, F.M_BY, F.M_BZ))
        R = self.rec_dummy
        if self.scheme == "ok2":
            # compute_StressPrf(Prf, 6 stresses, Vx, Vy, Vz, Qxft..Qzft, c11u_het, c12u_het, weights,
            # Rec x4, Src, dx, dy, dz, dt, c11u..c66u, alpha1-3, M1, nx, ny, nz, it, xsrc, ysrc, zsrc, ds)
            self.k_stress = self._fn("_Z17compute_StressPrf")
            self.a_stress = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 3
                + [("p", P(c11)), ("p", P(c12)), ("p", P(W))] + [("p", P(r)) for r in R] + [("p", P(self.src))]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 6
                + [("f", c44), ("f", c55), ("f", c66)] + [("f", 0.0)] * 4
                + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", xs), ("i", ys), ("i", zs), ("i", 2)])
            self.it_pos_stress = 21 + 17 + 3
            # update_Qxft(Prf, 6 stresses, Vx, Vy, Vz, Qxft..Qzold (6), vrhox11het, weights, Rec x4,
            # dx, dy, dz, dt, eta_k1-3, vrho_x/y/z_11, 6 unused, nx, ny, nz, chi, it)
            self.k_vel = self._fn("_Z11update_Qxft")
            self.a_vel = _Args(
                [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 7
                + [("p", P(W))] + [("p", P(r)) for r in R]
                + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt), ("f", 0.0), ("f", 0.0), ("f", 0.0),
                   ("f", bx), ("f", by), ("f", bz)] + [("f", 0.0)] * 6
                + [("i", nx), ("i", ny), ("i", nz), ("f", 0.5), ("i", 0)])
            self.it_pos_vel = 22 + 16 + 3 + 1
            self.k_src = None
            self.bc1 = False
            return
        # full: compute_StressPrf(Prf, 6 stresses, Vx, Vy, Vz, Qxft..Qzft, c11u_het, c12u_het, weights,
        # dx, dy, dz, dt, c11u..c66u, alpha1-3, M1, nx, ny, nz) (FastBiot_GPU3D_v1.cu:279), then BC1,
        # the source kernel and update_Qxft (:441-451)
        if m.src_order != F.SRC_AFTER_BC1:
            raise ValueError("the FULL reference injects after BC1")
        self.k_stress = self._fn("_Z17compute_StressPrf")
        self.a_stress = _Args(
            [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 3
            + [("p", P(c11)), ("p", P(c12)), ("p", P(W))]
            + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt)] + [("f", 0.0)] * 6
            + [("f", c44), ("f", c55), ("f", c66)] + [("f", 0.0)] * 4 + [("i", nx), ("i", ny), ("i", nz)])
        self.it_pos_stress = None
        self.k_src = self._fn("_Z6source")
        self.a_src = _Args(
            [("p", P(d))] * 4 + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1)] + [("p", P(d))] * 2
            + [("p", P(self.src))] + [("f", m.dx), ("f", m.dy), ("f", m.dz)] + [("f", 0.0)] * 6
            + [("i", nx), ("i", ny), ("i", nz), ("i", 0), ("i", xs), ("i", ys), ("i", zs), ("i", 2)]
            + [("f", m.dt)])
        self.it_pos_src = 15 + 9 + 3
        self.k_vel = self._fn("_Z11update_Qxft")
        self.a_vel = _Args(
            [("p", P(d))] + [("p", P(f[q])) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)] + [("p", P(d))] * 7
            + [("p", P(W))]
            + [("f", m.dx), ("f", m.dy), ("f", m.dz), ("f", m.dt), ("f", 0.0), ("f", 0.0), ("f", 0.0),
               ("f", bx), ("f", by), ("f", bz)] + [("f", 0.0)] * 6
            + [("i", nx), ("i", ny), ("i", nz), ("f", 0.5)])
        self.it_pos_vel = None

    def _mt_tuple(self):
        mt = {int(c): float(v) for (c, *_), v in zip(self.m.sources, self.m.source_coef)}
        return (mt[F.F_SXX], mt[F.F_SYY], mt[F.F_SZZ], mt[F.F_SXY], mt[F.F_SXZ], mt[F.F_SYZ])

    def _launch(self, fn, args):
        _ck(lib().refk_launch(fn, *self.grid, *self.block, args.argv), "launch")

    def run(self, nsteps: int) -> None:
        torch = self.torch
        for _ in range(nsteps):
            it = self.it
            if self.it_pos_stress is not None:
                self.a_stress.set_int(self.it_pos_stress, it)
            self._launch(self.k_stress, self.a_stress)
            if self.bc1:
                self.a_bc1.set_int(self.it_pos_bc1, it)
                self._launch(self.k_bc1, self.a_bc1)
            if self.k_src is not None:
                self.a_src.set_int(self.it_pos_src, it)
                self._launch(self.k_src, self.a_src)
            if self.it_pos_vel is not None:
                self.a_vel.set_int(self.it_pos_vel, it)
            self._launch(self.k_vel, self.a_vel)
            _ck(lib().refk_sync(), "sync")
            for c, rows, offs in self._rec_groups:
                self._dtraces[rows, it] = self.f[c].index_select(0, offs).double()
            self.it += 1
        torch.cuda.synchronize()
        if self._dtraces is not None:
            self.traces = self._dtraces.cpu().numpy()

    def fields(self) -> list[np.ndarray]:
        m = self.m
        return [self.f[q].cpu().numpy().reshape(F.shape(q, m.nx, m.ny, m.nz)) for q in F.STATE]

    def close(self):
        if self.mod:
            lib().refk_unload(self.mod)
            self.mod = None
        self._bufs.clear()
