"""The reference's file contract in numpy: write the MATLAB drivers' input files for a Model and
read back the solver's outputs.

Inputs (vizme_FastBiotED_GPU3D_OK_2024_final.m:348-429 / vizme_FastWaveED_GPU3D_9kmst_ANIS.m:
378-533): raw float32, no header, x fastest.  pa1 = [dx dy dz dt Lx Ly Lz lamx lamy lamz],
pa2 = [c11u c33u c13u c12u c23u c44u c55u c66u alpha1 alpha2 alpha3 M1 c22u], pa3 =
[vrho_x_11 vrho_y_11 vrho_z_11 vrho_x_12 ... eta_k3] (12 values), MTS = [xx yy zz xy xz yz],
Src = nt samples, plus the model arrays.  Outputs (FastWaveED_GPU3D_v1.cu:154-164, 521-532):
0_infos.inf = "PRECIS nx ny nz NB_PARAMS NB_EVOL" and 0_0_<name>.res raw arrays.
"""
from __future__ import annotations

import os

import numpy as np

from . import fields as F


def _w(path: str, a) -> None:
    np.ascontiguousarray(a, dtype=np.float32).tofile(path)


def write_inputs(m, workdir: str) -> None:
    """Writes the legacy input set of Model `m` into workdir."""
    os.makedirs(workdir, exist_ok=True)
    j = lambda name: os.path.join(workdir, name)  # noqa: E731
    Lx, Ly, Lz = (m.nx - 1) * m.dx, (m.ny - 1) * m.dy, (m.nz - 1) * m.dz
    _w(j("pa1.dat"), [m.dx, m.dy, m.dz, m.dt, Lx, Ly, Lz, Lx / 10, Ly / 10, Lz / 10])
    c66 = m.c66
    # pa2 = [c11u c33u c13u c12u c23u c44u c55u c66u ...] (OK4:402, 405)
    _w(j("pa2.dat"), [0, 0, 0, 0, 0, getattr(m, "c44", 0.0), getattr(m, "c55", 0.0), c66, 0, 0, 0, 0, 0])
    _w(j("pa3.dat"), [m.bx, m.by, m.bz] + [0.0] * 9)
    mt = np.zeros(6)
    if m.sources is not None:
        comp_to_slot = {F.F_SXX: 0, F.F_SYY: 1, F.F_SZZ: 2, F.F_SXY: 3, F.F_SXZ: 4, F.F_SYZ: 5}
        for (c, *_), v in zip(m.sources, m.source_coef):
            mt[comp_to_slot[int(c)]] = v
    _w(j("MTS.dat"), mt)
    _w(j("Src.dat"), np.asarray(m.stf[: m.nt]))
    col = int(m.model)
    for fid, arr in list(m.materials.items()) + list(m.damping_arrays.items()):
        name = F.LEGACY_FILES[fid][col]
        if name is None:
            raise ValueError(f"field {fid} has no legacy file for this model")
        _w(j(name), arr)
    if m.model != F.MODEL_ISO and F.D_W3D not in m.damping_arrays:
        from .inputs import separable_weights

        _w(j("weights.dat"), separable_weights(m.damping_arrays[F.D_WX], m.damping_arrays[F.D_WY],
                                               m.damping_arrays[F.D_WZ]))


def read_outputs(workdir: str, nt: int) -> dict:
    """Reads 0_infos.inf and the 0_0_*.res files (vizme_FastBiotED_GPU3D_OK_2024_final.m:457-467)."""
    info = open(os.path.join(workdir, "0_infos.inf")).read().split()
    precis, nx, ny, nz = (int(v) for v in info[:4])
    dt = np.float64 if precis == 8 else np.float32
    out = {"PRECIS": precis, "nx": nx, "ny": ny, "nz": nz, "info": info}
    for name in ("Src", "Rec", "Rec_x", "Rec_y", "Rec_y2"):
        out[name] = np.fromfile(os.path.join(workdir, f"0_0_{name}.res"), dtype=dt)
    for name, fid in (("Vx", F.F_VX), ("Vy", F.F_VY), ("Vz", F.F_VZ)):
        p = os.path.join(workdir, f"0_0_{name}.res")
        if os.path.exists(p):
            out[name] = np.fromfile(p, dtype=dt).reshape(F.shape(fid, nx, ny, nz))
    p = os.path.join(workdir, "0_0_Rec_all.res")
    if os.path.exists(p):
        out["Rec_all"] = np.fromfile(p, dtype=dt).reshape(-1, nt)
    return out
