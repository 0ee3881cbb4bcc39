"""Constants of the C ABI (include/ewfd.h) and the reference's array geometry.

Field extents follow the reference's allocations (FastWaveED_GPU3D_v1.cu:431-439 for the state,
FastWaveED_GPU3D_v1_9kmst_ANISO.cu:411-456 for the orthorhombic model arrays); numpy arrays use
shape (ez, ey, ex) in C order, i.e. x fastest as in the reference.
"""
from __future__ import annotations

import numpy as np

# ewf_model / ewf_precision / ewf_damping / ewf_src_order
MODEL_ISO, MODEL_ORTHO, MODEL_ISO_HET = 0, 1, 2
PREC_F32, PREC_F32_KAHAN, PREC_F64 = 0, 1, 2
STEP_SPLIT, STEP_FUSED, STEP_WAVE = 0, 1, 2   # ewf_params.fused: the step form
ONEPASS_TILE, ONEPASS_BAND4, ONEPASS_BAND8, ONEPASS_STAGED = 0, 1, 2, 3  # ewf_set_onepass: the one-pass kernel
DAMP_PML1D, DAMP_W3D, DAMP_SEPARABLE, DAMP_PERCOMP = 0, 1, 2, 3
SRC_BEFORE_BC1, SRC_AFTER_BC1 = 0, 1
FS_BC1, FS_NONE = 0, 1   # ewf_params.free_surface

# state fields
F_VX, F_VY, F_VZ, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ = range(9)
STATE = tuple(range(9))
STATE_NAMES = ("Vx", "Vy", "Vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")
# materials
M_C11, M_C12, M_C22, M_C33, M_C13, M_C23 = 16, 17, 18, 19, 20, 21
M_C66XY, M_C55XZ, M_C44YZ, M_BX, M_BY, M_BZ = 22, 23, 24, 25, 26, 27
ISO_MATERIALS = (M_C11, M_C12)
ORTHO_MATERIALS = (M_C11, M_C22, M_C33, M_C12, M_C13, M_C23, M_C66XY, M_C55XZ, M_C44YZ, M_BX, M_BY, M_BZ)
# the 9 km station scheme: c11u_het, c12u_het, c44u_het xy/xz/yz (edge shear moduli), staggered 1/rho
ISOHET_MATERIALS = (M_C11, M_C12, M_C66XY, M_C55XZ, M_C44YZ, M_BX, M_BY, M_BZ)
# 16 km station scheme's linear velocity damping factor, (float)2.2 * (float)4.6729e-04 in float
# (FastWaveED_GPU3D_v1_16kmst.cu:337-349)
VDAMP_16KM = float(np.float32(np.float32(2.2) * np.float32(4.6729e-04)))
# damping
D_WX, D_WY, D_WZ, D_W3D = 32, 33, 34, 35
# per-component weights (DC_Earthquake solver): Vx/sxx, Vy/syy, Vz/szz, sxy, sxz, syz layouts
D_PX, D_PY, D_PZ, D_PXY, D_PXZ, D_PYZ = 36, 37, 38, 39, 40, 41
PERCOMP_WEIGHTS = (D_PX, D_PY, D_PZ, D_PXY, D_PXZ, D_PYZ)

# status codes
STATUS = {
    0: "EWF_OK", -1: "EWF_ERR_ARG", -2: "EWF_ERR_CUDA", -3: "EWF_ERR_NOMEM", -4: "EWF_ERR_IO",
    -5: "EWF_ERR_STATE", -6: "EWF_ERR_CFL", -7: "EWF_ERR_NONFINITE", -8: "EWF_ERR_UNSUPPORTED",
    -9: "EWF_ERR_NODEVICE",
}

# legacy file names per model (iso, ortho, iso-het): FastWaveED_GPU3D_v1.cu:415-425,
# FastWaveED_GPU3D_v1_9kmst_ANISO.cu:411-456, FastWaveED_GPU3D_v1_9kmst.cu:434-452
LEGACY_FILES = {
    M_C11: ("c11u_het.dat", "C11m.dat", "c11u_het.dat"), M_C12: ("c12u_het.dat", "C12m.dat", "c12u_het.dat"),
    M_C22: (None, "C22m.dat", None), M_C33: (None, "C33m.dat", None), M_C13: (None, "C13m.dat", None),
    M_C23: (None, "C23m.dat", None),
    M_C66XY: (None, "C66mxy.dat", "c44u_hetxy.dat"), M_C55XZ: (None, "C55mxz.dat", "c44u_hetxz.dat"),
    M_C44YZ: (None, "C44myz.dat", "c44u_hetyz.dat"),
    M_BX: (None, "vrho_x_11_hc.dat", "vrho_x_11_hc.dat"), M_BY: (None, "vrho_y_11_hc.dat", "vrho_y_11_hc.dat"),
    M_BZ: (None, "vrho_z_11_hc.dat", "vrho_z_11_hc.dat"),
    D_WX: ("weights_x.dat", None, None), D_WY: ("weights_y.dat", None, None), D_WZ: ("weights_z.dat", None, None),
    D_W3D: (None, "weights.dat", "weights.dat"),
    D_PX: ("weights_x.dat", None, None), D_PY: ("weights_y.dat", None, None), D_PZ: ("weights_z.dat", None, None),
    D_PXY: ("weights_xy.dat", None, None), D_PXZ: ("weights_xz.dat", None, None), D_PYZ: ("weights_yz.dat", None, None),
}


def extent(fid: int, nx: int, ny: int, nz: int, damping: int = DAMP_PML1D) -> tuple[int, int, int]:
    """(ex, ey, ez) of a field id in the reference layout."""
    x, y, z = nx, ny, nz
    if fid in (F_VX, M_BX):
        x = nx + 1
    elif fid in (F_VY, M_BY):
        y = ny + 1
    elif fid in (F_VZ, M_BZ):
        z = nz + 1
    elif fid in (F_SXY, M_C66XY):
        x, y = nx + 1, ny + 1
    elif fid in (F_SXZ, M_C55XZ):
        x, z = nx + 1, nz + 1
    elif fid in (F_SYZ, M_C44YZ):
        y, z = ny + 1, nz + 1
    elif fid in (D_WX, D_WY, D_WZ):
        n = (nx, ny, nz)[fid - D_WX] + (1 if damping == DAMP_PML1D else 0)
        return n, 1, 1
    elif fid in PERCOMP_WEIGHTS:  # the layout of the component each weights
        return extent((F_VX, F_VY, F_VZ, F_SXY, F_SXZ, F_SYZ)[fid - D_PX], nx, ny, nz)
    return x, y, z


def shape(fid: int, nx: int, ny: int, nz: int, damping: int = DAMP_PML1D) -> tuple:
    ex, ey, ez = extent(fid, nx, ny, nz, damping)
    if fid in (D_WX, D_WY, D_WZ):
        return (ex,)
    return (ez, ey, ex)


def mt_entries(mt, xs: int, ys: int, zs: int, stencil: int) -> tuple[np.ndarray, np.ndarray]:
    """Point-source entries (comp, i, j, k) and coefficients of a moment tensor
    (xx, yy, zz, xy, xz, yz) at the reference's injection stencil around (xs, ys, zs).

    stencil 0 (FastWaveED_GPU3D_v1.cu:336-342): normals at (xs+1, ys+1, zs+1), yz at
    (xs+2, ys+2), xz and xy at (xs+3, ys+3); stencil 1 (FastWaveED_GPU3D_v1_9kmst_ANISO.cu:233-247):
    normals at (xs+1, ys+1), xy at (xs+2, ys+2), yz at (xs+3, ys+2), xz at (xs-1, ys+1); all at
    zs+1.  Order of the entries is the reference's statement order."""
    xx, yy, zz, xy, xz, yz = (float(v) for v in mt)
    if stencil == 0:
        e = [(F_SXX, 1, 1, xx), (F_SYY, 1, 1, yy), (F_SZZ, 1, 1, zz), (F_SYZ, 2, 2, yz), (F_SXZ, 3, 3, xz),
             (F_SXY, 3, 3, xy)]
    elif stencil == 1:
        e = [(F_SXX, 1, 1, xx), (F_SYY, 1, 1, yy), (F_SZZ, 1, 1, zz), (F_SXY, 2, 2, xy), (F_SYZ, 3, 2, yz),
             (F_SXZ, -1, 1, xz)]
    else:
        raise ValueError("stencil must be 0 or 1")
    ent = np.array([(c, xs + di, ys + dj, zs + 1) for c, di, dj, _ in e], dtype=np.int32)
    coef = np.array([v for *_, v in e], dtype=np.float64)
    return ent, coef


def mt_point_entries(mt, i: int, j: int, k: int) -> tuple[np.ndarray, np.ndarray]:
    """Entries of a moment tensor (xx, yy, zz, xy, xz, yz) as one point source at the centre of
    cell (i, j, k): the normal components there, each shear component split equally over the four
    edges around the centre (sxy[j', i'] sits at (i' - 1/2, j' - 1/2), so the edges are
    i' in {i, i+1}, j' in {j, j+1}; likewise sxz and syz).  Zero components are left out.  Unlike
    the reference's stencils above, every component acts at the same point, which keeps the
    radiation of a laterally homogeneous model symmetric about the source."""
    xx, yy, zz, xy, xz, yz = (float(v) for v in mt)
    e = [(F_SXX, i, j, k, xx), (F_SYY, i, j, k, yy), (F_SZZ, i, j, k, zz)]
    for a in (0, 1):
        for b in (0, 1):
            e += [(F_SXY, i + a, j + b, k, 0.25 * xy), (F_SXZ, i + a, j, k + b, 0.25 * xz),
                  (F_SYZ, i, j + a, k + b, 0.25 * yz)]
    e = [t for t in e if t[4] != 0.0]
    ent = np.array([t[:4] for t in e], dtype=np.int32).reshape(-1, 4)
    coef = np.array([t[4] for t in e], dtype=np.float64)
    return ent, coef


# the orthorhombic reference hard-codes its tensor (FastWaveED_GPU3D_v1_9kmst_ANISO.cu:233-247)
ANISO_LEGACY_MT = tuple(float(np.float32(v)) for v in (-0.6282, 0.9437, 0.2439, 0.4455, -0.2709, -0.2362))
# the 16 km station solver hard-codes another tensor in the same kernel and stencil
# (FastWaveED_GPU3D_v1_16kmst.cu:228-252)
ISO16KM_LEGACY_MT = tuple(float(np.float32(v)) for v in (-0.7448, 1.0603, 0.2439, -0.0387, -0.1953, -0.3017))
# the DC_Earthquake solver's source kernel injects only xz (1.0) and yz (0.8) at the ANISO stencil
# cells (src/FastWaveED_GPU3D_v1_DC_Earthquake/FastWaveED_GPU3D_v1.cu:228-246)
DCQ_LEGACY_MT = (0.0, 0.0, 0.0, 0.0, 1.0, float(np.float32(0.8)))
# the four legacy traces Rec, Rec_x, Rec_y, Rec_y2 (FastWaveED_GPU3D_v1.cu:383-386; ANISO:263-266)
OK4_LEGACY_RECEIVERS = ((504, 385, 1, F_VZ), (504, 385, 1, F_VX), (504, 388, 1, F_VY), (504, 387, 1, F_VY))
ANISO_LEGACY_RECEIVERS = ((631, 257, 1, F_VZ), (631, 257, 1, F_VX), (631, 257, 1, F_VY), (631, 257, 1, F_VY))
