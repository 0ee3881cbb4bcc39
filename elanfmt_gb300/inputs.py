"""Input generators: the reference's MATLAB input builders restated in numpy, and the synthetic
workloads the solver is measured on.

All 3-D arrays use the reference layout as numpy shape ``(ez, ey, ex)`` in C order (x fastest,
the order MATLAB's ``(:)`` writes).  Material and damping arrays are returned as float32, the
dtype the MATLAB drivers write (``fwrite(..., 'single')``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import fields as F

# ---------------------------------------------------------------------------------------------
# damping
# ---------------------------------------------------------------------------------------------


def pml_weights(n: int, lpml: int, dt: float, R: float = 1e-8, top_override: bool = False,
                sides: str = "both") -> np.ndarray:
    """1-D PML weights of length n+1 (vizme_FastBiotED_GPU3D_OK_2024_final.m:297-341).

    sigma_i = 1.5/(lpml/n) * log10(1/R) * ((lpml - i + 1)/lpml)^2 for i = 1..lpml, and
    w = exp(-sigma_i * dt) at index i and mirrored at n - i + 2 (1-based); 1 elsewhere.
    ``top_override`` applies the driver's ``weights_z(1:fix(nz/2)) = 1`` (no damping at the free
    surface); ``sides`` = "high" keeps only the mirrored (far) end.
    """
    w = np.ones(n + 1, dtype=np.float64)
    for i in range(1, lpml + 1):
        sigma = 3 * 1 / 2 / (lpml / n) * math.log10(1 / R) * ((lpml - i + 1) / lpml) ** 2
        d = math.exp(-sigma * dt)
        if sides in ("both", "low"):
            w[i - 1] = d
        if sides in ("both", "high"):
            w[n - i + 1] = d
    if top_override:
        w[: n // 2] = 1.0
    return w.astype(np.float32)


def sponge_3d_legacy(nx: int, ny: int, nz: int, thick: int = 120, margin_y: int = 210,
                     rate: float = 0.16) -> np.ndarray:
    """3-D sponge ``weights.dat`` (vizme_FastWaveED_GPU3D_9kmst_ANIS.m:466-512).

    w = exp(-(rate/thick)^2 * (i^2 + j^2 + k^2)) with i, k the distances into the x and y
    margins (both sides) and j the distance into the bottom z margin (no top damping).
    """
    ix = np.arange(1, nx + 1)
    iy = np.arange(1, ny + 1)
    iz = np.arange(1, nz + 1)
    di = np.where(ix < thick + 1, thick + 1 - ix, 0)
    di = np.where(nx - thick < ix, ix - nx + thick, di)
    dk = np.where(iy < margin_y + 1, margin_y + 1 - iy, 0)
    dk = np.where(ny - margin_y < iy, iy - ny + margin_y, dk)
    dj = np.where(nz - thick < iz, iz - nz + thick, 0)
    a = rate / thick
    rr = a * a * (di[None, None, :] ** 2 + dk[None, :, None] ** 2 + dj[:, None, None] ** 2).astype(np.float64)
    return np.exp(-rr).astype(np.float32)


def separable_weights(px: np.ndarray, py: np.ndarray, pz: np.ndarray, dtype=np.float32) -> np.ndarray:
    """The 3-D weight field W[k,j,i] = (px[i]*py[j])*pz[k] in `dtype` arithmetic -- bit-identical
    to what the separable-damping kernels of that precision form on the fly."""
    px = np.asarray(px, dtype)
    py = np.asarray(py, dtype)
    pz = np.asarray(pz, dtype)
    pxy = py[:, None] * px[None, :]
    return (pxy[None, :, :] * pz[:, None, None]).astype(dtype)


def pml_factors(n: int, lpml: int, dt: float, R: float = 1e-8, sides: str = "both") -> np.ndarray:
    """Per-axis damping factor of length n for the separable form: the PML formula above with the
    cell i taking the weight of node i (so the profile has n entries)."""
    return pml_weights(n, lpml, dt, R, sides=sides)[:n].copy()


def percomp_weights(nx: int, ny: int, nz: int, dt: float, lpml: int = 110, R: float = 1e-5) -> dict:
    """The DC_Earthquake driver's per-component weights (vizme_FastWaveED_GPU3D.m:293-358), keyed by
    the EWF_D_P* field ids, in the components' layouts.

    sigma_i = 1.5/(lpml/nx) log10(1/R) ((lpml - i + 1)/lpml)^2 on the first lpml cells of every
    axis and mirrored at the far end (the driver uses nx for all three axes); normal weights are
    exp(-sigma dt) on both x and y ends and the bottom z end (free surface on top); the shear
    weights exp(-(sigma_a + sigma_b) dt / 2) are painted by the driver's double loop, whose
    overlapping assignments are replayed here in the same order (1-based MATLAB indices moved to
    0-based; each shear pattern is constant along its third axis)."""
    pw = lpml
    if min(nx, ny, nz) <= 2 * pw + 2:
        raise ValueError(f"grid {nx}x{ny}x{nz} too small for lpml {lpml}")
    i_vec = np.arange(1, pw + 1, dtype=np.float64)
    sigma = 3 * 1 / 2 / (pw / nx) * math.log10(1 / R) * ((pw - i_vec + 1) / pw) ** 2
    px, py, pz = np.zeros(nx), np.zeros(ny), np.zeros(nz)
    for a, n in ((px, nx), (py, ny), (pz, nz)):
        a[:pw] = sigma
        a[n - pw:] = sigma[::-1]
    dfx, dfy, dfz = (np.exp(-a[:pw] * dt) for a in (px, py, pz))
    wx = np.ones((nz, ny, nx + 1))
    wx[:, :, :pw] = dfx
    wx[:, :, nx + 1 - pw:] = dfx[::-1]
    wy = np.ones((nz, ny + 1, nx))
    wy[:, :pw, :] = dfy[None, :, None]
    wy[:, ny + 1 - pw:, :] = dfy[::-1][None, :, None]
    wz = np.ones((nz + 1, ny, nx))
    wz[nz + 1 - pw:, :, :] = dfz[::-1][:, None, None]
    xy = np.ones((ny + 1, nx + 1))   # [y, x], every z
    xz = np.ones((nz + 1, nx + 1))   # [z, x], every y
    yz = np.ones((nz + 1, ny + 1))   # [z, y], every x
    for i in range(1, pw + 1):
        for j in range(1, pw + 1):
            dxy = math.exp(-0.5 * (px[i - 1] + py[j - 1]) * dt)
            dxz = math.exp(-0.5 * (px[i - 1] + pz[j - 1]) * dt)
            dyz = math.exp(-0.5 * (py[i - 1] + pz[j - 1]) * dt)
            xy[pw - 1:ny + 1 - pw, i - 1] = dxy
            xy[j - 1, pw - 1:nx + 1 - pw] = dxy
            xy[j - 1, i - 1] = dxy
            xy[pw - 1:ny + 1 - pw, nx - i - 1] = dxy
            xy[ny - j - 1, pw - 1:nx + 1 - pw] = dxy
            xy[ny - j - 1, nx - i - 1] = dxy
            xy[j - 1:pw, nx - i - 1] = dxy
            xy[ny - j - 1, i - 1:pw] = dxy
            xz[0:nz + 1 - pw, i - 1] = dxz
            xz[0:nz + 1 - pw, nx - i - 1] = dxz
            xz[nz - j - 1, pw - 1:nx + 1 - pw] = dxz
            xz[nz - j - 1, nx - i - 1] = dxz
            xz[nz - j - 1, i - 1:pw] = dxz
            yz[0:nz + 1 - pw, i - 1] = dyz
            yz[0:nz + 1 - pw, ny - i - 1] = dyz
            yz[nz - j - 1, pw - 1:ny + 1 - pw] = dyz
            yz[nz - j - 1, ny - i - 1] = dyz
            yz[nz - j - 1, i - 1:pw] = dyz
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    return {F.D_PX: f32(wx), F.D_PY: f32(wy), F.D_PZ: f32(wz),
            F.D_PXY: f32(np.broadcast_to(xy[None, :, :], (nz, ny + 1, nx + 1))),
            F.D_PXZ: f32(np.broadcast_to(xz[:, None, :], (nz + 1, ny, nx + 1))),
            F.D_PYZ: f32(np.broadcast_to(yz[:, :, None], (nz + 1, ny + 1, nx)))}


# ---------------------------------------------------------------------------------------------
# materials
# ---------------------------------------------------------------------------------------------


def harmonic_edges(C: np.ndarray, plane: str) -> np.ndarray:
    """Edge modulus from the 4 surrounding cells by harmonic mean, border planes 0
    (vizme_FastWaveED_GPU3D_9kmst_ANIS.m:438-454).  C has shape (nz, ny, nx).

    plane "xy" -> (nz, ny+1, nx+1) C66mxy; "xz" -> (nz+1, ny, nx+1) C55mxz; "yz" -> (nz+1, ny+1, nx) C44myz.
    """
    C = np.asarray(C, np.float64)
    nz, ny, nx = C.shape
    r = 1.0 / C
    if plane == "xy":
        out = np.zeros((nz, ny + 1, nx + 1))
        s = r[:, :-1, :-1] + r[:, :-1, 1:] + r[:, 1:, :-1] + r[:, 1:, 1:]
        out[:, 1:-1, 1:-1] = 4.0 / s
    elif plane == "xz":
        out = np.zeros((nz + 1, ny, nx + 1))
        s = r[:-1, :, :-1] + r[:-1, :, 1:] + r[1:, :, :-1] + r[1:, :, 1:]
        out[1:-1, :, 1:-1] = 4.0 / s
    elif plane == "yz":
        out = np.zeros((nz + 1, ny + 1, nx))
        s = r[:-1, :-1, :] + r[:-1, 1:, :] + r[1:, :-1, :] + r[1:, 1:, :]
        out[1:-1, 1:-1, :] = 4.0 / s
    else:
        raise ValueError(plane)
    return out.astype(np.float32)


def staggered_buoyancy(b: np.ndarray, axis: str) -> np.ndarray:
    """Face buoyancy from cell 1/rho by the 2-point mean, boundary faces 0
    (vizme_FastWaveED_GPU3D_9kmst_ANIS.m:386-399)."""
    b = np.asarray(b, np.float64)
    nz, ny, nx = b.shape
    if axis == "x":
        out = np.zeros((nz, ny, nx + 1))
        out[:, :, 1:-1] = (b[:, :, :-1] + b[:, :, 1:]) / 2
    elif axis == "y":
        out = np.zeros((nz, ny + 1, nx))
        out[:, 1:-1, :] = (b[:, :-1, :] + b[:, 1:, :]) / 2
    elif axis == "z":
        out = np.zeros((nz + 1, ny, nx))
        out[1:-1, :, :] = (b[:-1, :, :] + b[1:, :, :]) / 2
    else:
        raise ValueError(axis)
    return out.astype(np.float32)


def tsvankin_to_cij(vp0: float, vs0: float, rho: float, e1: float, e2: float, d1: float, d2: float, d3: float,
                    g1: float, g2: float) -> dict:
    """Orthorhombic stiffnesses from Tsvankin's (1997) parameters (symmetry planes = coordinate
    planes): Vp0 = sqrt(C33/rho), Vs0 = sqrt(C55/rho), eps^(1,2), delta^(1,2,3), gamma^(1,2)."""
    C33 = rho * vp0 * vp0
    C55 = rho * vs0 * vs0
    C11 = C33 * (1 + 2 * e2)
    C22 = C33 * (1 + 2 * e1)
    C66 = C55 * (1 + 2 * g1)
    C44 = C66 / (1 + 2 * g2)
    C13 = math.sqrt(2 * C33 * (C33 - C55) * d2 + (C33 - C55) ** 2) - C55
    C23 = math.sqrt(2 * C33 * (C33 - C44) * d1 + (C33 - C44) ** 2) - C44
    C12 = math.sqrt(2 * C11 * (C11 - C66) * d3 + (C11 - C66) ** 2) - C66
    return dict(C11=C11, C22=C22, C33=C33, C12=C12, C13=C13, C23=C23, C44=C44, C55=C55, C66=C66)


def is_positive_definite(c: dict) -> bool:
    A = np.array([[c["C11"], c["C12"], c["C13"]], [c["C12"], c["C22"], c["C23"]], [c["C13"], c["C23"], c["C33"]]])
    return bool(np.all(np.linalg.eigvalsh(A) > 0) and c["C44"] > 0 and c["C55"] > 0 and c["C66"] > 0)


def layered_ortho_layers(nlayers: int, seed: int) -> list[dict]:
    """Seeded layer table: Vp in U(3000,6500), Vp/Vs in U(1.6,1.9), rho in U(2200,2900), and
    eps1, eps2, delta1, delta2, delta3, gamma1, gamma2 in U(0, 0.15), redrawn until the
    stiffness is positive definite."""
    rng = np.random.default_rng(seed)
    layers = []
    while len(layers) < nlayers:
        vp = rng.uniform(3000, 6500)
        ratio = rng.uniform(1.6, 1.9)
        rho = rng.uniform(2200, 2900)
        e1, e2, d1, d2, d3, g1, g2 = rng.uniform(0.0, 0.15, size=7)
        c = tsvankin_to_cij(vp, vp / ratio, rho, e1, e2, d1, d2, d3, g1, g2)
        if not is_positive_definite(c):
            continue
        c["rho"] = rho
        layers.append(c)
    return layers


def layer_index(nz: int, nlayers: int) -> np.ndarray:
    """Layer of each z plane: equal thickness nz // nlayers, the remainder to the last layer."""
    th = nz // nlayers
    return np.minimum(np.arange(nz) // th, nlayers - 1)


# ---------------------------------------------------------------------------------------------
# sources
# ---------------------------------------------------------------------------------------------


def mt_strike_dip_rake(strike: float, dip: float, rake: float, M0: float = 1.0) -> np.ndarray:
    """Double-couple moment tensor (xx, yy, zz, xy, xz, yz) in x = north, y = east, z = down
    (Aki & Richards 2002, box 4.4)."""
    f, d, l = (math.radians(strike), math.radians(dip), math.radians(rake))
    sd, cd, s2d, c2d = math.sin(d), math.cos(d), math.sin(2 * d), math.cos(2 * d)
    sl, cl = math.sin(l), math.cos(l)
    sf, cf, s2f, c2f = math.sin(f), math.cos(f), math.sin(2 * f), math.cos(2 * f)
    mxx = -(sd * cl * s2f + s2d * sl * sf * sf)
    mxy = sd * cl * c2f + 0.5 * s2d * sl * s2f
    mxz = -(cd * cl * cf + c2d * sl * sf)
    myy = sd * cl * s2f - s2d * sl * cf * cf
    myz = -(cd * cl * sf - c2d * sl * cf)
    mzz = s2d * sl
    return M0 * np.array([mxx, myy, mzz, mxy, mxz, myz])


def lune_eigenvalues(gamma_deg: float, delta_deg: float) -> np.ndarray:
    """Unit eigenvalue triple (l1 >= l2 >= l3) at lune longitude gamma in [-30, 30] and latitude
    delta in [-90, 90] (the lune of Tape & Tape 2012): the deviatoric part runs from the CLVD
    (2,-1,-1)/sqrt6 at gamma = -30 through the double couple (1,0,-1)/sqrt2 to (1,1,-2)/sqrt6 at
    gamma = +30, and delta tilts it toward the isotropic (1,1,1)/sqrt3."""
    g, d = math.radians(gamma_deg), math.radians(delta_deg)
    dc = np.array([1.0, 0.0, -1.0]) / math.sqrt(2.0)
    cl = np.array([-1.0, 2.0, -1.0]) / math.sqrt(6.0)
    iso = np.array([1.0, 1.0, 1.0]) / math.sqrt(3.0)
    dev = math.cos(g) * dc + math.sin(g) * cl
    return math.cos(d) * dev + math.sin(d) * iso


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def lune_moment_tensor(seed: int, M0: float = 1.0) -> tuple[np.ndarray, dict]:
    """Seeded full moment tensor (DC + CLVD + ISO): lune point gamma ~ U(-30,30), delta ~ U(-90,90)
    (delta drawn uniform in sin so points are uniform on the lune) and a random orientation.
    Returns (xx, yy, zz, xy, xz, yz) scaled to Frobenius norm M0 and the draw."""
    rng = np.random.default_rng(seed)
    gamma = rng.uniform(-30.0, 30.0)
    delta = math.degrees(math.asin(rng.uniform(-1.0, 1.0)))
    lam = lune_eigenvalues(gamma, delta)
    U = random_rotation(rng)
    M = U @ np.diag(lam) @ U.T
    M = M0 * M / np.linalg.norm(M)
    return np.array([M[0, 0], M[1, 1], M[2, 2], M[0, 1], M[0, 2], M[1, 2]]), dict(gamma=gamma, delta=delta)


def rotate_mt(mt: np.ndarray, azimuth_deg: float) -> np.ndarray:
    """Q M Q^T with Q the rotation by `azimuth` about z (runmerotation.m:191-209)."""
    a = math.radians(azimuth_deg)
    Q = np.array([[math.cos(a), math.sin(a), 0.0], [-math.sin(a), math.cos(a), 0.0], [0.0, 0.0, 1.0]])
    xx, yy, zz, xy, xz, yz = mt
    M = np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])
    R = Q @ M @ Q.T
    return np.array([R[0, 0], R[1, 1], R[2, 2], R[0, 1], R[0, 2], R[1, 2]])


def ricker_stf(nt: int, dt: float, f0: float, t0: float | None = None, scale: float = 1.0) -> np.ndarray:
    """Per-step source increments of a Ricker moment-rate, integrated exactly in FP64.

    With tau = t - t0 the Ricker r(tau) = (1 - 2 pi^2 f0^2 tau^2) exp(-pi^2 f0^2 tau^2) has the
    antiderivative tau exp(-pi^2 f0^2 tau^2); Src[n] = scale * f0 * [R(t_{n+1}) - R(t_n)] is the
    moment-rate f0*r integrated over step n (so the injected stress is M_ij * Src[n])."""
    if t0 is None:
        t0 = 1.2 / f0
    t = np.arange(nt + 1, dtype=np.float64) * dt - t0
    a = (math.pi * f0) ** 2
    R = t * np.exp(-a * t * t)
    return scale * f0 * np.diff(R)


def matlab_colon(a: float, step: float, b: float) -> np.ndarray:
    """a:step:b as MATLAB's colon forms it -- n = floor((b - a)/step) + 1 elements (a relative
    tolerance of a few ulps admits the end point), element k = a + k*step.  MATLAB may round
    the second half of a long range from the far end instead; that differs in the last bit at
    most, below what a float32 Src.dat keeps."""
    n = int(math.floor((b - a) / step * (1.0 + 4 * np.finfo(float).eps))) + 1
    return a + step * np.arange(max(n, 0), dtype=np.float64)


def stf_isotropic_driver(nt: int, nx: int, lx: float, lam: float = 350.0, amp: float = 3.3 * 2e9,
                         shift: int = 199) -> np.ndarray:
    """The Src the isotropic MATLAB driver writes (FINAL.m:372-413, the last SourceGauss it builds):
    a Gaussian in the model's own x grid, init = amp exp(-(x / lam)^2) with x = -Lx/2 : dx : Lx/2,
    dx = Lx / (nx - 1) (FINAL.m:151, 373-381), shifted so that Src(1 : nx-shift) =
    init(shift+1 : end) (:395) and zero after.  Peak 6.6e9 with the driver's constants.  Needs no
    srctimefun.txt: the driver loads that file only for SourceSharp, which Src does not use.
    Returns FP64 samples (the driver writes them as float32)."""
    dx = lx / (nx - 1)
    x = matlab_colon(-lx / 2, dx, lx / 2)[:nx]
    init = amp * np.exp(-(x / lam) ** 2)
    n = nx - shift
    if n < 1:
        raise ValueError(f"nx = {nx}: the driver's shift of {shift} samples leaves no source")
    if n > nt:
        raise ValueError(f"Src(1:{n}) does not fit in nt = {nt} samples")
    src = np.zeros(nt)
    src[:n] = init[shift:shift + n]
    return src


def stf_orthorhombic_driver(nt: int, dx: float, dur: int = 400, lam: float = 1000.0, peak: float = 2.5e-3) -> np.ndarray:
    """The Src the orthorhombic MATLAB driver writes (ANIS.m:522-533): on the grid
    x = -20 dur : dx : 20 dur, init = peak exp(-(x / lam / 2)^2); SourceGauss(1 : 2 dur - 3) =
    -1e9 diff(diff(init)) (a negative second derivative of a Gaussian, Ricker-like), then scaled
    to a maximum of `peak` (2.5e-3).  The assignment needs exactly 2 dur - 1 grid points, as in the
    driver (dx = 15360 / 767 there); other spacings raise, as MATLAB's dimension check does.
    srctimefunL.txt, which the driver also loads, is only plotted."""
    x = matlab_colon(-dur * 20.0, dx, dur * 20.0)
    init = peak * np.exp(-(x / lam / 2) ** 2)
    g = -1e9 * np.diff(np.diff(init))
    if len(g) != 2 * dur - 3:
        raise ValueError(f"dx = {dx}: {len(x)} grid points give {len(g)} samples, the driver assigns {2 * dur - 3}")
    if 2 * dur - 3 > nt:
        raise ValueError(f"Src(1:{2 * dur - 3}) does not fit in nt = {nt} samples")
    src = np.zeros(nt)
    src[:len(g)] = g
    return src / src.max() * peak


# ---------------------------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------------------------


@dataclass
class Model:
    """Everything one run needs, in the reference layout."""

    nx: int
    ny: int
    nz: int
    nt: int
    dx: float
    dy: float
    dz: float
    dt: float
    model: int = F.MODEL_ISO
    damping: int = F.DAMP_PML1D
    src_order: int = F.SRC_BEFORE_BC1
    over_y: int = 0
    c66: float = 0.0
    bx: float = 0.0
    by: float = 0.0
    bz: float = 0.0
    vdamp: float = 0.0    # linear velocity damping of the 16 km scheme (0 = off)
    free_surface: int = F.FS_BC1   # F.FS_NONE: no BC1 (the diff_BC schemes)
    surface_mu: float = 0.0        # isotropic scheme: shear modulus on plane k = 1 when > 0 (0 = c66 there too)
    c44: float = 0.0      # per-component-weight scheme: shear moduli of yz and xz (c66: xy)
    c55: float = 0.0
    materials: dict = field(default_factory=dict)   # field id -> float32 array
    damping_arrays: dict = field(default_factory=dict)  # EWF_D_* -> float32 array
    sources: np.ndarray | None = None   # (n, 4) int32: comp, i, j, k
    source_coef: np.ndarray | None = None  # (n,) float64
    stf: np.ndarray | None = None       # (>= nt,) float64
    receivers: np.ndarray | None = None  # (n, 4) int32: i, j, k, comp
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    def set_moment_tensor(self, mt, xs: int, ys: int, zs: int, stencil: int) -> None:
        ent, coef = F.mt_entries(mt, xs, ys, zs, stencil)
        self.sources = ent
        self.source_coef = coef

    def courant(self) -> float:
        if self.model == F.MODEL_ISO:
            c = float(np.max(self.materials[F.M_C11]))
            b = max(self.bx, self.by, self.bz)
        else:
            c = max(float(np.max(self.materials[k])) for k in (F.M_C11, F.M_C22, F.M_C33) if k in self.materials)
            b = max(float(np.max(self.materials[k])) for k in (F.M_BX, F.M_BY, F.M_BZ))
        return math.sqrt(c * b) * self.dt * math.sqrt(1 / self.dx**2 + 1 / self.dy**2 + 1 / self.dz**2)


def ring_receivers(ci: int, cj: int, radius: float, n: int, k: int = 1, comps=(0, 1, 2)) -> np.ndarray:
    rec = []
    for q in range(n):
        a = 2 * math.pi * q / n
        i = int(round(ci + radius * math.cos(a)))
        j = int(round(cj + radius * math.sin(a)))
        for c in comps:
            rec.append((i, j, k, c))
    return np.array(rec, dtype=np.int32)


def grid_receivers(coords, k: int = 1, comps=(0, 1, 2)) -> np.ndarray:
    rec = [(i, j, k, c) for j in coords for i in coords for c in comps]
    return np.array(rec, dtype=np.int32)


def iso_homogeneous(n: int = 128, nt: int = 1000, dx: float = 50.0, vp: float = 6000.0, vs: float = 3464.0,
                    rho: float = 2700.0, lpml: int = 10, f0: float = 2.0, M0: float = 1e15,
                    strike: float = 30.0, dip: float = 60.0, rake: float = 90.0, n_rec: int = 8,
                    ring_radius_m: float = 2000.0) -> Model:
    """Plain isotropic FP32 workload: n^3 homogeneous grid, 1-D PML (lpml cells, all six faces),
    double couple at the grid centre, Ricker f0, dt at CFL 0.5 (dt = 0.5 dx / (Vp sqrt 3)),
    n_rec surface receivers (k = 1) on a ring, three components each."""
    dt = 0.5 * dx / (vp * math.sqrt(3.0))
    c11 = rho * vp * vp
    mu = rho * vs * vs
    c12 = c11 - 2 * mu
    shape = (n, n, n)
    m = Model(nx=n, ny=n, nz=n, nt=nt, dx=dx, dy=dx, dz=dx, dt=float(np.float32(dt)),
              model=F.MODEL_ISO, damping=F.DAMP_PML1D, src_order=F.SRC_BEFORE_BC1,
              c66=float(np.float32(mu)), bx=float(np.float32(1 / rho)), by=float(np.float32(1 / rho)),
              bz=float(np.float32(1 / rho)), name=f"iso{n}")
    m.dx = m.dy = m.dz = float(np.float32(dx))
    m.materials[F.M_C11] = np.full(shape, c11, np.float32)
    m.materials[F.M_C12] = np.full(shape, c12, np.float32)
    for axis, key in enumerate((F.D_WX, F.D_WY, F.D_WZ)):
        m.damping_arrays[key] = pml_weights(n, lpml, m.dt)
    c = n // 2
    # the OK4 stencil puts the normal stresses at (xs+1, ys+1, zs+1)
    m.set_moment_tensor(mt_strike_dip_rake(strike, dip, rake, 1.0), c - 1, c - 1, c - 1, stencil=0)
    m.stf = ricker_stf(nt, m.dt, f0, scale=M0 / (m.dx * m.dy * m.dz))
    m.receivers = ring_receivers(c, c, min(ring_radius_m / dx, 0.35 * n), n_rec)
    m.meta = dict(vp=vp, vs=vs, rho=rho, lpml=lpml, f0=f0, M0=M0, strike=strike, dip=dip, rake=rake)
    return m


def ortho_layered(nx: int = 320, ny: int = 320, nz: int = 256, nt: int = 4000, dx: float = 40.0,
                  nlayers: int = 12, seed: int = 20261203, mt_seed: int = 20261204, lpml: int = 15,
                  f0: float = 1.5, M0: float = 1e15, src=(160, 160, 128), rec_coords=None,
                  cfl: float = 0.5, damping: int | None = None) -> Model:
    """Orthorhombic layered FP32 workload: nlayers horizontal layers with seeded Vp, Vp/Vs, rho
    and Tsvankin anisotropy converted to 9 C_ij (edge moduli by harmonic 4-point means,
    staggered buoyancy by 2-point means, as the orthorhombic MATLAB driver builds them),
    15-cell PML on x, y and the bottom (free surface on top), seeded lune moment tensor at
    `src`, Ricker f0, dt at CFL 0.5 on max sqrt(C_ii/rho), 8x8 surface receivers."""
    layers = layered_ortho_layers(nlayers, seed)
    li = layer_index(nz, nlayers)
    prof = {k: np.array([layers[q][k] for q in li], np.float64) for k in
            ("C11", "C22", "C33", "C12", "C13", "C23", "C44", "C55", "C66", "rho")}
    vmax = max(math.sqrt(max(L["C11"], L["C22"], L["C33"]) / L["rho"]) for L in layers)
    dt = cfl * dx / (vmax * math.sqrt(3.0))
    m = Model(nx=nx, ny=ny, nz=nz, nt=nt, dx=float(np.float32(dx)), dy=float(np.float32(dx)),
              dz=float(np.float32(dx)), dt=float(np.float32(dt)), model=F.MODEL_ORTHO,
              damping=F.DAMP_SEPARABLE if damping is None else damping, src_order=F.SRC_AFTER_BC1,
              name=f"ortho{nx}x{ny}x{nz}")

    def full(v):
        return np.broadcast_to(v[:, None, None], (nz, ny, nx))

    for key, fid in (("C11", F.M_C11), ("C22", F.M_C22), ("C33", F.M_C33), ("C12", F.M_C12), ("C13", F.M_C13),
                     ("C23", F.M_C23)):
        m.materials[fid] = np.ascontiguousarray(full(prof[key]).astype(np.float32))
    m.materials[F.M_C44YZ] = harmonic_edges(full(prof["C44"]), "yz")
    m.materials[F.M_C55XZ] = harmonic_edges(full(prof["C55"]), "xz")
    m.materials[F.M_C66XY] = harmonic_edges(full(prof["C66"]), "xy")
    b = full(1.0 / prof["rho"])
    m.materials[F.M_BX] = staggered_buoyancy(b, "x")
    m.materials[F.M_BY] = staggered_buoyancy(b, "y")
    m.materials[F.M_BZ] = staggered_buoyancy(b, "z")
    px = pml_factors(nx, lpml, m.dt)
    py = pml_factors(ny, lpml, m.dt)
    pz = pml_factors(nz, lpml, m.dt, sides="high")
    if m.damping == F.DAMP_SEPARABLE:
        m.damping_arrays[F.D_WX] = px
        m.damping_arrays[F.D_WY] = py
        m.damping_arrays[F.D_WZ] = pz
    else:
        m.damping_arrays[F.D_W3D] = separable_weights(px, py, pz)
    mt, draw = lune_moment_tensor(mt_seed)
    xs, ys, zs = src
    # the ANISO stencil puts the normal stresses at (xs+1, ys+1, zs+1)
    m.set_moment_tensor(mt, xs - 1, ys - 1, zs - 1, stencil=1)
    m.stf = ricker_stf(nt, m.dt, f0, scale=M0 / (m.dx * m.dy * m.dz))
    if rec_coords is None:
        step = max(1, (nx - 2 * 40) // 7)
        rec_coords = [40 + step * q for q in range(8)]
    m.receivers = grid_receivers(rec_coords)
    m.meta = dict(nlayers=nlayers, seed=seed, mt_seed=mt_seed, lpml=lpml, f0=f0, M0=M0, mt=mt.tolist(), lune=draw,
                  vmax=vmax)
    return m


def iso_het_layered(nx: int, ny: int, nz: int, nt: int, dx: float, dt: float, layers: list[dict],
                    thick: int = 120, margin_y: int = 210, rate: float = 0.16) -> Model:
    """The 9 km station driver's model (vizme_FastWaveED_GPU3D_9kmst.m:255-444) for the
    EWF_MODEL_ISO_HET scheme.  ``layers`` = [{"top": k0, "vp": m/s, "vs": m/s, "rho": kg/m^3}, ...]
    by increasing top (the first layer's top is 0): cell fields c11 = rho vp^2 and
    c12 = K - 2/3 mu with K = c11 - 4/3 mu, mu = rho vs^2 (:262-268); the edge shear moduli are the
    4-cell harmonic means of mu with zero border planes (:377-396); the staggered 1/rho fields
    are the 2-point means with zero boundary faces (:323-350); the 3-D sponge weights.dat (:397-444,
    sponge_3d_legacy).  Source and receivers are left to the caller."""
    tops = [int(L["top"]) for L in layers] + [nz]
    mu = np.empty((nz, ny, nx))
    c11 = np.empty((nz, ny, nx))
    rho = np.empty((nz, ny, nx))
    for L, k0, k1 in zip(layers, tops[:-1], tops[1:]):
        r = float(L["rho"])
        rho[k0:k1] = r
        c11[k0:k1] = float(L["vp"]) ** 2 * r
        mu[k0:k1] = float(L["vs"]) ** 2 * r
    K = c11 - 4.0 / 3.0 * mu
    m = Model(nx=nx, ny=ny, nz=nz, nt=nt, dx=float(np.float32(dx)), dy=float(np.float32(dx)), dz=float(np.float32(dx)),
              dt=float(np.float32(dt)), model=F.MODEL_ISO_HET, damping=F.DAMP_W3D, src_order=F.SRC_AFTER_BC1,
              name=f"iso_het_{nx}x{ny}x{nz}")
    m.materials[F.M_C11] = c11.astype(np.float32)
    m.materials[F.M_C12] = (K - 2.0 / 3.0 * mu).astype(np.float32)
    m.materials[F.M_C66XY] = harmonic_edges(mu, "xy")
    m.materials[F.M_C55XZ] = harmonic_edges(mu, "xz")
    m.materials[F.M_C44YZ] = harmonic_edges(mu, "yz")
    b = 1.0 / rho
    m.materials[F.M_BX] = staggered_buoyancy(b, "x")
    m.materials[F.M_BY] = staggered_buoyancy(b, "y")
    m.materials[F.M_BZ] = staggered_buoyancy(b, "z")
    m.damping_arrays[F.D_W3D] = sponge_3d_legacy(nx, ny, nz, thick=thick, margin_y=margin_y, rate=rate)
    return m


def random_small(model: int, nx: int, ny: int, nz: int, nt: int, seed: int, damping: int | None = None,
                 src_order: int | None = None, stencil: int | None = None) -> Model:
    """Small heterogeneous test case with random (but stable) materials, random damping
    profiles, a random moment tensor and a random STF -- exercises every code path."""
    rng = np.random.default_rng(seed)
    dx, dy, dz = 10.0, 11.0, 12.0
    vp = 3000.0
    dt = 0.4 / (vp * 1.3 * math.sqrt(1 / dx**2 + 1 / dy**2 + 1 / dz**2))
    m = Model(nx=nx, ny=ny, nz=nz, nt=nt, dx=dx, dy=dy, dz=dz, dt=float(np.float32(dt)), model=model,
              name=f"rand{model}_{nx}x{ny}x{nz}")
    rho = rng.uniform(2000, 3000, size=(nz, ny, nx))
    vpf = rng.uniform(0.8, 1.3, size=(nz, ny, nx)) * vp
    vsf = vpf / rng.uniform(1.6, 2.0, size=(nz, ny, nx))
    c33 = rho * vpf**2
    mu = rho * vsf**2
    if model == F.MODEL_ISO and damping == F.DAMP_PERCOMP:
        # the DC_Earthquake solver: c11/c12 fields, three shear scalars, a weight field per
        # component (random near the faces), the ANISO loop order
        m.damping = F.DAMP_PERCOMP
        m.src_order = F.SRC_AFTER_BC1 if src_order is None else src_order
        m.materials[F.M_C11] = c33.astype(np.float32)
        m.materials[F.M_C12] = (c33 - 2 * mu).astype(np.float32)
        m.c66 = float(np.float32(np.median(mu)))
        m.c55 = float(np.float32(np.median(mu) * 1.03))
        m.c44 = float(np.float32(np.median(mu) * 0.97))
        m.bx, m.by, m.bz = (float(np.float32(1 / 2500.0)), float(np.float32(1 / 2600.0)), float(np.float32(1 / 2400.0)))
        for fid in F.PERCOMP_WEIGHTS:
            shp = F.shape(fid, nx, ny, nz)
            w = np.ones(shp, np.float32)
            for ax in range(3):
                sl = [slice(None)] * 3
                sl[ax] = slice(0, 3)
                w[tuple(sl)] *= rng.uniform(0.9, 1.0, size=w[tuple(sl)].shape).astype(np.float32)
                sl[ax] = slice(shp[ax] - 3, shp[ax])
                w[tuple(sl)] *= rng.uniform(0.9, 1.0, size=w[tuple(sl)].shape).astype(np.float32)
            m.damping_arrays[fid] = w
    elif model == F.MODEL_ISO:
        m.damping = F.DAMP_PML1D
        m.src_order = F.SRC_BEFORE_BC1 if src_order is None else src_order
        m.materials[F.M_C11] = c33.astype(np.float32)
        m.materials[F.M_C12] = (c33 - 2 * mu).astype(np.float32)
        m.c66 = float(np.float32(np.median(mu)))
        m.bx, m.by, m.bz = (float(np.float32(1 / 2500.0)), float(np.float32(1 / 2600.0)), float(np.float32(1 / 2400.0)))
        for key, n in ((F.D_WX, nx), (F.D_WY, ny), (F.D_WZ, nz)):
            w = np.ones(n + 1, np.float32)
            w[:3] = rng.uniform(0.9, 1.0, 3)
            w[-3:] = rng.uniform(0.9, 1.0, 3)
            m.damping_arrays[key] = w.astype(np.float32)
    elif model == F.MODEL_ISO_HET:
        m.damping = F.DAMP_W3D if damping is None else damping
        m.src_order = F.SRC_AFTER_BC1 if src_order is None else src_order
        m.materials[F.M_C11] = c33.astype(np.float32)
        m.materials[F.M_C12] = (c33 - 2 * mu).astype(np.float32)
        m.materials[F.M_C66XY] = harmonic_edges(mu, "xy")
        m.materials[F.M_C55XZ] = harmonic_edges(mu, "xz")
        m.materials[F.M_C44YZ] = harmonic_edges(mu, "yz")
        b = 1.0 / rho
        m.materials[F.M_BX] = staggered_buoyancy(b, "x")
        m.materials[F.M_BY] = staggered_buoyancy(b, "y")
        m.materials[F.M_BZ] = staggered_buoyancy(b, "z")
        px, py, pz = (np.ones(n, np.float32) for n in (nx, ny, nz))
        for p in (px, py, pz):
            p[:3] = rng.uniform(0.9, 1.0, 3)
            p[-3:] = rng.uniform(0.9, 1.0, 3)
        if m.damping == F.DAMP_SEPARABLE:
            m.damping_arrays[F.D_WX], m.damping_arrays[F.D_WY], m.damping_arrays[F.D_WZ] = px, py, pz
        else:
            m.damping_arrays[F.D_W3D] = separable_weights(px, py, pz) * rng.uniform(0.999, 1.0, size=(nz, ny, nx)).astype(np.float32)
    else:
        m.damping = F.DAMP_W3D if damping is None else damping
        m.src_order = F.SRC_AFTER_BC1 if src_order is None else src_order
        ani = rng.uniform(1.0, 1.15, size=(nz, ny, nx))
        m.materials[F.M_C11] = (c33 * ani).astype(np.float32)
        m.materials[F.M_C22] = (c33 * rng.uniform(1.0, 1.1, size=(nz, ny, nx))).astype(np.float32)
        m.materials[F.M_C33] = c33.astype(np.float32)
        lam = c33 - 2 * mu
        m.materials[F.M_C12] = (lam * rng.uniform(0.95, 1.05, size=(nz, ny, nx))).astype(np.float32)
        m.materials[F.M_C13] = (lam * rng.uniform(0.95, 1.05, size=(nz, ny, nx))).astype(np.float32)
        m.materials[F.M_C23] = (lam * rng.uniform(0.95, 1.05, size=(nz, ny, nx))).astype(np.float32)
        m.materials[F.M_C44YZ] = harmonic_edges(mu, "yz")
        m.materials[F.M_C55XZ] = harmonic_edges(mu * 1.05, "xz")
        m.materials[F.M_C66XY] = harmonic_edges(mu * 0.95, "xy")
        b = 1.0 / rho
        m.materials[F.M_BX] = staggered_buoyancy(b, "x")
        m.materials[F.M_BY] = staggered_buoyancy(b, "y")
        m.materials[F.M_BZ] = staggered_buoyancy(b, "z")
        px = np.ones(nx, np.float32)
        py = np.ones(ny, np.float32)
        pz = np.ones(nz, np.float32)
        for p in (px, py, pz):
            p[:3] = rng.uniform(0.9, 1.0, 3)
            p[-3:] = rng.uniform(0.9, 1.0, 3)
        if m.damping == F.DAMP_SEPARABLE:
            m.damping_arrays[F.D_WX], m.damping_arrays[F.D_WY], m.damping_arrays[F.D_WZ] = px, py, pz
        else:
            m.damping_arrays[F.D_W3D] = separable_weights(px, py, pz) * rng.uniform(0.999, 1.0, size=(nz, ny, nx)).astype(np.float32)
    st = (0 if model == F.MODEL_ISO and m.damping != F.DAMP_PERCOMP else 1) if stencil is None else stencil
    mt = rng.normal(size=6)
    xs, ys, zs = nx // 2 - 2, ny // 2 - 1, nz // 2 - 1
    m.set_moment_tensor(mt, xs, ys, zs, stencil=st)
    m.stf = (rng.normal(size=nt) * 1e6).astype(np.float32).astype(np.float64)
    recs = []
    for q in range(6):
        recs.append((int(rng.integers(1, nx - 1)), int(rng.integers(1, ny - 1)), int(rng.integers(1, nz - 1)), q % 3))
    recs.append((nx // 2, ny // 2, 1, 2))
    m.receivers = np.array(recs, dtype=np.int32)
    return m
