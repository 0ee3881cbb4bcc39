"""Input generators (restatements of the MATLAB drivers) -- CPU only."""
import math

import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I


def test_pml_weights_formula_and_mirror():
    n, lpml, dt = 40, 10, 1e-3
    w = I.pml_weights(n, lpml, dt)
    assert w.shape == (n + 1,) and w.dtype == np.float32
    s1 = 1.5 / (lpml / n) * 8.0 * 1.0  # i = 1: ((lpml-1+1)/lpml)^2 = 1, log10(1e8) = 8
    assert w[0] == np.float32(math.exp(-s1 * dt))
    assert w[n] == w[0]  # index n - i + 2 (1-based) mirrors index i
    assert np.all(w[lpml:n - lpml + 1] == 1.0)
    assert np.all(np.diff(w[:lpml]) > 0)
    wt = I.pml_weights(n, lpml, dt, top_override=True)
    assert np.all(wt[: n // 2] == 1.0) and wt[n] == w[n]


def test_sponge_3d_matches_loop_restatement():
    nx, ny, nz, thick, my = 12, 14, 10, 3, 4
    W = I.sponge_3d_legacy(nx, ny, nz, thick, my, 0.16)
    a = 0.16 / thick
    for iz in range(1, nz + 1):
        for iy in range(1, ny + 1):
            for ix in range(1, nx + 1):
                i = j = k = 0
                if ix < thick + 1:
                    i = thick + 1 - ix
                if iy < my + 1:
                    k = my + 1 - iy
                if nx - thick < ix:
                    i = ix - nx + thick
                if ny - my < iy:
                    k = iy - ny + my
                if nz - thick < iz:
                    j = iz - nz + thick
                want = 1.0 if (i == 0 and j == 0 and k == 0) else math.exp(-a * a * (i * i + j * j + k * k))
                assert W[iz - 1, iy - 1, ix - 1] == np.float32(want)


def test_separable_weights_is_float32_product():
    rng = np.random.default_rng(0)
    px, py, pz = (rng.uniform(0.5, 1, n).astype(np.float32) for n in (5, 6, 7))
    W = I.separable_weights(px, py, pz)
    assert W.shape == (7, 6, 5)
    assert W[3, 2, 1] == np.float32(np.float32(px[1] * py[2]) * pz[3])


def test_harmonic_edges_and_buoyancy():
    rng = np.random.default_rng(1)
    C = rng.uniform(1, 2, (4, 5, 6))
    E = I.harmonic_edges(C, "xy")
    assert E.shape == (4, 6, 7)
    assert np.all(E[:, 0, :] == 0) and np.all(E[:, :, 0] == 0) and np.all(E[:, -1, :] == 0)
    want = 4 / (1 / C[2, 1, 2] + 1 / C[2, 1, 3] + 1 / C[2, 2, 2] + 1 / C[2, 2, 3])
    assert abs(E[2, 2, 3] - want) < 1e-6 * want
    assert I.harmonic_edges(C, "xz").shape == (5, 5, 7)
    assert I.harmonic_edges(C, "yz").shape == (5, 6, 6)
    B = I.staggered_buoyancy(1 / C, "x")
    assert B.shape == (4, 5, 7) and np.all(B[:, :, 0] == 0) and np.all(B[:, :, -1] == 0)
    assert abs(B[1, 1, 3] - (1 / C[1, 1, 2] + 1 / C[1, 1, 3]) / 2) < 1e-6


def test_tsvankin_round_trip():
    c = I.tsvankin_to_cij(4000, 2300, 2500, 0.1, 0.12, 0.05, 0.07, 0.03, 0.08, 0.11)
    C33, C55, C44, C66, C11, C22 = c["C33"], c["C55"], c["C44"], c["C66"], c["C11"], c["C22"]
    assert abs(math.sqrt(C33 / 2500) - 4000) < 1e-9 * 4000
    assert abs((C11 - C33) / (2 * C33) - 0.12) < 1e-12
    assert abs((C22 - C33) / (2 * C33) - 0.1) < 1e-12
    assert abs((C66 - C55) / (2 * C55) - 0.08) < 1e-12
    assert abs((C66 - C44) / (2 * C44) - 0.11) < 1e-12
    d2 = ((c["C13"] + C55) ** 2 - (C33 - C55) ** 2) / (2 * C33 * (C33 - C55))
    assert abs(d2 - 0.07) < 1e-12
    d3 = ((c["C12"] + C66) ** 2 - (C11 - C66) ** 2) / (2 * C11 * (C11 - C66))
    assert abs(d3 - 0.03) < 1e-12
    assert I.is_positive_definite(c)


def test_layers_seeded_and_in_range():
    L1 = I.layered_ortho_layers(12, 20261203)
    L2 = I.layered_ortho_layers(12, 20261203)
    assert [x["C33"] for x in L1] == [x["C33"] for x in L2]
    for x in L1:
        vp = math.sqrt(x["C33"] / x["rho"])
        assert 3000 <= vp <= 6500 and 2200 <= x["rho"] <= 2900
    li = I.layer_index(256, 12)
    assert li[0] == 0 and li[-1] == 11 and np.sum(li == 11) == 256 - 11 * 21


def test_mt_strike_dip_rake_known_cases():
    # vertical strike-slip on a north-striking fault: pure Mxy
    mt = I.mt_strike_dip_rake(0, 90, 0)
    assert np.allclose(mt, [0, 0, 0, 1, 0, 0], atol=1e-12)
    # 45-degree thrust striking north: Myy = -1, Mzz = +1
    mt = I.mt_strike_dip_rake(0, 45, 90)
    assert np.allclose(mt, [0, -1, 1, 0, 0, 0], atol=1e-12)
    # always traceless, unit norm sqrt(2)
    mt = I.mt_strike_dip_rake(30, 60, 90)
    assert abs(mt[0] + mt[1] + mt[2]) < 1e-12
    M = np.array([[mt[0], mt[3], mt[4]], [mt[3], mt[1], mt[5]], [mt[4], mt[5], mt[2]]])
    assert abs(np.linalg.norm(M) - math.sqrt(2)) < 1e-12


def test_lune():
    assert np.allclose(I.lune_eigenvalues(0, 0), np.array([1, 0, -1]) / math.sqrt(2))
    assert np.allclose(I.lune_eigenvalues(-30, 0), np.array([2, -1, -1]) / math.sqrt(6))
    assert np.allclose(I.lune_eigenvalues(30, 0), np.array([1, 1, -2]) / math.sqrt(6))
    assert np.allclose(I.lune_eigenvalues(0, 90), np.ones(3) / math.sqrt(3))
    mt, draw = I.lune_moment_tensor(7)
    M = np.array([[mt[0], mt[3], mt[4]], [mt[3], mt[1], mt[5]], [mt[4], mt[5], mt[2]]])
    ev = np.sort(np.linalg.eigvalsh(M))[::-1]
    assert np.allclose(ev, I.lune_eigenvalues(draw["gamma"], draw["delta"]), atol=1e-12)


def test_rotate_mt_matches_reference_values():
    # known answer from the reference: runmerotation.m:200-207 rotates this tensor by 139 degrees
    # and its comment at :146-148 lists the result, which is also the tensor the orthorhombic
    # solver hard-codes (FastWaveED_GPU3D_v1_9kmst_ANISO.cu:233-247)
    src = np.array([0.4895, -0.1740, 0.2439, 0.8403, 0.3594, 0.0005])  # xx yy zz xy xz yz
    want = np.array([-0.6282, 0.9437, 0.2439, 0.4455, -0.2709, -0.2362])
    np.testing.assert_allclose(I.rotate_mt(src, 139.0), want, atol=1.5e-4)
    np.testing.assert_allclose(np.array(F.ANISO_LEGACY_MT), want, atol=1e-7)
    # and the rotation preserves invariants and inverts
    mt = np.array([0.3, -0.5, 0.2, 0.1, -0.4, 0.25])
    r = I.rotate_mt(I.rotate_mt(mt, 139.0), -139.0)
    assert np.allclose(r, mt)
    r = I.rotate_mt(mt, 90.0)
    assert abs(r[0] - mt[1]) < 1e-12 and abs(r[1] - mt[0]) < 1e-12 and abs(r[2] - mt[2]) < 1e-12


def test_ricker_integrated():
    dt, f0 = 1e-3, 2.0
    s = I.ricker_stf(4000, dt, f0)
    # increments of an antiderivative: the running sum is R(t) f0 evaluated exactly
    t1, t0 = 4000 * dt - 1.2 / f0, -1.2 / f0
    R = lambda t: f0 * t * math.exp(-(math.pi * f0 * t) ** 2)  # noqa: E731
    assert abs(s.sum() - (R(t1) - R(t0))) < 1e-15
    # close to the sampled moment-rate
    mid = (np.arange(4000) + 0.5) * dt - 1.2 / f0
    r = f0 * (1 - 2 * (math.pi * f0 * mid) ** 2) * np.exp(-(math.pi * f0 * mid) ** 2) * dt
    assert np.max(np.abs(s - r)) < 1e-4 * np.max(np.abs(r))


def test_mt_entries_stencils():
    e, c = F.mt_entries([1, 2, 3, 4, 5, 6], 10, 20, 30, 0)
    assert e.tolist() == [[3, 11, 21, 31], [4, 11, 21, 31], [5, 11, 21, 31], [8, 12, 22, 31], [7, 13, 23, 31],
                          [6, 13, 23, 31]]
    assert c.tolist() == [1, 2, 3, 6, 5, 4]
    e, c = F.mt_entries([1, 2, 3, 4, 5, 6], 10, 20, 30, 1)
    assert e.tolist() == [[3, 11, 21, 31], [4, 11, 21, 31], [5, 11, 21, 31], [6, 12, 22, 31], [8, 13, 22, 31],
                          [7, 9, 21, 31]]


def test_workloads_are_stable_and_sized():
    m = I.iso_homogeneous(n=48, nt=10)
    assert abs(m.courant() - 0.5) < 1e-6
    assert m.receivers[:, 0].max() < 48 and m.receivers[:, 0].min() >= 0
    m = I.ortho_layered(nx=48, ny=48, nz=40, nt=10, src=(24, 24, 20))
    assert m.courant() < 0.75
    assert m.materials[F.M_C66XY].shape == (40, 49, 49)
    assert len(m.receivers) == 64 * 3


def test_oracle_isohet_agrees_with_mapped_orthorhombic_scheme():
    """The 9 km scheme is the orthorhombic one with C22 = C33 = C11, C13 = C23 = C12 and the shear
    derivatives multiplied by 1/d instead of divided by d: the two oracle runs agree to rounding."""
    from oracle import oracle as O

    m = I.random_small(F.MODEL_ISO_HET, 24, 26, 18, nt=30, seed=3)
    a = O.run(m, 30)
    mo = I.random_small(F.MODEL_ISO_HET, 24, 26, 18, nt=30, seed=3)
    mo.model = F.MODEL_ORTHO
    mo.materials[F.M_C22] = mo.materials[F.M_C33] = mo.materials[F.M_C11]
    mo.materials[F.M_C13] = mo.materials[F.M_C23] = mo.materials[F.M_C12]
    b = O.run(mo, 30)
    assert np.abs(a.traces).max() > 0
    assert np.linalg.norm(a.traces - b.traces) / np.linalg.norm(a.traces) < 1e-5
    assert not np.array_equal(a.traces, b.traces)
    m.vdamp = F.VDAMP_16KM
    c = O.run(m, 30)
    assert not np.array_equal(a.traces, c.traces)


def test_iso_het_layered_fields():
    L = [{"top": 0, "vp": 3000.0, "vs": 1700.0, "rho": 2200.0}, {"top": 6, "vp": 5000.0, "vs": 2900.0, "rho": 2700.0}]
    m = I.iso_het_layered(12, 10, 14, nt=5, dx=100.0, dt=0.005, layers=L, thick=3, margin_y=3)
    mu1, mu2 = 2200.0 * 1700.0 ** 2, 2700.0 * 2900.0 ** 2
    assert m.materials[F.M_C11].shape == (14, 10, 12)
    assert m.materials[F.M_C11][0, 0, 0] == np.float32(2200.0 * 3000.0 ** 2)
    assert m.materials[F.M_C12][10, 0, 0] == np.float32(2700.0 * 5000.0 ** 2 - 2 * mu2)
    # edge moduli: harmonic means, zero on the border planes; interfaces mix the two layers
    xz = m.materials[F.M_C55XZ]
    assert xz.shape == (15, 10, 13) and xz[0].max() == 0 and xz[:, :, 0].max() == 0
    assert xz[3, 4, 5] == np.float32(mu1) and xz[10, 4, 5] == np.float32(mu2)
    assert np.isclose(xz[6, 4, 5], 4 / (2 / mu1 + 2 / mu2), rtol=1e-6)
    bz = m.materials[F.M_BZ]
    assert bz.shape == (15, 10, 12) and bz[0].max() == 0 and np.isclose(bz[6, 3, 3], (1 / 2200 + 1 / 2700) / 2)
    w = m.damping_arrays[F.D_W3D]
    assert w.shape == (14, 10, 12) and w[0, 5, 6] == 1.0 and w[-1, 5, 6] < 1.0


def test_percomp_weights_follow_the_driver():
    nx, ny, nz, lpml, dt = 30, 28, 26, 6, 0.002
    w = I.percomp_weights(nx, ny, nz, dt, lpml=lpml)
    for fid, arr in w.items():
        assert arr.shape == F.shape(fid, nx, ny, nz) and arr.dtype == np.float32
        assert arr.max() <= 1.0 and arr.min() > 0.0
    sig1 = 1.5 / (lpml / nx) * 5.0  # log10(1/1e-5) = 5, the outermost cell
    assert np.isclose(w[F.D_PX][3, 4, 0], np.exp(-sig1 * dt))
    assert w[F.D_PX][3, 4, nx // 2] == 1.0
    assert np.isclose(w[F.D_PX][3, 4, nx], np.exp(-sig1 * dt))           # mirrored at the far end
    assert w[F.D_PZ][0, 5, 5] == 1.0 and w[F.D_PZ][nz, 5, 5] < 1.0        # no damping at the top
    # shear weights: the corner cell carries the mean of both profiles; the interior is untouched
    assert np.isclose(w[F.D_PXY][7, 0, 0], np.exp(-sig1 * dt))
    assert w[F.D_PXY][7, ny // 2, nx // 2] == 1.0
    assert np.all(w[F.D_PXY] == w[F.D_PXY][:1])                           # constant along z
    assert np.all(w[F.D_PYZ] == w[F.D_PYZ][:, :, :1])                     # constant along x
    with pytest.raises(ValueError):
        I.percomp_weights(12, 12, 12, dt, lpml=6)


def _loop_isotropic_driver_stf(nt, nx, lx):
    """FINAL.m:372-395 as scalar loops: the x grid, the Gaussian, the shifted copy."""
    dx = lx / (nx - 1)
    init = [3.3 * 2e9 * math.exp(-((-lx / 2 + m * dx) / 350.0) ** 2) for m in range(nx)]
    src = [0.0] * nt
    for n in range(nx - 199):
        src[n] = init[n + 199]
    return src


def _loop_orthorhombic_driver_stf(nt, dx, dur=400):
    """ANIS.m:522-533 as scalar loops: the grid, the Gaussian, minus its second difference,
    normalised to a peak of 2.5e-3."""
    npts = int(math.floor(dur * 40.0 / dx * (1 + 4 * 2.0 ** -52))) + 1
    init = [2.5e-3 * math.exp(-((-dur * 20.0 + m * dx) / 1000.0 / 2) ** 2) for m in range(npts)]
    g = [-1e9 * ((init[m + 2] - init[m + 1]) - (init[m + 1] - init[m])) for m in range(npts - 2)]
    src = [0.0] * nt
    for n, v in enumerate(g):
        src[n] = v
    mx = max(src)
    return [v / mx * 2.5e-3 for v in src]


def test_driver_source_time_functions():
    # the isotropic driver's grid: nx = 64 * NBX = 768, Lx = 7680 m, nt = 3000; Src peaks at 6.6e9
    nt, nx, lx = 3000, 768, 7680.0
    a = I.stf_isotropic_driver(nt, nx, lx)
    b = np.array(_loop_isotropic_driver_stf(nt, nx, lx))
    assert a.shape == (nt,)
    np.testing.assert_allclose(a, b, rtol=1e-13, atol=0)
    np.testing.assert_array_equal(a.astype(np.float32), b.astype(np.float32))
    assert np.isclose(a.max(), 6.6e9, rtol=1e-3) and a[nx - 199:].max() == 0.0
    # the orthorhombic driver: dx = 15360 / 767, 2 * 400 - 3 = 797 samples, peak 2.5e-3
    dx = 2 * 7680 / (768 - 1)
    a = I.stf_orthorhombic_driver(4500, dx)
    b = np.array(_loop_orthorhombic_driver_stf(4500, dx))
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-18)
    np.testing.assert_array_equal(a.astype(np.float32)[a != 0].size, 797)
    assert a.max() == 2.5e-3 and a[797:].max() == 0.0
    assert a[398] == a.max() and a[0] < 0 and a[200] < 0     # Ricker-like: central peak, negative lobes
    with pytest.raises(ValueError):
        I.stf_orthorhombic_driver(4500, 25.0)                  # 641 points: MATLAB's dimension error
    with pytest.raises(ValueError):
        I.stf_isotropic_driver(500, nx, lx)
