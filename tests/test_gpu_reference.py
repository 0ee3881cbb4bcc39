"""Product and oracle against the reference's OWN kernels, compiled from the reference sources
into oracle/_ref/*.cubin and replayed by oracle/refrun.py on the same inputs.

* "exact" cubins (--fmad=false): bit-identical velocity fields, normal stresses and traces.
  Shear-stress cells on the planes i = 0 / j = 0 / k = 0 are excluded: there the isotropic
  reference reads a wrapped neighbour (FastWaveED_GPU3D_v1.cu:323-329) -- values the velocity
  update never reads back.
* "stock" cubins (-O3 with FMA contraction, the reference's own build flags): relative L2 error of
  every seismogram <= 1e-4 after the full run.
"""
import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300.solver import Solver
from oracle import oracle as O
from oracle import refrun as R

pytestmark = pytest.mark.gpu


def edge_mask(q, shape):
    """True where a cell is observable (not a never-read shear edge cell)."""
    mask = np.ones(shape, bool)
    if q == F.F_SXY:
        mask[:, 0, :] = False
        mask[:, :, 0] = False
    elif q == F.F_SXZ:
        mask[0, :, :] = False
        mask[:, :, 0] = False
    elif q == F.F_SYZ:
        mask[0, :, :] = False
        mask[:, 0, :] = False
    return mask


def reference(m, nsteps, variant):
    vd = getattr(m, "vdamp", 0.0)
    sc = (m.meta or {}).get("scheme")
    assert R.available(m.model, variant, vd, m.damping, sc), \
        f"missing {R.cubin(m.model, variant, vd, m.damping, sc)}: run oracle/build.py where the reference is"
    r = R.RefRunner(m, variant)
    try:
        r.run(nsteps)
        return r.fields(), r.traces.copy()
    finally:
        r.close()


def iso_case(nx=40, ny=44, nz=24, nt=60, seed=21, zs=9):
    m = I.random_small(F.MODEL_ISO, nx, ny, nz, nt=nt, seed=seed)
    m.set_moment_tensor(np.array([0.5, -1.0, 0.3, 0.2, 1.0, 0.8]), nx // 2 - 3, ny // 2 - 3, zs, 0)
    return m


def ortho_case(nx=36, ny=40, nz=26, nt=60, seed=22, zs=8, damping=F.DAMP_W3D):
    m = I.random_small(F.MODEL_ORTHO, nx, ny, nz, nt=nt, seed=seed, damping=damping)
    m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), nx // 2 - 2, ny // 2 - 2, zs, 1)
    return m


def isohet_case(nx=36, ny=40, nz=26, nt=60, seed=23, zs=8, damping=F.DAMP_W3D, vdamp=False):
    """The 9 km station scheme; with vdamp, the 16 km station scheme (its tensor and damping)."""
    m = I.random_small(F.MODEL_ISO_HET, nx, ny, nz, nt=nt, seed=seed, damping=damping)
    mt = F.ISO16KM_LEGACY_MT if vdamp else F.ANISO_LEGACY_MT
    m.set_moment_tensor(np.array(mt), nx // 2 - 2, ny // 2 - 2, zs, 1)
    m.vdamp = F.VDAMP_16KM if vdamp else 0.0
    return m


def dcq_case(nx=36, ny=40, nz=26, nt=60, seed=25, zs=8):
    """The DC_Earthquake solver: isotropic with per-component 3-D weights and its own source."""
    m = I.random_small(F.MODEL_ISO, nx, ny, nz, nt=nt, seed=seed, damping=F.DAMP_PERCOMP)
    m.set_moment_tensor(np.array(F.DCQ_LEGACY_MT), nx // 2 - 2, ny // 2 - 2, zs, 1)
    return m


# the built-in source of the DC_Earthquake FULL family: sigma_xz += 1.0 Src, sigma_yz += 0.8 Src
FULL_FAMILY_MT = np.array([0.0, 0.0, 0.0, 0.0, 1.0, 0.8])


def ok3_case(nx=40, ny=44, nz=24, nt=60, seed=27, zs=9):
    """The diff_BC2_OK3 scheme: OK4 without BC1 and with a shear modulus of 1e-5 on plane 1."""
    m = I.random_small(F.MODEL_ISO, nx, ny, nz, nt=nt, seed=seed)
    m.free_surface = F.FS_NONE
    m.surface_mu = 1e-5
    m.set_moment_tensor(FULL_FAMILY_MT, nx // 2 - 3, ny // 2 - 3, zs, 0)
    m.meta = dict(m.meta or {}, scheme="ok3")
    return m


def constant_moduli(m, c66, c55, c44, b, plane1=None):
    """The 9 km scheme's fields filled the way the FULL family's scalars act: constant edge shear
    moduli (plane1: one value on plane k = 1 for all three) and constant buoyancy."""
    for fid, v in ((F.M_C66XY, c66), (F.M_C55XZ, c55), (F.M_C44YZ, c44)):
        a = np.full(F.shape(fid, m.nx, m.ny, m.nz), v, np.float32)
        if plane1 is not None:
            a[1] = plane1
        m.materials[fid] = a
    for fid in (F.M_BX, F.M_BY, F.M_BZ):
        m.materials[fid] = np.full(F.shape(fid, m.nx, m.ny, m.nz), b, np.float32)
    return m


def ok2_case(nx=36, ny=40, nz=26, nt=60, seed=28, zs=8):
    """The diff_BC_OK2 scheme: the 3-D-weight form with scalar moduli, no BC1, 1e-5 on plane 1."""
    m = I.random_small(F.MODEL_ISO_HET, nx, ny, nz, nt=nt, seed=seed, damping=F.DAMP_W3D)
    mu = float(np.float32(np.median(m.materials[F.M_C66XY][m.materials[F.M_C66XY] > 0])))
    constant_moduli(m, mu, mu, mu, float(np.float32(1 / 2500.0)), plane1=1e-5)
    m.free_surface = F.FS_NONE
    m.set_moment_tensor(FULL_FAMILY_MT, nx // 2 - 3, ny // 2 - 3, zs, 0)
    m.meta = dict(m.meta or {}, scheme="ok2")
    return m


def full_case(nx=36, ny=40, nz=26, nt=60, seed=29, zs=8):
    """The FULL scheme: the 3-D-weight form with scalar c66 / c55 / c44, BC1, source kernel after it."""
    m = I.random_small(F.MODEL_ISO_HET, nx, ny, nz, nt=nt, seed=seed, damping=F.DAMP_W3D, src_order=F.SRC_AFTER_BC1)
    mu = float(np.median(m.materials[F.M_C66XY][m.materials[F.M_C66XY] > 0]))
    constant_moduli(m, float(np.float32(mu)), float(np.float32(0.9 * mu)), float(np.float32(1.1 * mu)),
                    float(np.float32(1 / 2600.0)))
    m.set_moment_tensor(FULL_FAMILY_MT, nx // 2 - 3, ny // 2 - 3, zs, 0)
    m.meta = dict(m.meta or {}, scheme="full")
    return m


@pytest.mark.parametrize("make", [iso_case, ortho_case, lambda: iso_case(zs=1), lambda: ortho_case(zs=0),
                                  lambda: ortho_case(damping=F.DAMP_SEPARABLE), isohet_case,
                                  lambda: isohet_case(zs=0, damping=F.DAMP_SEPARABLE), lambda: isohet_case(vdamp=True),
                                  dcq_case, lambda: dcq_case(zs=1), ok3_case, lambda: ok3_case(zs=0), ok2_case,
                                  lambda: ok2_case(zs=0), full_case, lambda: full_case(zs=0)],
                         ids=["iso", "ortho", "iso-surface-src", "ortho-surface-src", "ortho-separable", "iso9km",
                              "iso9km-surface-separable", "iso16km", "dcq", "dcq-surface-src", "ok3-no-bc1",
                              "ok3-surface-src", "ok2-no-bc1", "ok2-surface-src", "full", "full-surface-src"])
def test_product_bitwise_vs_reference_exact(cuda_device, make):
    m = make()
    rf, rt = reference(m, m.nt, "exact")
    with Solver.from_model(m) as s:
        s.run(m.nt)
        pf = [s.field(q) for q in F.STATE]
        pt = s.seismograms()
    of = O.run(m, m.nt)
    for q in F.STATE:
        mk = edge_mask(q, rf[q].shape)
        np.testing.assert_array_equal(pf[q][mk], rf[q][mk], err_msg=f"product vs reference {F.STATE_NAMES[q]}")
        np.testing.assert_array_equal(of.f[q][mk], rf[q][mk], err_msg=f"oracle vs reference {F.STATE_NAMES[q]}")
    np.testing.assert_array_equal(pt, rt)
    assert np.abs(rt).max() > 0


@pytest.mark.parametrize("model", [F.MODEL_ISO, F.MODEL_ORTHO, F.MODEL_ISO_HET, -1, -2, -3],
                         ids=["iso", "ortho", "iso16km", "dcq", "ok3", "ok2"])
def test_seismograms_vs_reference_stock_build(cuda_device, model):
    """North-star criterion: relative L2 seismogram error <= 1e-4 against the reference built with
    its own flags (FMA contraction on), after the full run."""
    if model == F.MODEL_ISO:
        m = I.iso_homogeneous(n=64, nt=400)
        c = 31
        m.set_moment_tensor(I.mt_strike_dip_rake(30, 60, 90), c, c, c, 0)
    elif model == F.MODEL_ORTHO:
        m = I.ortho_layered(nx=64, ny=64, nz=48, nt=400, src=(32, 32, 12), rec_coords=[8, 20, 32, 44, 56],
                            damping=F.DAMP_W3D)
        m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), 31, 31, 11, 1)
    elif model == F.MODEL_ISO_HET:
        m = isohet_case(nx=64, ny=64, nz=48, nt=400, seed=24, zs=11, vdamp=True)
    elif model == -1:
        m = dcq_case(nx=64, ny=64, nz=48, nt=400, seed=26, zs=11)
    elif model == -2:
        m = ok3_case(nx=64, ny=64, nz=48, nt=400, seed=30, zs=11)
    else:
        m = ok2_case(nx=64, ny=64, nz=48, nt=400, seed=31, zs=11)
    _, rt = reference(m, m.nt, "stock")
    with Solver.from_model(m) as s:
        s.run(m.nt)
        pt = s.seismograms()
    worst = 0.0
    for r in range(len(rt)):
        nrm = np.linalg.norm(rt[r])
        if nrm == 0:
            assert np.linalg.norm(pt[r]) == 0
            continue
        worst = max(worst, np.linalg.norm(pt[r] - rt[r]) / nrm)
    assert worst <= 1e-4, worst
