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
    assert R.available(m.model, variant, vd, m.damping), \
        f"missing {R.cubin(m.model, variant, vd, m.damping)}: run oracle/build.py where the reference is"
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


@pytest.mark.parametrize("make", [iso_case, ortho_case, lambda: iso_case(zs=1), lambda: ortho_case(zs=0),
                                  lambda: ortho_case(damping=F.DAMP_SEPARABLE), isohet_case,
                                  lambda: isohet_case(zs=0, damping=F.DAMP_SEPARABLE), lambda: isohet_case(vdamp=True),
                                  dcq_case, lambda: dcq_case(zs=1)],
                         ids=["iso", "ortho", "iso-surface-src", "ortho-surface-src", "ortho-separable", "iso9km",
                              "iso9km-surface-separable", "iso16km", "dcq", "dcq-surface-src"])
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


@pytest.mark.parametrize("model", [F.MODEL_ISO, F.MODEL_ORTHO, F.MODEL_ISO_HET, -1], ids=["iso", "ortho", "iso16km", "dcq"])
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
    else:
        m = dcq_case(nx=64, ny=64, nz=48, nt=400, seed=26, zs=11)
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
