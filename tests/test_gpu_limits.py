"""Edge cases of size: empty inputs (no source, no receivers, one step) and a grid whose fields
exceed 2^31 elements (64-bit indexing, ~100 GB of device memory)."""
import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300.solver import EwfError, Solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_no_source_no_receivers_one_step(cuda_device):
    for model in (F.MODEL_ISO, F.MODEL_ORTHO, F.MODEL_ISO_HET):
        m = I.random_small(model, 20, 18, 16, nt=5, seed=2)
        m.sources = np.zeros((0, 4), np.int32)
        m.source_coef = np.zeros(0)
        m.receivers = None
        with Solver.from_model(m) as s:
            s.run(1)
            s.run(4)
            assert all(np.abs(s.field(q)).max() == 0 for q in F.STATE)
            assert s.seismograms().size == 0
        m.receivers = np.array([[3, 4, 5, 0]], np.int32)
        ref = O.run(m, 5)
        with Solver.from_model(m) as s:
            s.run(5)
            np.testing.assert_array_equal(s.seismograms(), ref.traces)


def _corner_model(n: int, nt: int) -> "I.Model":
    """Homogeneous isotropic grid, no damping, the source in the corner at cell 8: after nt steps
    the stencil has carried the wave at most nt cells, so two grids of different size agree
    exactly on the corner region while the larger one's far boundaries are never reached."""
    vp, vs, rho, dx = 6000.0, 3464.0, 2700.0, 50.0
    c11 = rho * vp * vp
    mu = rho * vs * vs
    dt = 0.5 * dx / (vp * np.sqrt(3.0))
    m = I.Model(nx=n, ny=n, nz=n, nt=nt, dx=dx, dy=dx, dz=dx, dt=float(np.float32(dt)), model=F.MODEL_ISO,
                damping=F.DAMP_PML1D, src_order=F.SRC_BEFORE_BC1, c66=float(np.float32(mu)),
                bx=float(np.float32(1 / rho)), by=float(np.float32(1 / rho)), bz=float(np.float32(1 / rho)))
    m.materials[F.M_C11] = np.full((n, n, n), c11, np.float32)
    m.materials[F.M_C12] = np.full((n, n, n), c11 - 2 * mu, np.float32)
    for key in (F.D_WX, F.D_WY, F.D_WZ):
        m.damping_arrays[key] = np.ones(n + 1, np.float32)
    m.set_moment_tensor(I.mt_strike_dip_rake(30, 60, 90), 8, 8, 8, stencil=0)
    m.stf = I.ricker_stf(nt, m.dt, 20.0, t0=0.0, scale=1e6)
    coords = range(1, 40, 6)
    m.receivers = np.array([(i, j, k, c) for k in coords for j in coords for i in coords for c in (0, 1, 2)], np.int32)
    return m


def test_field_above_2_31_elements_matches_small_grid(cuda_device):
    nt = 20
    small = _corner_model(64, nt)
    with Solver.from_model(small) as s:
        s.run(nt)
        want = s.seismograms()
    assert np.abs(want).max() > 0
    big = _corner_model(1280, nt)   # padded box ~2.2e9 elements per field, 11 fields
    try:
        s = Solver.from_model(big)
    except EwfError as e:
        if e.status == -3:
            pytest.skip("not enough free device memory for the 1280^3 case")
        raise
    with s:
        s.run(nt)
        got = s.seismograms()
    np.testing.assert_array_equal(got, want)
