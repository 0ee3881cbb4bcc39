"""Seismogram error of the product against the reference's own kernels on the two benchmark
workloads, after the full run (the correctness bar: relative L2 <= 1e-4 for every trace).

The reference kernels are the "stock" build: compiled from the reference sources with the
reference's own flags (-O3, FMA contraction on) for sm_103a, replayed by oracle/refrun.py with
the loop order of the reference's main() (OK4:485-505, ANISO:519-555).

* isotropic homogeneous 128^3, dx 50 m, 1000 steps, double couple at the centre, 8 receivers on a
  2 km ring x 3 components (the OK4 scheme, its source stencil and injection order);
* orthorhombic layered 320 x 320 x 256, dx 40 m, 4000 steps, 64 receivers on an 8 x 8 surface
  grid x 3 components (the ANISO scheme).  The ANISO solver hard-codes its moment tensor
  (ANISO:233-247), so both codes run that tensor at the workload's source cell: the workload's
  own lune tensor cannot be handed to the reference kernels.
"""
import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300.solver import Solver
from oracle import refrun as R

pytestmark = pytest.mark.gpu

TOL = 1e-4


def iso128():
    return I.iso_homogeneous(n=128, nt=1000)


def ortho320():
    m = I.ortho_layered()
    xs, ys, zs = (int(v) - 1 for v in m.sources[0, 1:4])
    m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), xs, ys, zs, 1)
    return m


def reference_traces(m):
    assert R.available(m.model, "stock"), f"missing {R.cubin(m.model, 'stock')}: build oracle/ where the reference is"
    r = R.RefRunner(m, "stock")
    try:
        r.run(m.nt)
        return r.traces.copy()
    finally:
        r.close()


@pytest.mark.parametrize("make,step", [(iso128, F.STEP_SPLIT), (ortho320, F.STEP_SPLIT)],
                         ids=["iso128-1000steps", "ortho320x320x256-4000steps"])
def test_full_run_seismograms_vs_reference_stock(cuda_device, make, step):
    m = make()
    rt = reference_traces(m)
    with Solver.from_model(m, fused=step) as s:
        s.run(m.nt)
        pt = s.seismograms()
    err = R.trace_errors(pt, rt)
    print(f"{m.name}: {len(rt)} traces, max rel. L2 {err['max_rel_l2']:.3e}, median {err['median_rel_l2']:.3e}")
    assert np.abs(rt).max() > 0
    assert err["zero_mismatch"] == 0
    assert err["max_rel_l2"] <= TOL, err


@pytest.mark.parametrize("make", [iso128, ortho320], ids=["iso128-1000steps", "ortho320x320x256-4000steps"])
def test_step_forms_bit_identical_on_the_benchmark_workloads(cuda_device, make):
    """Every step form and one-pass kernel reproduces the two-kernel step bit for bit on the full
    benchmark workloads (so each meets the bar above), at the launch shapes of the autotuner's
    range: the band kernel's clusters span the whole x extent (2 and 5 CTAs) and the staged
    kernel's tiles are ragged on neither grid."""
    m = make()
    with Solver.from_model(m, fused=F.STEP_SPLIT) as s:
        s.run(m.nt)
        ref_traces = s.seismograms()
        ref_vz = s.field(F.F_VZ)
    assert np.abs(ref_traces).max() > 0
    for kernel, kchunk in ((F.ONEPASS_STAGED, 32), (F.ONEPASS_BAND4, 32), (F.ONEPASS_TILE, 16)):
        with Solver.from_model(m, fused=F.STEP_FUSED, kchunk=kchunk) as s:
            s.set_onepass(kernel)
            s.run(m.nt)
            np.testing.assert_array_equal(s.seismograms(), ref_traces, err_msg=f"one-pass kernel {kernel}")
            np.testing.assert_array_equal(s.field(F.F_VZ), ref_vz, err_msg=f"one-pass kernel {kernel}")
