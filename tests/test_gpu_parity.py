"""Product kernels (libewfd.so on the GPU) against the CPU oracle.

The product's device code is built without FMA contraction and keeps the reference's operand
order, as does the oracle (gcc -ffp-contract=off): the FP32, FP32-compensated and FP64 runs must
agree BIT FOR BIT on every state field and every receiver sample.
"""
import os
import subprocess

import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300 import legacy as L
from elanfmt_gb300.solver import EwfError, Solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def product(m, nsteps, prec=F.PREC_F32, chunks=None, **kw):
    dt = np.float64 if prec == F.PREC_F64 else np.float32
    with Solver.from_model(m, precision=prec, **kw) as s:
        for n in (chunks or [nsteps]):
            s.run(n)
        return [s.field(q, dt) for q in F.STATE], s.seismograms()


def assert_bitwise(prod, ref, what=""):
    fields, traces = prod
    for q in F.STATE:
        a, b = fields[q], ref.f[q]
        if not np.array_equal(a, b):
            d = np.argwhere(a != b)
            raise AssertionError(f"{what} field {F.STATE_NAMES[q]}: {len(d)} cells differ, first {d[:3].tolist()} "
                                 f"{a[tuple(d[0])]} vs {b[tuple(d[0])]}")
    np.testing.assert_array_equal(traces, ref.traces, err_msg=f"{what} traces")
    assert np.abs(traces).max() > 0, "degenerate case: receivers saw nothing"


CASES = [
    ("iso", F.MODEL_ISO, None, 37, 41, 23),
    ("iso-ragged", F.MODEL_ISO, None, 33, 9, 31),
    ("ortho-w3d", F.MODEL_ORTHO, F.DAMP_W3D, 35, 40, 21),
    ("ortho-sep", F.MODEL_ORTHO, F.DAMP_SEPARABLE, 29, 30, 27),
]


FUSED = pytest.mark.parametrize("fused", [F.STEP_FUSED, F.STEP_SPLIT, F.STEP_WAVE], ids=["fused", "split", "wave"])
# step forms built for every model and damping
FORMS = pytest.mark.parametrize("form", [F.STEP_SPLIT, F.STEP_WAVE], ids=["split", "wave"])


@pytest.mark.parametrize("name,model,damping,nx,ny,nz", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F32_KAHAN, F.PREC_F64], ids=["f32", "kahan", "f64"])
@FUSED
def test_bitwise_vs_oracle(cuda_device, name, model, damping, nx, ny, nz, prec, fused):
    m = I.random_small(model, nx, ny, nz, nt=48, seed=nx * 7 + nz, damping=damping)
    ref = O.run(m, 48, prec)
    assert_bitwise(product(m, 48, prec, fused=fused), ref, name)


ISOHET_CASES = [
    ("isohet-w3d", F.DAMP_W3D, 35, 40, 21),
    ("isohet-sep", F.DAMP_SEPARABLE, 29, 30, 27),
]


@pytest.mark.parametrize("name,damping,nx,ny,nz", ISOHET_CASES, ids=[c[0] for c in ISOHET_CASES])
@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F32_KAHAN, F.PREC_F64], ids=["f32", "kahan", "f64"])
@FORMS
def test_isohet_bitwise_vs_oracle(cuda_device, name, damping, nx, ny, nz, prec, form):
    """The 9 km scheme (edge shear moduli, staggered buoyancy; not the one-pass step)."""
    m = I.random_small(F.MODEL_ISO_HET, nx, ny, nz, nt=48, seed=nx * 5 + nz, damping=damping)
    ref = O.run(m, 48, prec)
    assert_bitwise(product(m, 48, prec, fused=form), ref, name)


@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F32_KAHAN, F.PREC_F64], ids=["f32", "kahan", "f64"])
@pytest.mark.parametrize("nx,ny,nz", [(35, 40, 21), (29, 30, 27)])
@FORMS
def test_percomp_bitwise_vs_oracle(cuda_device, prec, nx, ny, nz, form):
    """The DC_Earthquake form: isotropic, one 3-D weight field per component, three shear moduli."""
    m = I.random_small(F.MODEL_ISO, nx, ny, nz, nt=48, seed=nx + 3 * nz, damping=F.DAMP_PERCOMP)
    ref = O.run(m, 48, prec)
    assert_bitwise(product(m, 48, prec, fused=form), ref, "percomp")


@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F32_KAHAN, F.PREC_F64], ids=["f32", "kahan", "f64"])
@FORMS
def test_free_surface_options_bitwise_vs_oracle(cuda_device, prec, form):
    """No BC1 (the diff_BC schemes), with and without a plane-1 shear modulus on the isotropic
    scheme, and no BC1 on the orthorhombic and 9 km schemes; sources on planes 0-2."""
    for model, damping, smu in ((F.MODEL_ISO, None, 1e-5), (F.MODEL_ISO, None, 0.0), (F.MODEL_ORTHO, F.DAMP_W3D, 0.0),
                                (F.MODEL_ISO_HET, F.DAMP_SEPARABLE, 0.0)):
        for zs in (0, 1, 6):
            m = I.random_small(model, 31, 27, 19, nt=36, seed=41 + zs, damping=damping)
            m.free_surface = F.FS_NONE
            m.surface_mu = smu
            m.set_moment_tensor(np.array([0.3, -0.7, 1.1, 0.4, 1.0, 0.8]), 12, 11, zs, 0)
            ref = O.run(m, 36, prec)
            assert_bitwise(product(m, 36, prec, fused=form), ref, f"model {model} smu {smu} zs {zs}")
    m = I.random_small(F.MODEL_ISO, 31, 27, 19, nt=36, seed=47)
    m.surface_mu = 2e3                 # with BC1 on
    assert_bitwise(product(m, 36, prec, fused=form), O.run(m, 36, prec), "plane-1 modulus with BC1")


def test_free_surface_options_are_checked(cuda_device):
    m = I.random_small(F.MODEL_ORTHO, 24, 24, 16, nt=4, seed=3, damping=F.DAMP_W3D)
    m.surface_mu = 1e-5
    with pytest.raises(EwfError) as e:
        Solver.from_model(m)
    assert e.value.status == -8
    m = I.random_small(F.MODEL_ISO, 24, 24, 16, nt=4, seed=3)
    m.free_surface = F.FS_NONE
    with pytest.raises(EwfError) as e:
        Solver.from_model(m, fused=F.STEP_FUSED)
    assert e.value.status == -8
    m.free_surface = 7
    with pytest.raises(EwfError) as e:
        Solver.from_model(m)
    assert e.value.status == -1


@pytest.mark.parametrize("model", [F.MODEL_ORTHO, F.MODEL_ISO_HET], ids=["ortho", "isohet"])
@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F64], ids=["f32", "f64"])
@FORMS
def test_velocity_damping_bitwise_vs_oracle(cuda_device, model, prec, form):
    """Linear velocity damping of the 16 km scheme (V -= vdamp * V_old after each update)."""
    m = I.random_small(model, 31, 28, 22, nt=40, seed=9, damping=F.DAMP_W3D)
    m.vdamp = F.VDAMP_16KM
    ref = O.run(m, 40, prec)
    assert_bitwise(product(m, 40, prec, fused=form), ref, "vdamp")
    m.vdamp = 0.0
    undamped = O.run(m, 40, prec)
    assert not np.array_equal(undamped.traces, ref.traces)


def test_isohet_and_vdamp_limits(cuda_device):
    m = I.random_small(F.MODEL_ISO_HET, 20, 20, 16, nt=10, seed=1)
    with pytest.raises(EwfError) as e:
        Solver.from_model(m, fused=True)
    assert e.value.status == -8
    m = I.random_small(F.MODEL_ISO, 20, 20, 16, nt=10, seed=1)
    m.vdamp = 0.001
    with pytest.raises(EwfError) as e:
        Solver.from_model(m)
    assert e.value.status == -8


@pytest.mark.parametrize("order", [F.SRC_BEFORE_BC1, F.SRC_AFTER_BC1])
@pytest.mark.parametrize("stencil", [0, 1])
@pytest.mark.parametrize("zs", [0, 1, 5])
@FUSED
def test_source_next_to_free_surface(cuda_device, order, stencil, zs, fused):
    """Injection on planes 1-2 interacts with BC1 (before-BC1 order drops / propagates it)."""
    for model in (F.MODEL_ISO, F.MODEL_ORTHO):
        m = I.random_small(model, 24, 26, 18, nt=30, seed=3 + zs, src_order=order, stencil=stencil)
        m.set_moment_tensor(np.array([1.0, -0.5, 0.25, 0.7, -0.9, 1.3]), 10, 11, zs, stencil)
        ref = O.run(m, 30)
        assert_bitwise(product(m, 30, fused=fused), ref, f"model {model} order {order} stencil {stencil} zs {zs}")


@FUSED
def test_sources_on_tile_edges(cuda_device, fused):
    """Point sources on the cells a CTA recomputes as halo (tile borders, chunk borders), with
    several entries on one cell, in both injection orders."""
    for model in (F.MODEL_ISO, F.MODEL_ORTHO):
        for order in (F.SRC_BEFORE_BC1, F.SRC_AFTER_BC1):
            m = I.random_small(model, 70, 20, 40, nt=25, seed=17, src_order=order)
            ent, coef = [], []
            rng = np.random.default_rng(1)
            for comp in range(3, 9):
                for (i, j, k) in ((31, 7, 1), (32, 8, 2), (31, 8, 15), (32, 7, 16), (63, 15, 17), (64, 16, 1),
                                  (1, 1, 2), (0, 0, 31)):
                    ent.append((comp, i, j, k))
                    coef.append(rng.normal())
            ent = ent[:62] + [ent[0], ent[1]]
            coef = coef[:62] + [0.5, -0.25]
            m.sources = np.array(ent, np.int32)
            m.source_coef = np.array(coef)
            ref = O.run(m, 25)
            assert_bitwise(product(m, 25, fused=fused, kchunk=16), ref, f"model {model} order {order}")


@pytest.mark.parametrize("kchunk,graph_steps", [(4, -1), (7, 5), (16, 0), (64, 64), (5, 3)])
@FUSED
def test_tiling_and_graph_do_not_change_results(cuda_device, kchunk, graph_steps, fused):
    m = I.random_small(F.MODEL_ORTHO, 40, 33, 29, nt=40, seed=11, damping=F.DAMP_SEPARABLE)
    ref = O.run(m, 40)
    assert_bitwise(product(m, 40, kchunk=kchunk, graph_steps=graph_steps, chunks=[13, 20, 7], fused=fused), ref)


def test_wave_scheduler_settings(cuda_device):
    """The wavefront step on a grid with hundreds of items per step (many CTAs in flight, velocity
    items waiting on stress items): every lag and slab depth gives the oracle's bits, with
    sources on tile and slab borders, and the autotuner's pick as well."""
    m = I.random_small(F.MODEL_ORTHO, 100, 72, 48, nt=30, seed=23, damping=F.DAMP_W3D)
    ent, coef = [], []
    for comp in range(3, 9):
        for (i, j, k) in ((31, 7, 3), (32, 8, 4), (64, 16, 7), (63, 15, 8), (99, 71, 2), (10, 40, 47)):
            ent.append((comp, i, j, k))
            coef.append(0.1 * (comp - 5) + 0.01 * i)
    m.sources = np.array(ent, np.int32)
    m.source_coef = np.array(coef)
    ref = O.run(m, 30)
    for lag in (1, 100, 100000):
        for kchunk in (4, 7):
            with Solver.from_model(m, fused=F.STEP_WAVE, kchunk=kchunk, graph_steps=8) as s:
                s.set_wave(lag)
                assert s.wave_lag() == lag
                s.run(30)
                got = ([s.field(q, np.float32) for q in F.STATE], s.seismograms())
            assert_bitwise(got, ref, f"lag {lag} kchunk {kchunk}")
    with Solver.from_model(m, fused=F.STEP_WAVE) as s:
        s.autotune(4)
        s.run(30)
        got = ([s.field(q, np.float32) for q in F.STATE], s.seismograms())
    assert_bitwise(got, ref, "autotuned")
    with Solver.from_model(m) as s, pytest.raises(EwfError) as e:
        s.set_wave(100)
    assert e.value.status == -5


def test_wave_wait_gives_up_and_handle_recovers(cuda_device):
    """A done flag that nothing sets (withheld by the diagnostic hook): the velocity items waiting
    for it give up after their bounded wait, ewf_run reports the failure instead of hanging, and
    after a reset the same handle runs bit-exact again."""
    m = I.random_small(F.MODEL_ORTHO, 64, 48, 24, nt=12, seed=31, damping=F.DAMP_W3D)
    ref = O.run(m, 12)
    with Solver.from_model(m, fused=F.STEP_WAVE, kchunk=4, graph_steps=-1) as s:
        s.wave_hold(7)
        with pytest.raises(EwfError) as e:
            s.run(2)
        assert e.value.status == -2 and "gave up" in str(e.value)
        s.wave_hold(-1)
        s.reset()
        s.run(12)
        got = ([s.field(q, np.float32) for q in F.STATE], s.seismograms())
    assert_bitwise(got, ref, "after recovery")


@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F32_KAHAN, F.PREC_F64], ids=["f32", "kahan", "f64"])
def test_split_tile_heights(cuda_device, prec):
    """The two-kernel step over its CTA tile heights (rows of 32 columns) and the autotuner's
    pick of z-chunk and height: every setting gives the oracle's bits, on grids whose extents
    are not multiples of the tile."""
    heights = (1, 2, 4, 8, 16) if prec != F.PREC_F64 else (1, 2, 4, 8)
    for model, damping, shape in ((F.MODEL_ORTHO, F.DAMP_SEPARABLE, (35, 37, 21)), (F.MODEL_ISO, None, (33, 19, 17))):
        m = I.random_small(model, *shape, nt=20, seed=53, damping=damping)
        ref = O.run(m, 20, prec)
        dt = np.float64 if prec == F.PREC_F64 else np.float32
        for ty in heights:
            with Solver.from_model(m, precision=prec, kchunk=6, graph_steps=4) as s:
                s.set_tile(ty)
                s.set_l2_prefetch(ty % 5)  # the L2 hint off and on (1-4 planes ahead)
                assert s.tile() == ty and s.l2_prefetch() == ty % 5
                s.run(20)
                got = ([s.field(q, dt) for q in F.STATE], s.seismograms())
            assert_bitwise(got, ref, f"model {model} tile height {ty}")
        with Solver.from_model(m, precision=prec) as s:
            s.autotune(3)
            assert s.tile() in (4, 8, 16)
            s.run(20)
            got = ([s.field(q, dt) for q in F.STATE], s.seismograms())
        assert_bitwise(got, ref, f"model {model} autotuned")
    m = I.random_small(F.MODEL_ORTHO, 24, 24, 16, nt=4, seed=3, damping=F.DAMP_W3D)
    with Solver.from_model(m, precision=prec) as s:
        for bad in (0, 3, 32):
            with pytest.raises(EwfError) as e:
                s.set_tile(bad)
            assert e.value.status == -1
        if prec == F.PREC_F64:
            with pytest.raises(EwfError):
                s.set_tile(16)
    with Solver.from_model(m, fused=F.STEP_WAVE) as s, pytest.raises(EwfError) as e:
        s.set_tile(4)
    assert e.value.status == -5


def border_source_case():
    """A grid of a few hundred CTAs with point sources on tile and chunk borders, on several
    entries of one cell, and on cells the stress pass never updates (sxy at i = nx and at i = 0,
    sxz and syz on plane nz): their values are carried over from the previous step."""
    m = I.random_small(F.MODEL_ORTHO, 100, 72, 40, nt=24, seed=29, damping=F.DAMP_W3D, src_order=F.SRC_BEFORE_BC1)
    ent, coef = [], []
    for comp in range(3, 9):
        for (i, j, k) in ((31, 0, 3), (32, 0, 4), (99, 2, 2), (0, 3, 1), (50, 40, 20), (51, 40, 2), (50, 41, 39)):
            ent.append((comp, i, j, k))
            coef.append(0.1 * (comp - 5) + 0.01 * i + 0.001 * k)
    ent += [(6, 100, 5, 3), (7, 100, 4, 40), (8, 3, 72, 40), (6, 0, 9, 6), (6, 0, 9, 6), (5, 50, 40, 20)]
    coef += [0.3, -0.2, 0.7, 0.5, 0.25, -1.5]
    m.sources = np.array(ent, np.int32)
    m.source_coef = np.array(coef)
    return m


def test_split_step_dependent_launches(cuda_device):
    """Programmatic dependent launches (default) and plain launches give the same bits, in the
    captured graph and on the direct path (steps left over after the graph launches)."""
    m = I.random_small(F.MODEL_ORTHO, 35, 37, 21, nt=30, seed=57, damping=F.DAMP_SEPARABLE)
    ref = O.run(m, 30)
    for on in (True, False):
        with Solver.from_model(m, kchunk=6, graph_steps=8) as s:
            assert s.dependent_launch()
            s.set_dependent_launch(on)
            s.run(30)
            assert s.dependent_launch() == on
            got = ([s.field(q, np.float32) for q in F.STATE], s.seismograms())
        assert_bitwise(got, ref, f"dependent launches {on}")


@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F32_KAHAN, F.PREC_F64], ids=["f32", "kahan", "f64"])
def test_split_step_receivers_in_the_velocity_kernel(cuda_device, tmp_path, prec):
    """The two-kernel step samples receivers in the velocity kernel and advances its step counter
    there (two launches per step) when every receiver is a velocity component on a cell its
    threads visit, with k_record otherwise; both give the oracle's bits -- receivers on the planes
    the update leaves unchanged (vx at j = ny-1, vz at k = nz-1), two on one column, odd run
    lengths around the graph (the counter alternates between two locations), and a checkpoint
    taken at an odd step."""
    dt = np.float64 if prec == F.PREC_F64 else np.float32
    m = I.random_small(F.MODEL_ORTHO, 35, 37, 21, nt=40, seed=61, damping=F.DAMP_SEPARABLE)
    inside = np.array([[5, 6, 1, F.F_VZ], [5, 6, 7, F.F_VX], [34, 20, 3, F.F_VY], [12, 36, 2, F.F_VX],
                       [17, 18, 20, F.F_VZ], [1, 1, 1, F.F_VY]], np.int32)
    outside = [np.array([[5, 0, 1, F.F_VX]], np.int32), np.array([[5, 6, 0, F.F_VZ]], np.int32),
               np.array([[5, 6, 3, F.F_SXY]], np.int32)]
    for rec, launches in [(inside, 2)] + [(np.concatenate([inside, o]), 3) for o in outside]:
        m.receivers = rec
        ref = O.run(m, 40, prec)
        with Solver.from_model(m, precision=prec, kchunk=6, graph_steps=8) as s:
            assert s.launches_per_step() == launches
            for n in (3, 13, 5, 11, 8):  # graph launches start at odd and even steps
                s.run(n)
            got = ([s.field(q, dt) for q in F.STATE], s.seismograms())
        assert_bitwise(got, ref, f"{len(rec)} receivers")
    m.receivers = inside
    ref = O.run(m, 40, prec)
    ck = str(tmp_path / "odd.ckpt")
    with Solver.from_model(m, precision=prec, kchunk=6, graph_steps=8) as s:
        s.run(17)
        s.checkpoint(ck)
    with Solver.from_model(m, precision=prec, kchunk=6, graph_steps=8) as s:
        s.restore(ck)
        s.run(23)
        got = ([s.field(q, dt) for q in F.STATE], s.seismograms())
    assert_bitwise(got, ref, "resumed at an odd step")


@pytest.mark.parametrize("order", [F.SRC_BEFORE_BC1, F.SRC_AFTER_BC1], ids=["before-bc1", "after-bc1"])
def test_split_step_sources_in_the_stress_kernel(cuda_device, order):
    """The two-kernel step applies point sources in the stress kernel's owning threads when every
    entry lies in its cells (no k_inject launch), and falls back to k_inject otherwise; both give
    the oracle's bits -- entries on planes 0-2 (BC1), on chunk borders, several on one cell, and on
    cells the stress update leaves unchanged."""
    m = border_source_case()
    m.src_order = order
    inside = [q for q in range(len(m.sources))
              if m.sources[q][1] < m.nx and m.sources[q][2] < m.ny and m.sources[q][3] < m.nz]
    assert len(inside) < len(m.sources)
    for sel, launches in ((list(range(len(m.sources))), 3), (inside, 2)):
        mm = border_source_case()
        mm.src_order = order
        mm.sources, mm.source_coef = m.sources[sel], m.source_coef[sel]
        ref = O.run(mm, 24)
        with Solver.from_model(mm, kchunk=4, graph_steps=6) as s:
            assert s.launches_per_step() == launches
            s.run(24)
            got = ([s.field(q, np.float32) for q in F.STATE], s.seismograms())
        assert_bitwise(got, ref, f"{len(sel)} entries")


@pytest.mark.parametrize("form", [F.STEP_SPLIT, F.STEP_WAVE], ids=["split", "wave"])
def test_workload_shapes_small(cuda_device, form):
    """The two benchmark workloads at reduced size, FP32, bit-exact."""
    m = I.iso_homogeneous(n=48, nt=120)
    assert_bitwise(product(m, 120, fused=form), O.run(m, 120), "iso48")
    m = I.ortho_layered(nx=48, ny=48, nz=40, nt=60, src=(24, 24, 4), rec_coords=[4, 20, 40])
    assert_bitwise(product(m, 60, fused=form), O.run(m, 60), "ortho48")


def test_reset_restart_and_checkpoint(cuda_device, tmp_path):
    m = I.random_small(F.MODEL_ISO, 30, 30, 20, nt=50, seed=5)
    ref = O.run(m, 50)
    with Solver.from_model(m) as s:
        s.run(20)
        ck = str(tmp_path / "run.ckpt")
        s.checkpoint(ck)
        s.run(30)
        full = ([s.field(q) for q in F.STATE], s.seismograms())
        assert_bitwise(full, ref, "uninterrupted")
        s.reset()
        assert s.step() == 0
        assert np.abs(s.field(F.F_VX)).max() == 0
        s.restore(ck)
        assert s.step() == 20
        s.run(30)
        assert_bitwise(([s.field(q) for q in F.STATE], s.seismograms()), ref, "resumed")
    # a fresh handle restored from the file resumes bit-exactly too
    with Solver.from_model(m) as s2:
        s2.restore(ck)
        s2.run(30)
        assert_bitwise(([s2.field(q) for q in F.STATE], s2.seismograms()), ref, "resumed in new handle")


def test_errors_are_status_codes(cuda_device):
    m = I.random_small(F.MODEL_ISO, 20, 20, 16, nt=10, seed=1)
    with Solver.from_model(m) as s:
        with pytest.raises(EwfError) as e:
            s.run(11)  # past nt
        assert e.value.status == -1
        with pytest.raises(EwfError):
            s.set_field(F.M_C11, np.zeros((3, 3, 3), np.float32))
        with pytest.raises(EwfError):
            s.set_receivers(np.array([[20, 0, 0, 0]]))  # Vx has nx+1 = 21 cells in x: ok
            s.set_receivers(np.array([[21, 0, 0, 0]]))
        with pytest.raises(EwfError):
            s.set_sources(np.array([[0, 1, 1, 1]]), np.array([1.0]))  # not a stress field
    m.materials[F.M_C11] = m.materials[F.M_C11].copy()
    m.materials[F.M_C11][1, 10, 10] = np.nan  # next to the receiver at (10, 10, 1)
    with Solver.from_model(m) as s:
        with pytest.raises(EwfError) as e:
            s.run(10)
        assert e.value.status == -7  # non-finite traces detected on the host
    with Solver.from_model(m, check_finite=False) as s:
        s.run(10)
        tr = s.seismograms()
    bad = ~np.isfinite(tr)
    t_star = int(np.nonzero(bad.any(axis=0))[0][0])  # first step with a non-finite sample
    if t_star > 0:  # the check covers the samples of each call: a later call reports them
        r0 = int(np.nonzero(bad[:, t_star:].any(axis=1))[0][0])
        t0 = t_star + int(np.nonzero(bad[r0, t_star:])[0][0])
        with Solver.from_model(m) as s:
            s.run(t_star)
            with pytest.raises(EwfError) as e:
                s.run(10 - t_star)
            assert e.value.status == -7
            assert f"receiver {r0} has a non-finite sample at step {t0}" in str(e.value)
    # inputs missing
    with Solver.from_model(I.random_small(F.MODEL_ISO, 20, 20, 16, nt=10, seed=1)) as s0:
        params = s0.params
    with Solver(params) as s:
        with pytest.raises(EwfError) as e:
            s.run(1)
        assert e.value.status == -5


def test_legacy_file_contract_through_ewfd(cuda_device, tmp_path):
    """MATLAB-style inputs in, ewfd run, 0_infos.inf + 0_0_*.res out; compared with the oracle."""
    m = I.random_small(F.MODEL_ISO, 40, 44, 24, nt=40, seed=9)
    xs, ys, zs = 12, 13, 9
    m.set_moment_tensor(np.array([0.5, -1.0, 0.3, 0.2, 1.0, 0.8]), xs, ys, zs, 0)
    m.receivers = np.array([[30, 20, 1, F.F_VZ], [30, 20, 1, F.F_VX], [30, 23, 1, F.F_VY], [30, 22, 1, F.F_VY],
                            [5, 6, 7, F.F_VZ]], np.int32)
    L.write_inputs(m, str(tmp_path))
    with open(tmp_path / "rec.txt", "w") as fh:
        for r in m.receivers:
            fh.write(" ".join(str(int(v)) for v in r) + "\n")
    exe = os.path.join(ROOT, "elanfmt_gb300", "ewfd")
    r = subprocess.run([exe, "--nx", "40", "--ny", "44", "--nz", "24", "--workdir", str(tmp_path), "--src",
                        f"{xs},{ys},{zs}", "--receivers", str(tmp_path / "rec.txt"), "--quiet"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = L.read_outputs(str(tmp_path), m.nt)
    assert out["PRECIS"] == 4 and (out["nx"], out["ny"], out["nz"]) == (40, 44, 24)
    ref = O.run(m, 40)
    np.testing.assert_array_equal(out["Vx"], ref.f[F.F_VX])
    np.testing.assert_array_equal(out["Vy"], ref.f[F.F_VY])
    np.testing.assert_array_equal(out["Vz"], ref.f[F.F_VZ])
    for q, name in enumerate(("Rec", "Rec_x", "Rec_y", "Rec_y2")):
        np.testing.assert_array_equal(out[name], ref.traces[q].astype(np.float32))
    np.testing.assert_array_equal(out["Rec_all"], ref.traces.astype(np.float32))
    np.testing.assert_array_equal(out["Src"], m.stf[: m.nt].astype(np.float32))
    # autotuned launch shapes (state reset after tuning): the same files, byte for byte
    names = [f for f in os.listdir(tmp_path) if f.endswith(".res")]
    before = {f: (tmp_path / f).read_bytes() for f in names}
    r = subprocess.run([exe, "--nx", "40", "--ny", "44", "--nz", "24", "--workdir", str(tmp_path), "--src",
                        f"{xs},{ys},{zs}", "--receivers", str(tmp_path / "rec.txt"), "--autotune", "6", "--quiet"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for f in names:
        assert (tmp_path / f).read_bytes() == before[f], f
    # the same through the Python mirror of the executable
    s = Solver.legacy(str(tmp_path), 40, 44, 24)
    try:
        s.set_moment_tensor(np.fromfile(tmp_path / "MTS.dat", np.float32).astype(np.float64), xs, ys, zs, 0)
        s.set_receivers(m.receivers)
        s.run(40)
        np.testing.assert_array_equal(s.seismograms(), ref.traces)
    finally:
        s.close()


@pytest.mark.parametrize("flag,model,damping", [("ortho", F.MODEL_ORTHO, F.DAMP_W3D),
                                                ("isohet", F.MODEL_ISO_HET, F.DAMP_W3D),
                                                ("dcq", F.MODEL_ISO, F.DAMP_PERCOMP)])
def test_legacy_file_contract_other_schemes(cuda_device, tmp_path, flag, model, damping):
    """The orthorhombic, 9 km and DC_Earthquake file sets through `ewfd --model ...`."""
    m = I.random_small(model, 40, 44, 24, nt=40, seed=19, damping=damping)
    xs, ys, zs = 12, 13, 9
    m.set_moment_tensor(np.array([0.5, -1.0, 0.3, 0.2, 1.0, 0.8]), xs, ys, zs, 1)
    m.receivers = np.array([[30, 20, 1, F.F_VZ], [30, 20, 1, F.F_VX], [30, 23, 1, F.F_VY], [30, 22, 1, F.F_VY],
                            [5, 6, 7, F.F_VZ]], np.int32)
    L.write_inputs(m, str(tmp_path))
    with open(tmp_path / "rec.txt", "w") as fh:
        for r in m.receivers:
            fh.write(" ".join(str(int(v)) for v in r) + "\n")
    exe = os.path.join(ROOT, "elanfmt_gb300", "ewfd")
    r = subprocess.run([exe, "--nx", "40", "--ny", "44", "--nz", "24", "--model", flag, "--workdir", str(tmp_path),
                        "--src", f"{xs},{ys},{zs}", "--receivers", str(tmp_path / "rec.txt"), "--quiet"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = L.read_outputs(str(tmp_path), m.nt)
    ref = O.run(m, 40)
    for q, name in ((F.F_VX, "Vx"), (F.F_VY, "Vy"), (F.F_VZ, "Vz")):
        np.testing.assert_array_equal(out[name], ref.f[q])
    np.testing.assert_array_equal(out["Rec_all"], ref.traces.astype(np.float32))


def test_legacy_file_contract_without_free_surface(cuda_device, tmp_path):
    """The diff_BC2_OK3 scheme through the executable: the isotropic file set with
    `--free-surface none --surface-mu 1e-5` (no BC1, shear modulus 1e-5 on plane 1)."""
    m = I.random_small(F.MODEL_ISO, 40, 44, 24, nt=40, seed=21)
    m.free_surface = F.FS_NONE
    m.surface_mu = 1e-5
    xs, ys, zs = 12, 13, 1
    m.set_moment_tensor(np.array([0.0, 0.0, 0.0, 0.0, 1.0, 0.8]), xs, ys, zs, 0)
    m.receivers = np.array([[30, 20, 1, F.F_VZ], [30, 20, 1, F.F_VX], [30, 23, 1, F.F_VY], [30, 22, 1, F.F_VY]],
                           np.int32)
    L.write_inputs(m, str(tmp_path))
    with open(tmp_path / "rec.txt", "w") as fh:
        for r in m.receivers:
            fh.write(" ".join(str(int(v)) for v in r) + "\n")
    exe = os.path.join(ROOT, "elanfmt_gb300", "ewfd")
    r = subprocess.run([exe, "--nx", "40", "--ny", "44", "--nz", "24", "--workdir", str(tmp_path), "--src",
                        f"{xs},{ys},{zs}", "--receivers", str(tmp_path / "rec.txt"), "--free-surface", "none",
                        "--surface-mu", "1e-5", "--quiet"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = L.read_outputs(str(tmp_path), m.nt)
    ref = O.run(m, 40)
    for q, name in ((F.F_VX, "Vx"), (F.F_VY, "Vy"), (F.F_VZ, "Vz")):
        np.testing.assert_array_equal(out[name], ref.f[q])
    for q, name in enumerate(("Rec", "Rec_x", "Rec_y", "Rec_y2")):
        np.testing.assert_array_equal(out[name], ref.traces[q].astype(np.float32))
    bad = subprocess.run([exe, "--nx", "40", "--ny", "44", "--nz", "24", "--workdir", str(tmp_path),
                          "--free-surface", "sometimes", "--quiet"], capture_output=True, text=True)
    assert bad.returncode == 1 and "--free-surface" in bad.stderr


def test_async_snapshots_are_the_fields_at_their_step(cuda_device, tmp_path):
    """Queued snapshots (device copy in stream order, D2H on a second stream, files by a library
    thread) hold the fields of the step they were requested at, while later steps run; three
    requests in a row exercise the wait for a free slot."""
    m = I.random_small(F.MODEL_ORTHO, 30, 28, 22, nt=60, seed=4, damping=F.DAMP_W3D)
    want = {}
    with Solver.from_model(m, workdir=str(tmp_path)) as s:
        for isave in (1, 2, 3):
            s.run(12)
            s.write_snapshot(isave, wait=False)
            want[isave] = [s.field(q) for q in (F.F_VX, F.F_VY, F.F_VZ)]
        s.write_snapshot(4, wait=False)
        s.write_snapshot(5, wait=True)  # the synchronous form of the same step
        s.run(12)
        s.snapshot_wait()
    for isave, fields in want.items():
        for name, f in zip(("Vx", "Vy", "Vz"), fields):
            got = np.fromfile(tmp_path / f"{isave}_0_{name}.res", np.float32).reshape(f.shape)
            np.testing.assert_array_equal(got, f, err_msg=f"snapshot {isave} {name}")
    for name in ("Vx", "Vy", "Vz"):
        a = np.fromfile(tmp_path / f"4_0_{name}.res", np.float32)
        b = np.fromfile(tmp_path / f"5_0_{name}.res", np.float32)
        np.testing.assert_array_equal(a, b)
    assert np.abs(want[3][2]).max() > 0
