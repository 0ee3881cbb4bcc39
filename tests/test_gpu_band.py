"""The band kernel of the one-pass step (one thread-block cluster per band of full-width rows,
stress edge columns exchanged through distributed shared memory) against the CPU oracle, bit for
bit: several CTAs per band (3 to 9, a ragged last CTA, the non-portable cluster size above 8),
ragged bands, z-chunks, sources on CTA and band borders and next to the free surface, and the
tile kernel it replaces on the same cases."""
import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300.solver import EwfError, Solver
from oracle import oracle as O

from .test_gpu_parity import assert_bitwise

pytestmark = pytest.mark.gpu

ERR_ARG, ERR_STATE, ERR_UNSUPPORTED = -1, -5, -8  # ewf_status


KERNEL = {0: F.ONEPASS_TILE, 4: F.ONEPASS_BAND4, 8: F.ONEPASS_BAND8}


def run_band(m, nsteps, rows, prec=F.PREC_F32, kchunk=0, chunks=None, graph_steps=0):
    dt = np.float64 if prec == F.PREC_F64 else np.float32
    with Solver.from_model(m, precision=prec, fused=F.STEP_FUSED, kchunk=kchunk, graph_steps=graph_steps) as s:
        s.set_onepass(KERNEL[rows])
        assert s.onepass() == KERNEL[rows]
        for n in (chunks or [nsteps]):
            s.run(n)
        return [s.field(q, dt) for q in F.STATE], s.seismograms()


CASES = [
    ("iso", F.MODEL_ISO, None, 150, 37, 20),
    ("ortho-w3d", F.MODEL_ORTHO, F.DAMP_W3D, 192, 30, 19),
    ("ortho-sep", F.MODEL_ORTHO, F.DAMP_SEPARABLE, 131, 26, 22),
]


@pytest.mark.parametrize("name,model,damping,nx,ny,nz", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("prec,rows", [(F.PREC_F32, 4), (F.PREC_F32, 8), (F.PREC_F32_KAHAN, 4), (F.PREC_F32_KAHAN, 8),
                                       (F.PREC_F64, 4)], ids=["f32-4", "f32-8", "kahan-4", "kahan-8", "f64-4"])
def test_band_bitwise_vs_oracle(cuda_device, name, model, damping, nx, ny, nz, prec, rows):
    m = I.random_small(model, nx, ny, nz, nt=24, seed=5, damping=damping)
    ref = O.run(m, 24, prec)
    assert_bitwise(run_band(m, 24, rows, prec, kchunk=8, chunks=[9, 15]), ref, f"{name} rows {rows}")


@pytest.mark.parametrize("rows", [0, 4, 8], ids=["tile", "band4", "band8"])
def test_band_chunks_and_graphs(cuda_device, rows):
    """z-chunks of every length (one chunk per plane range, the whole depth), graphs of odd and
    even lengths, runs that stop on odd steps: the band kernel and the tile kernel give the
    oracle's bits."""
    m = I.random_small(F.MODEL_ORTHO, 140, 21, 33, nt=30, seed=9, damping=F.DAMP_SEPARABLE)
    ref = O.run(m, 30)
    for kchunk, gs in ((4, -1), (11, 5), (33, 4), (64, 0)):
        assert_bitwise(run_band(m, 30, rows, kchunk=kchunk, graph_steps=gs, chunks=[7, 12, 11]), ref,
                       f"rows {rows} kchunk {kchunk} graph {gs}")


def test_band_nine_ctas(cuda_device):
    """576 columns = 9 CTAs per band: a cluster above the portable size of 8."""
    m = I.random_small(F.MODEL_ORTHO, 576, 13, 10, nt=12, seed=21, damping=F.DAMP_W3D)
    with Solver.from_model(m, fused=F.STEP_FUSED) as s:
        try:
            s.set_onepass(F.ONEPASS_BAND4)
        except EwfError:
            pytest.skip("no cluster of 9 CTAs fits this device")
    ref = O.run(m, 12)
    assert_bitwise(run_band(m, 12, 4, kchunk=5), ref, "nine CTAs")


@pytest.mark.parametrize("rows", [4, 8])
def test_band_sources_on_borders(cuda_device, rows):
    """Point sources on CTA borders (x = 63/64, 127/128), on the rows a band recomputes (j0-1,
    j0+rows), on chunk borders and on planes 0-2 under the free surface, several entries per cell,
    in both injection orders."""
    for model in (F.MODEL_ISO, F.MODEL_ORTHO):
        for order in (F.SRC_BEFORE_BC1, F.SRC_AFTER_BC1):
            m = I.random_small(model, 140, 3 * rows + 2, 24, nt=20, seed=31, src_order=order)
            ent, coef = [], []
            rng = np.random.default_rng(7)
            cells = ((63, rows - 1, 1), (64, rows, 2), (127, rows, 8), (128, 2 * rows - 1, 9), (63, 2 * rows, 0),
                     (64, rows - 1, 16), (1, 1, 2), (127, 0, 1), (128, 3 * rows, 2), (0, rows, 17))
            for comp in range(3, 9):
                for c in cells:
                    ent.append((comp,) + c)
                    coef.append(rng.normal())
            ent = ent[:60] + [ent[0], ent[7], ent[12], ent[25]]
            coef = coef[:60] + [0.5, -0.25, 0.75, 1.5]
            m.sources = np.array(ent, np.int32)
            m.source_coef = np.array(coef)
            ref = O.run(m, 20)
            assert_bitwise(run_band(m, 20, rows, kchunk=8), ref, f"rows {rows} model {model} order {order}")


def test_band_default_and_limits(cuda_device):
    """The tile kernel is the default; band heights are checked against the precision, the step
    form and the grid width."""
    m = I.random_small(F.MODEL_ORTHO, 96, 12, 8, nt=4, seed=2, damping=F.DAMP_W3D)
    with Solver.from_model(m, fused=F.STEP_FUSED) as s:
        assert s.onepass() == F.ONEPASS_TILE  # the tile kernel by default
        s.set_onepass(F.ONEPASS_BAND4)
        assert s.onepass() == F.ONEPASS_BAND4
        with pytest.raises(EwfError) as e:
            s.set_onepass(4)
        assert e.value.status == ERR_ARG
        s.set_onepass(F.ONEPASS_TILE)
        assert s.onepass() == F.ONEPASS_TILE
    with Solver.from_model(m, fused=F.STEP_FUSED, precision=F.PREC_F64) as s:
        with pytest.raises(EwfError) as e:
            s.set_onepass(F.ONEPASS_BAND8)  # FP64: 4 rows only
        assert e.value.status == ERR_UNSUPPORTED
        with pytest.raises(EwfError) as e:
            s.set_onepass(F.ONEPASS_STAGED)  # FP32 only
        assert e.value.status == ERR_UNSUPPORTED
    with Solver.from_model(m, fused=F.STEP_FUSED, precision=F.PREC_F32_KAHAN) as s:
        with pytest.raises(EwfError) as e:
            s.set_onepass(F.ONEPASS_STAGED)  # no compensation
        assert e.value.status == ERR_UNSUPPORTED
    with Solver.from_model(m) as s:  # two-kernel step
        with pytest.raises(EwfError) as e:
            s.set_onepass(F.ONEPASS_BAND4)
        assert e.value.status == ERR_STATE
    wide = I.random_small(F.MODEL_ORTHO, 1100, 4, 4, nt=2, seed=2, damping=F.DAMP_W3D)
    with Solver.from_model(wide, fused=F.STEP_FUSED) as s:  # 18 CTAs per band: not the band kernel
        with pytest.raises(EwfError) as e:
            s.set_onepass(F.ONEPASS_BAND4)
        assert e.value.status == ERR_UNSUPPORTED
        s.set_onepass(F.ONEPASS_STAGED)  # tiles: any width


def test_band_autotune_keeps_results(cuda_device):
    """The autotuner chooses among the tile, band and staged kernels; the pick gives the oracle's
    bits."""
    m = I.random_small(F.MODEL_ORTHO, 140, 24, 30, nt=24, seed=13, damping=F.DAMP_SEPARABLE)
    ref = O.run(m, 24)
    with Solver.from_model(m, fused=F.STEP_FUSED) as s:
        s.autotune(4)
        s.run(24)
        assert_bitwise(([s.field(q, np.float32) for q in F.STATE], s.seismograms()), ref, f"autotuned kernel {s.onepass()}")
