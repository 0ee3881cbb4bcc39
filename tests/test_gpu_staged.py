"""The staged kernel of the one-pass step (planes of each 64 x 8 tile staged in shared memory by TMA,
the stress ring recomputed from the staged plane) against the CPU oracle, bit for bit: ragged
tiles in x and y, z-chunks of every length, graphs of odd and even lengths, runs stopping on odd
steps, sources on tile and chunk borders and next to the free surface in both injection orders."""
import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300.solver import Solver
from oracle import oracle as O

from .test_gpu_parity import assert_bitwise

pytestmark = pytest.mark.gpu


def run_staged(m, nsteps, kchunk=0, chunks=None, graph_steps=0):
    with Solver.from_model(m, fused=F.STEP_FUSED, kchunk=kchunk, graph_steps=graph_steps) as s:
        s.set_onepass(F.ONEPASS_STAGED)
        assert s.onepass() == F.ONEPASS_STAGED
        for n in (chunks or [nsteps]):
            s.run(n)
        return [s.field(q, np.float32) for q in F.STATE], s.seismograms()


CASES = [
    ("iso", F.MODEL_ISO, None, 150, 37, 20),
    ("iso-small", F.MODEL_ISO, None, 33, 9, 31),
    ("ortho-w3d", F.MODEL_ORTHO, F.DAMP_W3D, 192, 30, 19),
    ("ortho-sep", F.MODEL_ORTHO, F.DAMP_SEPARABLE, 131, 26, 22),
    ("ortho-sep-narrow", F.MODEL_ORTHO, F.DAMP_SEPARABLE, 29, 17, 27),
]


@pytest.mark.parametrize("name,model,damping,nx,ny,nz", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("kchunk", [0, 8], ids=["kc16", "kc8"])
def test_staged_bitwise_vs_oracle(cuda_device, name, model, damping, nx, ny, nz, kchunk):
    m = I.random_small(model, nx, ny, nz, nt=24, seed=5, damping=damping)
    ref = O.run(m, 24)
    assert_bitwise(run_staged(m, 24, kchunk=kchunk, chunks=[9, 15]), ref, f"{name} kchunk {kchunk}")


def test_staged_chunks_and_graphs(cuda_device):
    m = I.random_small(F.MODEL_ORTHO, 140, 21, 33, nt=30, seed=9, damping=F.DAMP_SEPARABLE)
    ref = O.run(m, 30)
    for kchunk, gs in ((4, -1), (5, 3), (11, 5), (33, 4), (64, 0)):
        assert_bitwise(run_staged(m, 30, kchunk=kchunk, graph_steps=gs, chunks=[7, 12, 11]), ref,
                       f"kchunk {kchunk} graph {gs}")


def test_staged_sources_on_borders(cuda_device):
    """Point sources on tile borders in x (63/64, 127/128) and y (7/8, 15/16), on chunk borders
    and on planes 0-2 under the free surface, several entries per cell, both injection orders."""
    for model in (F.MODEL_ISO, F.MODEL_ORTHO):
        for order in (F.SRC_BEFORE_BC1, F.SRC_AFTER_BC1):
            m = I.random_small(model, 140, 26, 24, nt=20, seed=31, src_order=order)
            ent, coef = [], []
            rng = np.random.default_rng(7)
            cells = ((63, 7, 1), (64, 8, 2), (127, 8, 8), (128, 15, 9), (63, 16, 0), (64, 7, 16), (1, 1, 2),
                     (127, 0, 1), (128, 24, 2), (0, 8, 17))
            for comp in range(3, 9):
                for c in cells:
                    ent.append((comp,) + c)
                    coef.append(rng.normal())
            ent = ent[:60] + [ent[0], ent[7], ent[12], ent[25]]
            coef = coef[:60] + [0.5, -0.25, 0.75, 1.5]
            m.sources = np.array(ent, np.int32)
            m.source_coef = np.array(coef)
            ref = O.run(m, 20)
            assert_bitwise(run_staged(m, 20, kchunk=8), ref, f"model {model} order {order}")


def test_staged_free_surface_sources(cuda_device):
    """Moment-tensor sources on planes 0-2 next to the free surface (the BC1 replay), both orders
    and stencils."""
    for order in (F.SRC_BEFORE_BC1, F.SRC_AFTER_BC1):
        for stencil in (0, 1):
            for zs in (0, 1, 2):
                for model in (F.MODEL_ISO, F.MODEL_ORTHO):
                    m = I.random_small(model, 70, 26, 18, nt=30, seed=3 + zs, src_order=order, stencil=stencil)
                    m.set_moment_tensor(np.array([1.0, -0.5, 0.25, 0.7, -0.9, 1.3]), 63, 7, zs, stencil)
                    ref = O.run(m, 30)
                    assert_bitwise(run_staged(m, 30), ref, f"model {model} order {order} stencil {stencil} zs {zs}")


def test_staged_wait_gives_up_and_handle_recovers(cuda_device):
    """A stage fill that nothing completes (test hook): the bounded waits give up, the launch still
    ends, ewf_run reports EWF_ERR_CUDA; after the hook is cleared and the state reset, the next run
    is bit-exact."""
    from elanfmt_gb300.solver import EwfError, load_library

    lib = load_library()
    m = I.random_small(F.MODEL_ORTHO, 70, 20, 24, nt=12, seed=41, damping=F.DAMP_SEPARABLE)
    ref = O.run(m, 12)
    with Solver.from_model(m, fused=F.STEP_FUSED, kchunk=8, graph_steps=-1) as s:
        s.set_onepass(F.ONEPASS_STAGED)
        assert lib.ewf_staged_test_hold(5, 4096) == 0
        try:
            with pytest.raises(EwfError) as e:
                s.run(3)
            assert e.value.status == -2  # EWF_ERR_CUDA
        finally:
            assert lib.ewf_staged_test_hold(-1, 0) == 0
        s.reset()
        s.run(12)
        assert_bitwise(([s.field(q, np.float32) for q in F.STATE], s.seismograms()), ref, "after the failed run")
