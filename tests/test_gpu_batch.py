"""Batched solver: every (problem, right-hand side) of a batch must equal its solo run bit for bit
(and therefore the oracle), whatever the mix of model families, sizes and RHS counts."""
import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300.solver import Batch, Solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def problems(nt=36):
    rng = np.random.default_rng(3)
    ortho = I.random_small(F.MODEL_ORTHO, 37, 41, 22, nt=nt, seed=5, damping=F.DAMP_SEPARABLE)
    ortho_w3 = I.random_small(F.MODEL_ORTHO, 26, 30, 19, nt=nt, seed=8, damping=F.DAMP_W3D)
    iso_a = I.random_small(F.MODEL_ISO, 33, 35, 20, nt=nt, seed=6)
    iso_b = I.random_small(F.MODEL_ISO, 21, 18, 27, nt=nt, seed=7, src_order=F.SRC_AFTER_BC1)
    out = []
    for m, nrhs in ((ortho, 3), (iso_a, 1), (ortho_w3, 2), (iso_b, 2)):
        rl = []
        for r in range(nrhs):
            mt = rng.normal(size=6)
            zs = int(rng.integers(0, 6))
            ent, coef = F.mt_entries(mt, m.nx // 2 - 2 + r, m.ny // 2 - 1, zs, 0 if m.model == F.MODEL_ISO else 1)
            rl.append((ent, coef))
        out.append((m, rl))
    return out


def solo(m, ent, coef, nsteps):
    with Solver.from_model(m) as s:
        s.set_sources(ent, coef)
        s.run(nsteps)
        return [s.field(q) for q in F.STATE], s.seismograms()


def test_batch_equals_solo_runs(cuda_device):
    probs = problems()
    with Batch(probs) as b:
        b.run(20)
        b.run(16)  # two runs: the graph (64 steps) is not used, then the tail path
        for pid, (m, rl) in enumerate(probs):
            for r, (ent, coef) in enumerate(rl):
                fields, traces = solo(m, ent, coef, 36)
                for q in F.STATE:
                    np.testing.assert_array_equal(b.field(pid, r, q), fields[q], err_msg=f"problem {pid} rhs {r} {q}")
                np.testing.assert_array_equal(b.seismograms(pid, r), traces)
                assert np.abs(traces).max() > 0
                # and the oracle
                mm = m
                mm.sources, mm.source_coef = ent, coef
                ref = O.run(mm, 36)
                np.testing.assert_array_equal(b.seismograms(pid, r), ref.traces)


def test_batch_tile_heights(cuda_device):
    """Every CTA tile height gives the same bits (multi-RHS launches and the persistent family
    launches alike); the autotuner picks one of them."""
    probs = problems(nt=24)
    ref = None
    for ty in (4, 8, 16):
        with Batch(probs) as b:
            b.set_tile(ty)
            assert b.tile() == ty
            b.run(24)
            got = [[b.seismograms(p, r) for r in range(len(rl))] + [b.field(p, 0, F.F_SXY)]
                   for p, (_, rl) in enumerate(probs)]
        if ref is None:
            ref = got
            m, rl = probs[0]
            np.testing.assert_array_equal(got[0][2], solo(m, rl[2][0], rl[2][1], 24)[1])
        else:
            for a, c in zip(got, ref):
                for x, y in zip(a, c):
                    np.testing.assert_array_equal(x, y, err_msg=f"tile height {ty}")
    with Batch(probs) as b:
        b.autotune(3)
        assert b.tile() in (4, 8, 16)
        for bad in (2, 5, 32):
            with pytest.raises(Exception):
                b.set_tile(bad)


def test_batch_launch_forms(cuda_device):
    """Single-RHS problems in one persistent family launch or in launches of their own on parallel
    graph branches: the same bits, graph replays included."""
    probs = problems(nt=70)
    ref = None
    for own in (0, 1):
        with Batch(probs) as b:
            b.set_launch(own)
            assert b.launch() == own
            b.run(70)  # one graph of 64 steps + 6 direct steps
            got = [[b.seismograms(p, r) for r in range(len(rl))] + [b.field(p, 0, F.F_SYY)]
                   for p, (_, rl) in enumerate(probs)]
        if ref is None:
            ref = got
            m, rl = probs[-1]
            np.testing.assert_array_equal(got[-1][0], solo(m, rl[0][0], rl[0][1], 70)[1])
        else:
            for a, c in zip(got, ref):
                for x, y in zip(a, c):
                    np.testing.assert_array_equal(x, y, err_msg=f"launch form {own}")


def test_batch_l2_prefetch(cuda_device):
    """The multi-RHS velocity kernel's L2 prefetch is a hint: every distance gives the same bits."""
    probs = problems(nt=24)
    ref = None
    for pf in (0, 2, 5):
        with Batch(probs) as b:
            b.set_l2_prefetch(pf)
            assert b.l2_prefetch() == pf
            b.run(24)
            got = [[b.seismograms(p, r) for r in range(len(rl))] + [b.field(p, 0, F.F_VX)]
                   for p, (_, rl) in enumerate(probs)]
        if ref is None:
            ref = got
        else:
            for a, c in zip(got, ref):
                for x, y in zip(a, c):
                    np.testing.assert_array_equal(x, y, err_msg=f"prefetch {pf}")
    with Batch(probs) as b:
        with pytest.raises(Exception):
            b.set_l2_prefetch(9)


def test_batch_graph_autotune_and_reset(cuda_device):
    probs = problems(nt=140)
    with Batch(probs) as b:
        k = b.autotune(6)
        assert k in (8, 12, 16, 24, 32, 48, 64)
        b.run(140)  # 2 graph launches of 64 steps + 12 direct steps
        got = [[b.seismograms(p, r) for r in range(len(rl))] for p, (_, rl) in enumerate(probs)]
        b.reset()
        b.run(70)
        b.run(70)
        for p, (m, rl) in enumerate(probs):
            for r, (ent, coef) in enumerate(rl):
                np.testing.assert_array_equal(b.seismograms(p, r), got[p][r])
        m, rl = probs[0]
        np.testing.assert_array_equal(got[0][1], solo(m, rl[1][0], rl[1][1], 140)[1])


def test_single_handle_autotune(cuda_device):
    m = I.random_small(F.MODEL_ORTHO, 40, 33, 48, nt=60, seed=11, damping=F.DAMP_SEPARABLE)
    ref = O.run(m, 60)
    with Solver.from_model(m) as s:
        k = s.autotune(8)
        assert k in (4, 6, 8, 12, 16, 24, 32, 48)
        assert s.step() == 0
        s.run(60)
        np.testing.assert_array_equal(s.seismograms(), ref.traces)
