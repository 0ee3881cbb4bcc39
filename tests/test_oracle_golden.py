"""The CPU oracle pinned to the reference's own outputs (CPU only).

tests/golden/*.npz were produced by the reference kernels themselves (compiled from the
reference sources, replayed on a GPU by tests/golden/make_golden.py).  The oracle's FP32 build
must reproduce the FMA-free reference build bit for bit and the reference's stock build within
rounding.  Shear cells on the planes i = 0 / j = 0 / k = 0 are excluded: the isotropic reference
reads a wrapped neighbour there (FastWaveED_GPU3D_v1.cu:323-329) and never reads those cells back.
"""
import os

import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from oracle import oracle as O

from .golden import make_golden as G

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def edge_mask(q, shape):
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


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_oracle_matches_reference_kernels(built_oracle, name):
    path = os.path.join(HERE, f"{name}.npz")
    if not os.path.exists(path):
        pytest.fail(f"golden fixture {path} missing: generate it with tests/golden/make_golden.py on a GPU")
    g = np.load(path)
    m = G.CASES[name]()
    assert str(g["digest"]) == G.input_digest(m), "input generator changed since the fixture was made"
    s = O.run(m, int(g["nsteps"]))
    for q in F.STATE:
        nm = F.STATE_NAMES[q]
        mk = edge_mask(q, s.f[q].shape)
        np.testing.assert_array_equal(s.f[q][mk], g[f"exact_{nm}"][mk], err_msg=f"{name} {nm} vs exact build")
        stock = g[f"stock_{nm}"][mk]
        err = np.linalg.norm(s.f[q][mk].astype(np.float64) - stock) / max(np.linalg.norm(stock), 1e-300)
        assert err < 1e-5, (name, nm, err)
    np.testing.assert_array_equal(s.traces, g["exact_traces"])
    st = g["stock_traces"]
    for r in range(len(st)):
        n = np.linalg.norm(st[r])
        if n > 0:
            assert np.linalg.norm(s.traces[r] - st[r]) / n < 1e-5
    assert np.abs(s.traces).max() > 0
