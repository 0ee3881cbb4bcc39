"""The FP64 MLP oracle used to check the surrogate's CUDA gradients, checked itself against
central finite differences (CPU only)."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    sizes = [5, 7, 6, 4]
    Ws = [rng.normal(size=(sizes[l + 1], sizes[l])) * 0.5 for l in range(3)]
    bs = [rng.normal(size=sizes[l + 1]) * 0.1 for l in range(3)]
    x = rng.normal(size=(9, 5))
    t = rng.normal(size=(9, 4))
    loss, gW, gb = M.loss_and_grads(x, t, Ws, bs)
    h = 1e-6
    for l in range(3):
        for (a, b) in ((0, 0), (sizes[l + 1] - 1, sizes[l] - 1), (1, 2 % sizes[l])):
            Wp = [w.copy() for w in Ws]
            Wm = [w.copy() for w in Ws]
            Wp[l][a, b] += h
            Wm[l][a, b] -= h
            fd = (M.loss_and_grads(x, t, Wp, bs)[0] - M.loss_and_grads(x, t, Wm, bs)[0]) / (2 * h)
            assert abs(fd - gW[l][a, b]) < 1e-7 * max(1.0, abs(fd)), (l, a, b, fd, gW[l][a, b])
        bp = [v.copy() for v in bs]
        bm = [v.copy() for v in bs]
        bp[l][0] += h
        bm[l][0] -= h
        fd = (M.loss_and_grads(x, t, Ws, bp)[0] - M.loss_and_grads(x, t, Ws, bm)[0]) / (2 * h)
        assert abs(fd - gb[l][0]) < 1e-7 * max(1.0, abs(fd))


def test_gelu_matches_definition():
    x = np.linspace(-5, 5, 101)
    from math import erf, sqrt
    want = np.array([0.5 * v * (1 + erf(v / sqrt(2))) for v in x])
    np.testing.assert_allclose(M.gelu(x), want, rtol=0, atol=1e-15)
    h = 1e-6
    np.testing.assert_allclose(M.gelu_grad(x), (M.gelu(x + h) - M.gelu(x - h)) / (2 * h), atol=1e-8)


def test_mixing_matrices_reproduce_far_field_radiation():
    """Far-field P and S radiation of a point moment tensor in a homogeneous whole space,
    u = g (g.M.g) fP + (M.g - g (g.M.g)) fS for ray direction g, is reproduced exactly by 10
    azimuth-independent traces mixed with mixing_matrices (the symmetry the structured surrogate
    relies on)."""
    from elanfmt_gb300 import surrogate as S

    rng = np.random.default_rng(4)
    nt = 12
    fP, fS = rng.normal(size=nt), rng.normal(size=nt)
    for theta in (0.3, 1.0, 1.4):
        az = rng.uniform(-np.pi, np.pi, 40)
        R = S.mixing_matrices(az).astype(np.float64)
        Y = np.zeros((len(az), 18, nt))
        for n, a in enumerate(az):
            g = np.array([np.sin(theta) * np.cos(a), np.sin(theta) * np.sin(a), np.cos(theta)])
            for q, (i, j) in enumerate(S._MT_PAIRS):
                E = np.zeros((3, 3))
                E[i, j] = E[j, i] = 1.0
                p = g @ E @ g
                u = np.outer(g * p, fP) + np.outer(E @ g - g * p, fS)
                Y[n, 3 * q:3 * q + 3] = u
        G = np.einsum("nfo,not->nft", np.linalg.pinv(R), Y)
        # one set of fundamentals serves every azimuth (R is float32)
        assert np.abs(G - G[:1]).max() < 1e-5
        np.testing.assert_allclose(np.einsum("nof,nft->not", R, G), Y, atol=1e-5)
