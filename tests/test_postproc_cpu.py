"""The driver's Butterworth band-pass (FINAL.m:535-614) against scipy: the filter design
(zeros, poles, gain) and the filtered traces.  The recursion runs in libewfd.so's host path."""
import numpy as np
import pytest

from elanfmt_gb300 import postproc as P

signal = pytest.importorskip("scipy.signal")


def sorted_c(v):
    v = np.asarray(v, complex)
    return v[np.lexsort((np.round(v.imag, 12), np.round(v.real, 12)))]


@pytest.mark.parametrize("order,w1,w2", [(4, 1.9e-3, 9.6e-3), (4, 0.1, 0.3), (2, 0.05, 0.6), (6, 0.2, 0.25)])
def test_design_matches_scipy(order, w1, w2):
    z, p, k = P.butter_bandpass_zpk(order, w1, w2)
    zs, ps, ks = signal.butter(order, [w1, w2], btype="bandpass", output="zpk")
    np.testing.assert_allclose(sorted_c(z), sorted_c(zs), atol=1e-12)
    np.testing.assert_allclose(sorted_c(p), sorted_c(ps), rtol=1e-12, atol=1e-14)
    assert np.isclose(k, ks, rtol=1e-10)
    # the sections multiply out to the same transfer function
    sos = P.zpk_to_sos(z, p, k)
    w = np.linspace(0.0, np.pi, 257)
    _, h = signal.sosfreqz(sos, worN=w)
    _, hs = signal.sosfreqz(signal.zpk2sos(zs, ps, ks), worN=w)
    np.testing.assert_allclose(np.abs(h), np.abs(hs), atol=1e-9 * np.abs(hs).max())


def test_filtered_traces_match_scipy():
    rng = np.random.default_rng(3)
    dt = 2.4056e-3                       # the isotropic benchmark workload's time step
    x = rng.standard_normal((3, 4000)).cumsum(axis=1)
    sos = P.butter_bandpass(4, 1 / 2.5, 1 / 0.5, 1 / dt)
    sos_ref = signal.butter(4, [1 / 2.5, 1 / 0.5], btype="bandpass", output="sos", fs=1 / dt)
    y = P.sosfilt(sos, x)
    y_ref = signal.sosfilt(sos_ref, x, axis=-1)
    assert y.shape == x.shape
    np.testing.assert_allclose(y, y_ref, atol=1e-7 * np.abs(y_ref).max())
    # one trace, and the driver's recipe: 2799 samples padded to 150000 with zeros
    np.testing.assert_array_equal(P.sosfilt(sos, x[1]), y[1])
    d = P.bandpass_driver(x[0], dt)
    sig = np.zeros(150000)
    sig[:2799] = x[0, :2799]
    d_ref = signal.sosfilt(sos_ref, sig)
    assert d.shape == (150000,)
    np.testing.assert_allclose(d, d_ref, atol=1e-7 * np.abs(d_ref).max())


def test_bad_filters_are_refused():
    with pytest.raises(ValueError):
        P.butter_bandpass_zpk(4, 0.3, 0.2)
    with pytest.raises(ValueError):
        P.sosfilt(np.zeros((17, 6)), np.zeros(10))
    from elanfmt_gb300.solver import EwfError

    bad = np.array([[1.0, 0.0, -1.0, 0.0, 0.1, 0.2]])   # a0 = 0
    with pytest.raises(EwfError):
        P.sosfilt(bad, np.zeros(10))
