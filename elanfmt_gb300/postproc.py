"""Seismogram post-processing of the isotropic MATLAB driver: the 4th-order Butterworth band-pass
applied before its traces are compared (vizme_FastBiotED_GPU3D_OK_2024_final.m:535-614).

The driver builds the filter as `[z, p, k] = butter(4, [flo fhi]/(fs/2), 'bandpass');
sos = zp2sos(z, p, k)` with flo = 1/2.5 Hz, fhi = 1/0.5 Hz and fs = 1/dt, copies the first 2799
samples of a trace into a zero signal of 150000 samples and runs `sosfilt(sos, signal)`
(:551-558 vertical, :579-582 radial, :604-607 transverse).

* `butter_bandpass_zpk` restates the published digital Butterworth design: the analog low-pass
  prototype (poles equally spaced on the left unit half-circle), the low-pass to band-pass
  transform around the pre-warped band edges, and the bilinear transform.
* `zpk_to_sos` pairs each complex-conjugate pole pair into one second-order section whose
  numerator is one zero at z = 1 and one at z = -1 (the band-pass has N of each); the gain goes
  into the first section, and sections are ordered by increasing pole radius, so the poles
  nearest the unit circle are applied last.
* The recursion itself runs in libewfd.so (`ewf_sosfilt` on host arrays, `ewf_sosfilt_device` on
  device arrays, one thread per trace): direct form II transposed sections from zero state.

The driver's comparison against frequency-wavenumber synthetics (Zhu's third-party `fk`, which
the reference does not ship) is not reproduced: parity of that overlay is unpinned.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .solver import _check, load_library

MAX_SECTIONS = 16   # EWF_SOS_MAX_SECTIONS


def butter_bandpass_zpk(order: int, w1: float, w2: float) -> tuple[np.ndarray, np.ndarray, float]:
    """Zeros, poles and gain of the digital Butterworth band-pass of the given order; w1 < w2 are
    the band edges as fractions of the Nyquist frequency."""
    if not (order >= 1 and 0.0 < w1 < w2 < 1.0):
        raise ValueError(f"order {order}, band [{w1}, {w2}]: need order >= 1 and 0 < w1 < w2 < 1")
    # analog prototype: p_k = exp(i pi (2k + N + 1) / (2N)), k = 0 .. N-1, unit gain
    k = np.arange(order)
    p = np.exp(1j * np.pi * (2 * k + order + 1) / (2.0 * order))
    # band edges pre-warped for the bilinear transform with sampling rate 2 (edges in Nyquist units)
    fs = 2.0
    W1, W2 = (2 * fs * np.tan(np.pi * w / fs) for w in (w1, w2))
    bw, w0 = W2 - W1, np.sqrt(W1 * W2)
    # low-pass -> band-pass: each pole splits into the two roots of s^2 - p bw s + w0^2; N zeros at s = 0
    half = p * bw / 2
    root = np.sqrt(half * half - w0 * w0)
    pa = np.concatenate([half + root, half - root])
    za = np.zeros(order)
    ka = bw ** order
    # bilinear transform z = (2 fs + s) / (2 fs - s); the N zeros at infinity map to z = -1
    f2 = 2 * fs
    zd = np.concatenate([(f2 + za) / (f2 - za), -np.ones(order)])
    pd = (f2 + pa) / (f2 - pa)
    kd = float(ka * np.real(np.prod(f2 - za) / np.prod(f2 - pa)))
    return zd, pd, kd


def zpk_to_sos(z: np.ndarray, p: np.ndarray, k: float) -> np.ndarray:
    """Second-order sections (rows b0 b1 b2 a0 a1 a2) of a band-pass whose zeros are at +1 and -1
    (as many of each) and whose poles come in complex-conjugate pairs."""
    z = np.asarray(z)
    n1 = int(np.sum(np.isclose(z, 1.0)))
    n2 = int(np.sum(np.isclose(z, -1.0)))
    upper = p[np.imag(p) > 0]
    if n1 != n2 or n1 + n2 != len(z) or 2 * len(upper) != len(p) or len(upper) != n1:
        raise ValueError("zpk_to_sos handles band-pass filters: zeros at +-1, conjugate pole pairs")
    upper = upper[np.argsort(np.abs(upper))]
    sos = np.zeros((len(upper), 6))
    for s, pole in enumerate(upper):
        sos[s] = [1.0, 0.0, -1.0, 1.0, -2.0 * pole.real, abs(pole) ** 2]
    sos[0, :3] *= k
    return sos


def butter_bandpass(order: int, flo_hz: float, fhi_hz: float, fs_hz: float) -> np.ndarray:
    """The driver's `zp2sos(butter(order, [flo fhi]/(fs/2), 'bandpass'))` as second-order sections."""
    nyq = fs_hz / 2.0
    return zpk_to_sos(*butter_bandpass_zpk(order, flo_hz / nyq, fhi_hz / nyq))


def sosfilt(sos: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Filters each row of x (traces x samples, or one trace) with the sections; returns a new
    float64 array."""
    s = np.ascontiguousarray(sos, dtype=np.float64).reshape(-1, 6)
    if len(s) > MAX_SECTIONS:
        raise ValueError(f"{len(s)} sections, at most {MAX_SECTIONS}")
    y = np.array(x, dtype=np.float64, order="C", copy=True)
    ntr = 1 if y.ndim == 1 else int(np.prod(y.shape[:-1]))
    _check(load_library().ewf_sosfilt(s.ctypes.data_as(C.c_void_p), len(s), y.ctypes.data_as(C.c_void_p), ntr,
                                      y.shape[-1]), "ewf_sosfilt")
    return y


def sosfilt_device(sos: np.ndarray, traces) -> None:
    """Filters a contiguous float64 torch tensor of traces (..., samples) on its GPU, in place,
    on the current stream."""
    import torch

    s = np.ascontiguousarray(sos, dtype=np.float64).reshape(-1, 6)
    if traces.dtype != torch.float64 or not traces.is_cuda or not traces.is_contiguous():
        raise ValueError("traces: a contiguous float64 CUDA tensor")
    ntr = 1 if traces.dim() == 1 else int(np.prod(traces.shape[:-1]))
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _check(load_library().ewf_sosfilt_device(s.ctypes.data_as(C.c_void_p), len(s), C.c_void_p(traces.data_ptr()), ntr,
                                             traces.shape[-1], st), "ewf_sosfilt_device")


def bandpass_driver(trace: np.ndarray, dt: float, flo_hz: float = 1 / 2.5, fhi_hz: float = 1 / 0.5,
                    keep: int = 2799, length: int = 150000) -> np.ndarray:
    """The driver's recipe for one trace (:548-558): its first `keep` samples in a zero signal of
    `length` samples, band-passed by the 4th-order Butterworth between flo and fhi."""
    sig = np.zeros(length)
    n = min(keep, len(trace))
    sig[:n] = np.asarray(trace, np.float64)[:n]
    return sosfilt(butter_bandpass(4, flo_hz, fhi_hz, 1.0 / dt), sig)
