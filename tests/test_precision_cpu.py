"""The precision study's error measures (no GPU): relative L2 and peak error per trace, and the
traces left out because no arrival has reached them."""
import numpy as np

from elanfmt_gb300.precision import errors


def test_errors_per_trace_and_floor():
    t = np.linspace(0, 1, 200)
    ref = np.stack([np.sin(20 * t), 2 * np.cos(15 * t), 1e-9 * np.sin(50 * t), np.zeros_like(t)])
    a = ref.copy()
    a[0] *= 1 + 1e-5
    a[1] += 1e-4 * np.sin(3 * t)
    a[2] = -a[2]  # rounding-level noise, 100 % "relative" error
    e = errors(a, ref)
    assert e["traces"] == 2 and e["traces_without_arrival"] == 2
    np.testing.assert_allclose(e["rel_l2_per_trace"][0], 1e-5, rtol=1e-6)
    expect1 = np.linalg.norm(1e-4 * np.sin(3 * t)) / np.linalg.norm(ref[1])
    np.testing.assert_allclose(e["rel_l2_per_trace"][1], expect1, rtol=1e-9)
    assert e["rel_l2_max"] == max(e["rel_l2_per_trace"])
    # with no floor the quiet trace counts, and dominates the maximum
    e0 = errors(a, ref, floor=0.0)
    assert e0["traces"] == 3 and np.isclose(e0["rel_l2_max"], 2.0)
