"""The band-pass on device-resident traces (one thread per trace) gives the host path's bits."""
import numpy as np
import pytest

from elanfmt_gb300 import postproc as P

pytestmark = pytest.mark.gpu


def test_device_filter_matches_host_bitwise(cuda_device):
    import torch

    rng = np.random.default_rng(7)
    x = rng.standard_normal((192, 6000)).cumsum(axis=1)
    sos = P.butter_bandpass(4, 1 / 2.5, 1 / 0.5, 1 / 2.4056e-3)
    ref = P.sosfilt(sos, x)
    t = torch.from_numpy(x.copy()).cuda()
    P.sosfilt_device(sos, t)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(t.cpu().numpy(), ref)
    assert np.abs(ref).max() > 0
