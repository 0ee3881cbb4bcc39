"""ewf_pack_field_noalloc: the layout conversion for callers that cannot call cudaMalloc.

Such a caller owns its device memory (another framework's pool, a fixed budget reserved up front)
and wants the solver's box layout written into an array it already has.  The entry point's only
scratch is a fixed array compiled into the library.  Here the caller's array comes from torch;
the result must equal what ewf_set_field (which stages through its handle's own buffer) stores,
read back with ewf_get_field -- on two calls in a row, with different data, dtypes and shapes,
so the second call runs on a scratch array that still holds the first call's contents.
"""
import numpy as np
import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300.solver import Solver, load_library

pytestmark = pytest.mark.gpu


def unbox(t, ex, ey, ez, sx, sy):
    a = t.cpu().numpy()
    out = np.empty((ez, ey, ex), a.dtype)
    for k in range(ez):
        out[k] = a[k * sy: k * sy + sx * ey].reshape(ey, sx)[:, :ex]
    return out


@pytest.mark.parametrize("precision,dst_dt", [(F.PREC_F32, np.float32), (F.PREC_F64, np.float64)],
                         ids=["float32-dst", "float64-dst"])
def test_noalloc_pack_matches_set_field(cuda_device, precision, dst_dt):
    import torch

    lib = load_library()
    m = I.random_small(F.MODEL_ORTHO, 30, 26, 20, nt=4, seed=31, damping=F.DAMP_W3D)
    rng = np.random.default_rng(5)
    calls = [(F.M_C66XY, np.float32), (F.F_SYZ, np.float64)]  # second call: larger, float64 input
    tdt = torch.float32 if dst_dt == np.float32 else torch.float64
    with Solver.from_model(m, precision=precision) as s:
        for fid, host_dt in calls:
            ez, ey, ex = F.shape(fid, m.nx, m.ny, m.nz)
            host = np.ascontiguousarray(rng.standard_normal((ez, ey, ex)).astype(host_dt))
            s.set_field(fid, host)
            ref = s.field(fid, dst_dt)  # the existing entry point's result, in the handle's precision
            sx, sy = ex + 7, (ex + 7) * (ey + 2)
            dst = torch.full((sy * ez + 16,), float("nan"), dtype=tdt, device="cuda")
            st = lib.ewf_pack_field_noalloc(dst.data_ptr(), dst.element_size(), sx, sy, host.ctypes.data,
                                            host.itemsize, ex, ey, ez, None)
            assert st == 0, lib.ewf_last_error()
            got = unbox(dst, ex, ey, ez, sx, sy)
            np.testing.assert_array_equal(got, ref)
            assert torch.isnan(dst[ex:sx]).all(), "cells outside the extent must stay untouched"


def test_noalloc_rejects_bad_destinations(cuda_device):
    """Every case is refused on the host, before any device work: a misaligned float64 pointer,
    host memory, and an extent whose pitches end past the destination's allocation."""
    import torch

    lib = load_library()
    host = np.zeros((4, 4, 4), np.float64)
    dst = torch.zeros(4 * 4 * 4 + 2, dtype=torch.float64, device="cuda")
    st = lib.ewf_pack_field_noalloc(dst.data_ptr() + 4, 8, 4, 16, host.ctypes.data, 8, 4, 4, 4, None)
    assert st == -1 and b"aligned" in lib.ewf_last_error()
    hdst = np.zeros(64, np.float64)
    st = lib.ewf_pack_field_noalloc(hdst.ctypes.data, 8, 4, 16, host.ctypes.data, 8, 4, 4, 4, None)
    assert st == -1 and b"device memory" in lib.ewf_last_error()
    st = lib.ewf_pack_field_noalloc(dst.data_ptr(), 8, 4, 1 << 39, host.ctypes.data, 8, 4, 4, 4, None)
    assert st == -1 and b"past its allocation" in lib.ewf_last_error()
    st = lib.ewf_pack_field_noalloc(dst.data_ptr(), 8, 4, 16, host.ctypes.data, 8, 4, 4, 4, None)
    assert st == 0, lib.ewf_last_error()
    np.testing.assert_array_equal(dst[:64].cpu().numpy(), host.ravel())


def test_noalloc_rejects_arrays_beyond_the_scratch(cuda_device):
    import torch

    lib = load_library()
    n = (16 << 20) // 4 + 1
    host = np.zeros(n, np.float32)
    dst = torch.zeros(n, device="cuda")
    st = lib.ewf_pack_field_noalloc(dst.data_ptr(), 4, n, n, host.ctypes.data, 4, n, 1, 1, None)
    assert st == -1
    assert b"scratch" in lib.ewf_last_error()
