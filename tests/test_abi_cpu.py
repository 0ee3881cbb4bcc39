"""C ABI checks that need no GPU: the library loads, exports every symbol include/ewfd.h
declares, and reports errors by status code (never exit/abort)."""
import ctypes as C
import os
import re

import pytest

from elanfmt_gb300 import fields as F
from elanfmt_gb300 import solver as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ewfd.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ewf_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_abi():
    names = declared_functions()
    for must in ("ewf_create", "ewf_destroy", "ewf_load_legacy_inputs", "ewf_set_field", "ewf_run",
                 "ewf_get_seismograms", "ewf_write_legacy_outputs", "ewf_checkpoint", "ewf_restore", "ewf_strerror"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(S.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the binding covers them all
    assert set(declared_functions()) == set(S.SIGNATURES)


def test_abi_version_and_strerror(built_lib):
    lib = S.load_library()
    assert lib.ewf_abi_version() == 6
    for code, name in F.STATUS.items():
        assert lib.ewf_strerror(code)
    assert lib.ewf_strerror(-99) == b"unknown status"


def test_params_struct_layout(built_lib):
    p = S.default_params()
    assert p.model == F.MODEL_ISO and p.precision == F.PREC_F32 and p.check_finite == 1
    assert p.fused == 0 and p.free_surface == 0 and p.surface_mu == 0.0
    assert C.sizeof(S.Params) == 14 * 4 + 11 * 8 + 8 + 2 * 4 + 8


def _have_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_have_gpu(), reason="checks the no-device path")
def test_create_without_device_fails_cleanly(built_lib):
    p = S.default_params()
    p.nx = p.ny = p.nz = 16
    p.nt = 10
    with pytest.raises(S.EwfError) as e:
        S.Solver(p)
    assert e.value.status in (-9, -2)


def test_create_rejects_bad_params(built_lib):
    for field, value in (("nx", 2), ("nt", 0), ("model", 7), ("precision", 9), ("kchunk", 2)):
        p = S.default_params()
        p.nx = p.ny = p.nz = 16
        p.nt = 10
        setattr(p, field, value)
        with pytest.raises(S.EwfError) as e:
            S.Solver(p)
        assert e.value.status == -1, (field, e.value)


def test_create_rejects_undefined_reference_cases(built_lib):
    p = S.default_params()
    p.nx, p.ny, p.nz, p.nt = 32, 16, 16, 10
    p.over_y = 3  # nx > ny with OVERY > 0: the reference's BC1 races
    with pytest.raises(S.EwfError) as e:
        S.Solver(p)
    assert e.value.status == -8
    p = S.default_params()
    p.nx = p.ny = p.nz = 16
    p.nt = 10
    p.model = F.MODEL_ISO
    p.damping = F.DAMP_W3D
    with pytest.raises(S.EwfError) as e:
        S.Solver(p)
    assert e.value.status == -8


def test_legacy_params_missing_files(built_lib, tmp_path):
    p = S.default_params()
    p.workdir = os.fsencode(str(tmp_path))
    st = S.load_library().ewf_legacy_params(C.byref(p))
    assert st == -4
    assert b"pa1.dat" in S.load_library().ewf_last_error()


def test_ewfd_executable_reports_errors(built_lib, tmp_path):
    import subprocess

    exe = os.path.join(ROOT, "elanfmt_gb300", "ewfd")
    r = subprocess.run([exe, "--nx", "16", "--ny", "16", "--nz", "16", "--workdir", str(tmp_path)],
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert "pa1.dat" in r.stderr
    r = subprocess.run([exe, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1


def test_null_handles_are_rejected(built_lib):
    """The launch-setting entry points answer a NULL handle with EWF_ERR_ARG (no device needed)."""
    lib = S.load_library()
    v = C.c_int32()
    for name in ("ewf_set_onepass", "ewf_set_tile", "ewf_set_l2_prefetch", "ewf_set_dependent_launch", "ewf_set_wave",
                 "ewf_batch_set_launch", "ewf_batch_set_l2_prefetch", "ewf_batch_set_tile"):
        assert getattr(lib, name)(None, 0) == -1, name
    for name in ("ewf_get_onepass", "ewf_get_tile", "ewf_get_l2_prefetch", "ewf_get_dependent_launch", "ewf_get_wave",
                 "ewf_batch_get_launch", "ewf_batch_get_l2_prefetch", "ewf_batch_get_tile"):
        assert getattr(lib, name)(None, C.byref(v)) == -1, name
