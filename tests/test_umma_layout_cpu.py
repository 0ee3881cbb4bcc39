"""The tcgen05 GEMM's stage layout and descriptors, checked on the host: the C++ checker
(tests/umma_layout_check.cpp) compiles the header the kernel uses (elanfmt_gb300/csrc/ewf_umma.h)
and verifies shared-memory fit and 1024-byte stage alignment, that the TMA boxes deliver the bytes
the stage barrier expects, that every byte range an MMA reads stays inside its operand tile, and
that the descriptor fields decode back to their inputs, for both tile widths."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "elanfmt_gb300", "csrc")


def test_umma_layout_and_descriptors(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "umma_layout_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "umma_layout_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
