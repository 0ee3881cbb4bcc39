"""The tcgen05 GEMM checked on the host; both C++ programs compile the header the kernel uses
(elanfmt_gb300/csrc/ewf_umma.h):
  * umma_layout_check.cpp: shared-memory fit and 1024-byte stage alignment, TMA boxes delivering
    the bytes the stage barrier expects, every byte range an MMA reads inside its operand tile,
    and descriptor fields that decode back to their inputs, for both tile widths;
  * umma_pipeline_sim.cpp: the mbarrier protocol of producer, MMA issuer and epilogue warps (the
    header's phase-parity functions) under random interleavings -- no deadlock, no slot refilled
    or accumulator overwritten while in use, no stage or accumulator read before it is ready."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "elanfmt_gb300", "csrc")


def _run(tmp_path, name):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / name)
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, name + ".cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr


def test_umma_layout_and_descriptors(tmp_path):
    _run(tmp_path, "umma_layout_check")


def test_umma_pipeline_protocol(tmp_path):
    _run(tmp_path, "umma_pipeline_sim")
