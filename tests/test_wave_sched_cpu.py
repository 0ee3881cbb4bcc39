"""The wavefront step's scheduling code, checked on the host.  Both C++ programs compile the
header the kernel uses (elanfmt_gb300/csrc/ewfd_wave_sched.h):
  * wave_sched_check.cpp, exhaustively: the ticket bijection, that every dependency holds an
    earlier ticket (the order cannot deadlock), the plane coverage of both phases, that every
    read/write conflict between a stress item and a velocity item is ordered by a dependency,
    and the owners of point-source cells;
  * wave_ctrl_sim.cpp, randomised: the control warp's loop (wave_control_step) driven by
    simulated CTAs that start late, compute items for random times and interleave at random --
    no deadlock, every item run once, stress items published once after being written, velocity
    items handed over only with their dependencies published."""
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
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr


def test_wave_schedule_exhaustive(tmp_path):
    _run(tmp_path, "wave_sched_check")


def test_wave_control_loop_simulation(tmp_path):
    _run(tmp_path, "wave_ctrl_sim")
