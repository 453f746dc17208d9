"""Host-side test of the per-device kernel set-up bookkeeping.

The launchers keep their one-time set-up (kernel attributes, resident CTA
counts) and the allocation-free norm keeps its scratch address per device
ordinal, in atomics.  tests/native/device_state_check.cpp drives that
bookkeeping (libcugpe_gb300/csrc/gpe_device_state.h) with g++ and threads:
no CUDA device is needed.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "libcugpe_gb300", "csrc")


def test_device_state_bookkeeping(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "device_state_check")
    src = os.path.join(HERE, "native", "device_state_check.cpp")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", CSRC, src, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert "device state ok" in r.stdout
