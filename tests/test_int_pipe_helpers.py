"""The integer-pipe replacements for FP64 comparisons, floor, modf and truncation used by the FP64
kernels (mithra_gb300/csrc/device_common.cuh) agree with the C library exactly.  The helpers are
host-callable, so the check compiles them into a host program with nvcc and runs it here."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_int_pipe_helpers_match_libm(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "int_pipe_helpers")
    src = os.path.join(HERE, "native", "int_pipe_helpers.cu")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-o", exe, src], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout
