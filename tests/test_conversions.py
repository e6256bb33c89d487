"""f32_rn and f64_of, the integer-pipe conversions between FP64 and FP32
(dem_device.cuh), against the C conversions on the host: tests/conv_check.cu
compiled as a host program and run (f64_of over every float bit pattern)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_pipe_conversions_match_the_c_conversions(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "conv_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", os.path.join(HERE, "conv_check.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout[-3000:]
