"""The step adjoints' vector-Jacobian products (dem_adjoint.cuh) against
central differences, on the CPU: tests/adjoint_vjp_check.cu compiled as a
host program and run."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_vjps_match_central_differences(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "adjoint_vjp_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-x", "cu", os.path.join(HERE, "adjoint_vjp_check.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout[-3000:]
