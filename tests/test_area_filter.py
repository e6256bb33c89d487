"""The particle-triangle candidate filter (tri_disk, dem_device.cuh) against
the area routine, on the CPU: tests/area_filter_check.cu compiled as a host
program and run.  Every triangle the filter rejects must have a reference
area scale at or below its 1e-12 threshold, and every triangle with a scale
above it must be kept."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_filter_rejects_only_triangles_the_edge_sum_scores_zero(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "area_filter_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-x", "cu", os.path.join(HERE, "area_filter_check.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout[-3000:]
