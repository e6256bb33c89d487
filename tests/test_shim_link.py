"""The reference's own host program (main, simulation, integrator, loaders,
writers, dyneq, async output) compiled from its sources against the
CudaDemSolver shim and libdemgb300.so: it links and runs its --cuda-info
entry through the engine's dem_device_available.  Skipped where the
reference tree is not available."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle.reference_build import reference_root

REF = reference_root()


@pytest.mark.skipif(REF is None, reason="reference tree not available")
def test_reference_host_program_links_against_engine(engine_lib):
    shim = os.path.join(ROOT, "dem_mbd_cuda_gb300", "shim")
    r = subprocess.run(["make", "-C", shim, f"REF={REF}", "-j8"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    exe = os.path.join(shim, "_build", "dem_mbd_gb300")
    out = subprocess.run([exe, "--cuda-info"], capture_output=True, text=True, timeout=60)
    text = out.stdout + out.stderr
    if engine_lib.dem_device_available():
        assert out.returncode == 0, text
    else:
        assert "CUDA" in text
