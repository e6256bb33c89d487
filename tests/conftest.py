"""Shared test helpers.  GPU tests carry @pytest.mark.gpu and call the CUDA
engine through its C ABI; everything else runs on the CPU."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def load_golden(name):
    """Scene and ODE settings of a reference validation case (fixtures made
    by tests/golden/make_golden.py from the reference's validation inputs)."""
    from dem_mbd_cuda_gb300.scene import Mech, Scene
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    ode = meta.pop("ode")
    kw = {k: z[k] for k in z.files if k != "meta"}
    for m in ("pp", "pt", "pw"):
        kw[m] = Mech(**meta.pop(m))
    kw.update({k: (tuple(v) if isinstance(v, list) else v) for k, v in meta.items()})
    return Scene(**kw), ode


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if needed) and load the CUDA engine library."""
    from dem_mbd_cuda_gb300 import build, engine
    build.build()
    return engine.load_library()
