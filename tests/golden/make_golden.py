"""Regenerate the golden input fixtures from the reference's validation cases.

Run in a checkout where the reference tree is available:
    python tests/golden/make_golden.py /path/to/reference
Each reference case directory (validation/cases/<name> and
validation/ctest_data1_{pure_dem,mbd}) is parsed with the reference's file
formats (dem_mbd_cuda_gb300.formats) and stored as tests/golden/<name>.npz:
the scene arrays plus its ODE settings.  The expected answers of the
analytic cases live in the tests that use them, with the reference
file:line they come from.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from dem_mbd_cuda_gb300.formats import read_case  # noqa: E402

CASES = {
    "free_fall": "validation/cases/free_fall",
    "wall_contact": "validation/cases/wall_contact",
    "two_particle": "validation/cases/two_particle",
    "triangle_contact": "validation/cases/triangle_contact",
    "body_states": "validation/cases/body_states",
    "data1_pure_dem": "validation/ctest_data1_pure_dem",
    "data1_mbd": "validation/ctest_data1_mbd",
}


def main(ref_root):
    for name, rel in CASES.items():
        scene, ode = read_case(os.path.join(ref_root, rel))
        arrays = {k: v for k, v in scene.__dict__.items() if isinstance(v, np.ndarray)}
        meta = {k: (v.__dict__ if hasattr(v, "__dict__") else v) for k, v in scene.__dict__.items()
                if not isinstance(v, np.ndarray) and v is not None}
        meta["ode"] = ode
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
        print(name, scene.n, scene.n_walls, scene.n_bodies, scene.n_triangles)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.reference_build import reference_root
    root = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    if root is None:
        sys.exit("pass the reference checkout or set DEM_REFERENCE_ROOT")
    main(root)
