"""The oracle's disk/triangle overlap area against the reference's own
compiled CPU routine (src/contact_geometry.cpp, built into oracle/_ref by
oracle/reference_build.py).  Skipped where the reference tree was not
available to build it."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import circle_triangle_area

REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref")
LIB = os.path.join(REF, "libref_geometry.so")

pytestmark = pytest.mark.skipif(not os.path.exists(LIB), reason="reference geometry not built here")


def ref_area(center, radius, a, b, c):
    lib = C.CDLL(LIB)
    lib.ref_sphere_triangle_area.restype = C.c_double
    lib.ref_sphere_triangle_area.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    arrs = [np.ascontiguousarray(x, float) for x in (center, a, b, c)]
    return lib.ref_sphere_triangle_area(C.c_void_p(arrs[0].ctypes.data), float(radius),
                                        *[C.c_void_p(x.ctypes.data) for x in arrs[1:]])


def test_reference_known_answer_binary_passes():
    exe = os.path.join(REF, "contact_geometry_tests")
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and "passed" in out.stdout


def test_area_matches_reference_routine_on_random_cases():
    rng = np.random.default_rng(1234)
    worst = 0.0
    for _ in range(3000):
        tri = rng.uniform(-2e-3, 2e-3, size=(3, 3))
        tri[:, 2] = rng.uniform(-1e-4, 1e-4) if rng.random() < 0.5 else tri[:, 2] * 0.1
        n = np.cross(tri[1] - tri[0], tri[2] - tri[0])
        ln = np.linalg.norm(n)
        if ln < 1e-9:
            continue
        n = n / ln
        p = rng.uniform(-2e-3, 2e-3, size=3)
        r = rng.uniform(0.2e-3, 2e-3)
        dist = np.dot(n, p - tri[0])
        c2 = r * r - dist * dist
        expect = ref_area(p, r, *tri)
        if c2 <= 0:
            assert expect == 0.0
            continue
        ce = p - n * dist
        got = circle_triangle_area(ce, n, tri[0], tri[1], tri[2], math.sqrt(c2))
        scale = math.pi * c2
        worst = max(worst, abs(got - expect) / scale)
    assert worst <= 1e-9, worst
