"""The CPU oracle against the reference's own known answers.

Expected values are the reference's test assertions:
tests/scenario_validator.cpp:80-113 (analytic cases),
tests/contact_geometry_test.cpp:37-72 (disk-triangle areas),
tests/component_transform_test.cu:50-104 (clump component transform).
"""
import math

import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import Oracle, circle_triangle_area
from dem_mbd_cuda_gb300.scene import Scene, make_spheres


def test_free_fall():
    sc, ode = load_golden("free_fall")
    o = Oracle(sc)
    o.run(ode["end"])
    st = o.state()
    o2 = Oracle(sc)
    o2.compute_forces()
    f = o2.forces()
    assert abs(st["pos"][0, 2] - (1.0 + 0.5 * -9.8 * 0.01 * 0.01)) <= 2e-12
    assert abs(st["vel"][0, 2] - (-9.8 * 0.01)) <= 2e-12
    assert abs(f["total"][0, 2] - (-9.8)) <= 2e-12


def test_wall_contact():
    sc, _ = load_golden("wall_contact")
    o = Oracle(sc)
    o.compute_forces()
    f = o.forces()
    assert abs(f["wall"][0, 2] - 100.0) <= 1e-9
    assert abs(f["total"][0, 2] - 100.0) <= 1e-9


def test_two_particle():
    sc, _ = load_golden("two_particle")
    o = Oracle(sc)
    o.compute_forces()
    c = o.forces()["contact"]
    assert abs(c[0, 0] + 100.0) <= 1e-9
    assert abs(c[1, 0] - 100.0) <= 1e-9
    assert abs(c[0, 0] + c[1, 0]) <= 1e-12


def test_triangle_contact():
    sc, _ = load_golden("triangle_contact")
    o = Oracle(sc)
    loads = o.compute_forces(bodies=sc.body_states())
    f = o.forces()["total"]
    assert abs(f[0, 2] - 100.0) <= 1e-8
    assert abs(loads[0, 2] + 100.0) <= 1e-8
    assert abs(f[0, 2] + loads[0, 2]) <= 1e-10
    diag = o.body_diagnostics()
    inst = diag["regime_instant"][0]
    assert inst[0] == 1 and inst[1] + inst[2] + inst[3] == inst[0]


def test_body_states():
    sc, ode = load_golden("body_states")
    o = Oracle(sc)
    o.run(ode["end"])
    b = o.bodies()
    assert np.all(np.abs(b["center"][0]) <= 1e-12) and np.all(np.abs(b["vel"][0]) <= 1e-12)
    assert abs(b["center"][1, 0] - 10.02) <= 1e-11
    assert abs(b["vel"][1, 0] - 2.0) <= 1e-12
    assert abs(b["omega"][1, 2] - 1.0) <= 1e-12
    assert abs(b["quat"][1, 3] - math.sin(0.005)) <= 2e-9


AREA_CASES = [
    # name, expected, sphere centre, radius, a, b, c  (contact_geometry_test.cpp:37-72)
    ("disk inside triangle", math.pi, (0, 0, 0), 1.0, (-10, -10, 0), (10, -10, 0), (0, 10, 0)),
    ("offset disk inside triangle", 0.64 * math.pi, (0, 0, 0.6), 1.0, (-10, -10, 0), (10, -10, 0), (0, 10, 0)),
    ("sphere tangent to plane", 0.0, (0, 0, 1), 1.0, (-10, -10, 0), (10, -10, 0), (0, 10, 0)),
    ("sphere misses plane", 0.0, (0, 0, 2), 1.0, (-10, -10, 0), (10, -10, 0), (0, 10, 0)),
    ("triangle inside disk", 0.5, (0, 0, 0), 10.0, (0, 0, 0), (1, 0, 0), (0, 1, 0)),
    ("disjoint", 0.0, (0, 0, 0), 1.0, (2, 2, 0), (3, 2, 0), (2, 3, 0)),
    ("half disk", 0.5 * math.pi, (0, 0, 0), 1.0, (0, -10, 0), (10, 0, 0), (0, 10, 0)),
    ("quarter disk", 0.25 * math.pi, (0, 0, 0), 1.0, (0, 0, 0), (10, 0, 0), (0, 10, 0)),
    ("reversed orientation", 0.25 * math.pi, (0, 0, 0), 1.0, (0, 10, 0), (10, 0, 0), (0, 0, 0)),
    ("degenerate triangle", 0.0, (0, 0, 0), 1.0, (0, 0, 0), (1, 0, 0), (2, 0, 0)),
    ("zero-radius sphere", 0.0, (0, 0, 0), 0.0, (-10, -10, 0), (10, -10, 0), (0, 10, 0)),
]


def sphere_triangle_area(center, radius, a, b, c):
    """The GPU disk routine fed the way bodyTriangleAreaScale feeds it: the
    cut disk of a sphere with the triangle plane."""
    a, b, c, p = (np.asarray(x, float) for x in (a, b, c, center))
    n = np.cross(b - a, c - a)
    ln = np.linalg.norm(n)
    if ln == 0.0:
        return 0.0
    n = n / ln
    dist = abs(np.dot(n, p - a))
    r2 = radius * radius - dist * dist
    if r2 <= 0.0:
        return 0.0
    ce = p - n * np.dot(n, p - a)
    return circle_triangle_area(ce, n, a, b, c, math.sqrt(r2))


@pytest.mark.parametrize("case", AREA_CASES, ids=[c[0] for c in AREA_CASES])
def test_disk_triangle_area(case):
    name, expected, center, radius, a, b, c = case
    got = sphere_triangle_area(center, radius, a, b, c)
    assert abs(got - expected) <= 1e-12 * max(1.0, abs(expected)), (name, got, expected)


def test_disk_triangle_area_scale_invariance():
    s = 1.0e6
    got = sphere_triangle_area((3 * s, -2 * s, 5 * s), s, (-7 * s, -12 * s, 5 * s), (13 * s, -12 * s, 5 * s),
                               (3 * s, 8 * s, 5 * s))
    assert abs(got - math.pi * s * s) <= 1e-12 * math.pi * s * s


def test_component_transform():
    """One owner rotated 90 deg about z, body offset (1,0,0)
    (component_transform_test.cu:64-104)."""
    kw = make_spheres([[3.0, 4.0, 5.0]], [0.5])
    h = math.sqrt(0.5)
    kw["quat"] = np.array([[h, 0, 0, h]])
    kw["vel"] = np.array([[0.1, 0.2, 0.3]])
    kw["omega"] = np.array([[0.0, 1.0, 0.0]])
    sc = Scene(**kw, comp_owner=np.array([0], np.int32), comp_id=np.array([0], np.int32),
               comp_radius=np.array([0.5]), comp_offset=np.array([[1.0, 0.0, 0.0]]))
    o = Oracle(sc)
    import ctypes as C
    from oracle.oracle import lib
    vh = np.array([[0.4, 0.5, 0.6]])
    wh = np.array([[1.0, 0.0, 0.0]])
    lib().orc_set_half(C.c_void_p(o.h), C.c_void_p(vh.ctypes.data), C.c_void_p(wh.ctypes.data))
    lib().orc_update_components(C.c_void_p(o.h))
    c = o.components()
    np.testing.assert_allclose(c["offset"][0], [0, 1, 0], atol=1e-14)
    np.testing.assert_allclose(c["pos"][0], [3, 5, 5], atol=1e-14)
    np.testing.assert_allclose(c["vel"][0], [0.1, 0.2, -0.7], atol=1e-14)
    np.testing.assert_allclose(c["vh"][0], [0.4, 0.5, 0.6], atol=1e-14)


def test_grid_is_stable_sort_of_keys():
    """sortedCellKey / sortedEntityId equal a stable sort of the packed keys
    (thrust::sort_by_key of a sequence, cuda_grid_backend.cu:121-145)."""
    from dem_mbd_cuda_gb300 import generate as G
    sc = G.small_dem(n=300, seed=11)
    o = Oracle(sc)
    o.compute_forces()
    keys, ids = o.grid()
    mesh = o.mesh_size()
    cell = np.floor(sc.pos * (1.0 / mesh)).astype(np.int64) + (1 << 20)
    packed = (cell[:, 0] << 42) | (cell[:, 1] << 21) | cell[:, 2]
    order = np.argsort(packed, kind="stable")
    np.testing.assert_array_equal(ids, order)
    np.testing.assert_array_equal(keys, packed[order].astype(np.uint64))


def test_history_expiry_semantics():
    """A contact missed for one step keeps its slot ("zombie") and is dropped
    the step after (expireHistory, cuda_contact_backend.cu:217-229)."""
    kw = make_spheres([[0.0, 0.0, 0.0], [0.0019, 0.0, 0.0]], [0.001, 0.001])
    kw["vel"] = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    from dem_mbd_cuda_gb300.generate import mech
    m = mech(kN=1e3, epsN=0.9, epsS=0.9, mu=0.3)
    sc = Scene(**kw, pp=m, pt=m, pw=m, dt=1e-4)
    o = Oracle(sc)
    o.compute_forces()
    keys, last, _ = o.history(0)
    assert keys[0, 0] == 2 and last[0, 0] == 0
    o.leapfrog_init(0.5e-4)
    for step in range(1, 5):
        o.advance(1e-4)
        o.compute_forces()
        o.finish(1e-4)
        keys, last, _ = o.history(0)
        d = abs(o.state()["pos"][1, 0] - o.state()["pos"][0, 0])
        if d < 0.002:
            assert keys[0, 0] == 2 and last[0, 0] == step
    # separated: the slot survives one step, then expires
    assert keys[0, 0] in (0, 2)


def test_oracle_planted_mistake_is_detected():
    """The parity checks are sensitive: a 1e-9 perturbation of one particle's
    position changes the oracle's forces by far more than the FP64 tolerance
    used in the GPU parity tests."""
    from dem_mbd_cuda_gb300 import generate as G
    sc = G.small_dem(n=200, seed=5)
    a = Oracle(sc)
    a.compute_forces()
    k = int(np.argmax(np.abs(a.forces()["contact"][:, :3]).sum(axis=1)))
    sc2 = sc.copy()
    sc2.pos[k, 0] += 1e-9
    b = Oracle(sc2)
    b.compute_forces()
    fa, fb = a.forces()["total"], b.forces()["total"]
    err = np.abs(fa - fb).max() / max(np.abs(fa).max(), 1e-30)
    assert err > 1e-9


def test_data1_mbd_reference_case_runs():
    """The reference's DATA1 validation inputs (1704 particles, 5 walls,
    2 x 1416 triangles) step through the oracle with contacts on both
    plates and no capacity overflow."""
    sc, ode = load_golden("data1_mbd")
    o = Oracle(sc, threads=4)
    loads = o.compute_forces(bodies=sc.body_states())
    st = o.stats()
    assert st["particle_contacts"] > 0 and st["body_contacts"] > 0
    assert st["particle_history_overflows"] == 0 and st["body_history_overflows"] == 0
    assert np.all(np.isfinite(loads))
