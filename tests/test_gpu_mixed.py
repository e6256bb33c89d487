"""Mixed form (FP32 particle-particle and wall law, FP64 state, overlaps,
contact decisions and particle-triangle contacts) against the FP64 oracle.

Contact decisions use the FP64 overlap test, so the contact lists stay
bit-exact; forces carry FP32 rounding (bar: 1e-5 of the largest force); body
loads come from the FP64 particle-triangle path (bar: 1e-9 relative at the
first evaluation, where the states are identical)."""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import engine_for
from oracle.oracle import Oracle
from dem_mbd_cuda_gb300 import generate as G

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


@pytest.mark.parametrize("maker", ["small_dem", "small_mbd", "data1_mbd"])
def test_mixed_first_evaluation(maker):
    sc = load_golden(maker)[0] if maker.startswith("data1") else getattr(G, maker)()
    e = engine_for(sc, precision="mixed")
    o = Oracle(sc)
    bs = sc.body_states() if sc.n_bodies else None
    le = e.computeForces(0.0, bs, True, True)
    lo = o.compute_forces(bs)
    ke, ie = e.grid()
    ko, io = o.grid()
    np.testing.assert_array_equal(ie, io)
    np.testing.assert_array_equal(ke, ko)
    for kind in (0, 1, 2):
        k1, l1, _ = e.history(kind)
        k2, l2, _ = o.history(kind)
        np.testing.assert_array_equal(k1, k2)
        np.testing.assert_array_equal(l1, l2)
    fe, fo = e.downloadForceOutput(False, False), o.forces()
    for name in ("contact", "wall", "total"):
        scale = max(np.abs(fo[name][:, :3]).max(), 1e-30)
        assert np.abs(fe[name][:, :3] - fo[name][:, :3]).max() <= 1e-5 * scale, name
    if sc.n_bodies:
        assert np.abs(le - lo).max() <= 1e-9 * np.abs(lo).max()
    assert e.stepStats()["particle_contacts"] == o.stats()["particle_contacts"]


def test_mixed_pt_fp32_option():
    """With the particle-triangle law in FP32 too, body loads carry FP32
    error (bar 1e-4 relative), but the set of manifolds is the FP64 one:
    areas that decide the 1e-12 cut are recomputed in FP64."""
    sc = G.small_mbd()
    e = engine_for(sc, precision="mixed", pt_fp32=True)
    o = Oracle(sc)
    le = e.computeForces(0.0, sc.body_states(), True, True)
    lo = o.compute_forces(sc.body_states())
    assert np.abs(le - lo).max() <= 1e-4 * np.abs(lo).max()
    assert e.stepStats()["body_contacts"] == o.stats()["body_contacts"]
    k1, _, _ = e.history(2)
    k2, _, _ = o.history(2)
    np.testing.assert_array_equal(k1, k2)


def test_mixed_trajectory_stays_close():
    sc = G.small_dem(n=400, seed=9)
    e = engine_for(sc, precision="mixed")
    o = Oracle(sc)
    e.run(20)
    o.run(20)
    pe, po = e.downloadParticleState()["pos"], o.state()["pos"]
    assert np.abs(pe - po).max() <= 1e-9
