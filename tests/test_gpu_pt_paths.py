"""The two particle-triangle kernels (one warp per contact item for small
counts, one thread per item for large ones) against the oracle and against
each other.

Both take the manifold and per-triangle sums in triangle order, so they must
agree bit for bit; each must match the oracle to the same bar as the rest of
the engine.  The crossover is forced with the engine's set_pt_warp_items.
"""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import close, compare_evaluation, engine_for
from oracle.oracle import Oracle
from dem_mbd_cuda_gb300 import generate as G

pytestmark = pytest.mark.gpu

WARP, THREAD = 1 << 30, -1


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def _scene(maker):
    if maker == "data1_mbd":
        return load_golden(maker)[0]
    if maker == "small_mbd_nocap":
        return G.small_mbd(caps=False)
    return G.small_mbd()


@pytest.mark.parametrize("path", [WARP, THREAD], ids=["warp", "thread"])
@pytest.mark.parametrize("maker", ["small_mbd", "data1_mbd"])
def test_pt_path_single_evaluation(maker, path):
    sc = _scene(maker)
    e = engine_for(sc).set_pt_warp_items(path)
    o = Oracle(sc)
    bodies = sc.body_states()
    le = e.computeForces(0.0, bodies, True, True)
    lo = o.compute_forces(bodies)
    compare_evaluation(e, o, 0)
    assert np.abs(le - lo).max() <= 1e-9 * np.abs(lo).max() + 1e-12


@pytest.mark.parametrize("precision,scene", [("fp64", "small"), ("mixed", "small"), ("fp64", "drum")])
def test_pt_paths_bit_identical(precision, scene):
    """small_mbd: about 100 items, the warp kernel's paired mode (a block per
    item, the second warp computing the microstate); the drum generator at
    40,000 spheres: several thousand items, more than the paired blocks
    resident at once, so the forced warp kernel runs one item per warp."""
    if scene == "small":
        sc = G.small_mbd(caps=False)
    else:
        import torch
        sc = G.drum(n=40000)[0]
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        e = engine_for(sc)
        e.run(1)
        items = e.stepStats()["body_candidate_items"]
        assert items > 4 * sms, (items, sms)
        del e
    out = []
    for path in (WARP, THREAD):
        e = engine_for(sc, precision=precision).set_pt_warp_items(path)
        e.run(12)
        k, l, v = e.history(2)
        out.append((e.downloadParticleState(), e.bodies(), e.downloadForceOutput(), k, l, v))
    (sa, ba, fa, ka, la, va), (sb, bb, fb, kb, lb, vb) = out
    for name in ("pos", "vel", "omega", "quat"):
        np.testing.assert_array_equal(sa[name], sb[name], err_msg=name)
    for name in ("center", "quat", "vel", "omega", "loads"):
        np.testing.assert_array_equal(ba[name], bb[name], err_msg="body " + name)
    for name in ("contact", "wall", "total"):
        np.testing.assert_array_equal(fa[name], fb[name], err_msg=name)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(la, lb)
    np.testing.assert_array_equal(va, vb)


def test_thread_path_trajectory_parity():
    sc = G.small_mbd(caps=False)
    steps = 25
    e = engine_for(sc).set_pt_warp_items(THREAD)
    o = Oracle(sc)
    e.run(steps)
    o.run(steps)
    se, so = e.downloadParticleState(), o.state()
    for k in ("pos", "vel", "quat"):
        close(se[k], so[k], what=k)
    be, bo = e.bodies(), o.bodies()
    for k in ("center", "quat", "vel", "omega"):
        close(be[k], bo[k], what="body " + k)
    close(be["loads"], bo["loads"], atol=1e-8 + 1e-6 * np.abs(bo["loads"]).max(), what="body loads")
