"""Batched scenes (segmented cell tables, per-scene walls, bodies and
materials) advance exactly like the same scenes run one by one."""
import numpy as np
import pytest

from gpu_helpers import engine_for
from dem_mbd_cuda_gb300 import generate as G
from dem_mbd_cuda_gb300.engine import CudaDemSolver

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def scenes():
    a = G.small_dem(n=300, seed=1)
    b = G.small_dem(n=200, seed=2)
    b.pp.mu = b.pw.mu = 0.7
    b.pp.epsN = b.pw.epsN = 0.3
    b.pos = b.pos + np.array([0.001, -0.002, 0.0])   # overlapping coordinates on purpose
    c = G.small_mbd(n=250, seed=3, caps=False, dt=a.dt)
    return [a, b, c]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_individual_runs(precision):
    sc = scenes()
    steps = 12
    batch = CudaDemSolver().initialize(sc, precision=precision)
    batch.run(steps)
    st = batch.downloadParticleState()
    off = 0
    for s in sc:
        e = engine_for(s, precision=precision)
        e.run(steps)
        si = e.downloadParticleState()
        for k in ("pos", "vel", "omega", "quat"):
            np.testing.assert_array_equal(st[k][off:off + s.n], si[k], err_msg=f"{s.name} {k}")
        off += s.n
    bodies = batch.bodies()
    e = engine_for(sc[2], precision=precision)
    e.run(steps)
    np.testing.assert_array_equal(bodies["center"][0], e.bodies()["center"][0])


def test_batch_rejects_mixed_dt():
    sc = scenes()
    sc[1].dt = sc[0].dt * 2
    with pytest.raises(RuntimeError, match="dt"):
        CudaDemSolver().initialize(sc)
