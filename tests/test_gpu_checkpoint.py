"""DMHIST2 checkpoints (saveContactHistory / loadContactHistory,
src/cuda_backend_cuda.cu:545-822)."""
import os

import numpy as np
import pytest

import dmhist2
from gpu_helpers import engine_for
from oracle.oracle import Oracle
from dem_mbd_cuda_gb300 import generate as G

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def test_save_matches_state_and_oracle(tmp_path):
    sc = G.small_mbd(n=200, seed=4, caps=False)
    e = engine_for(sc)
    o = Oracle(sc)
    e.run(6)
    o.run(6)
    path = str(tmp_path / "contact_history.bt")
    e.saveContactHistory(path)
    d = dmhist2.read(path)
    assert d["version"] == 2 and d["endian"] == 0x01020304 and d["slots"] == (64, 16, 64)
    assert d["topo_size"] == 40 and d["owner_size"] == 188
    assert d["owners"] == sc.n and d["comps"] == sc.n
    np.testing.assert_array_equal(d["topology"]["id"], sc.owner_id)
    np.testing.assert_array_equal(d["owner_state"]["id"], sc.owner_id)
    st = e.downloadParticleState()
    np.testing.assert_array_equal(d["owner_state"]["state"][:, 0:3], st["pos"])
    np.testing.assert_array_equal(d["owner_state"]["state"][:, 6:10], st["quat"])
    for kind in (0, 1, 2):
        k2, _, v2 = o.history(kind)
        np.testing.assert_array_equal(d["keys"][kind], k2)
        assert np.abs(d["values"][kind] - v2).max() <= 1e-9 * max(np.abs(v2).max(), 1e-30) + 1e-15


def test_load_roundtrip_is_byte_identical(tmp_path):
    sc = G.small_dem(n=250, seed=8)
    e = engine_for(sc)
    e.run(5)
    p1 = str(tmp_path / "a.bt")
    e.saveContactHistory(p1)
    f = engine_for(sc)
    f.loadContactHistory(p1)
    assert f.hasRestoredParticleLeapfrogState()
    p2 = str(tmp_path / "b.bt")
    f.saveContactHistory(p2)
    assert open(p1, "rb").read() == open(p2, "rb").read()


def test_restart_continues_like_the_reference(tmp_path):
    """After a load the next evaluation is the dt = 0 start evaluation and no
    half-step initialisation runs (src/cuda_simulation_integrator.cpp:249-261);
    the engine and a second engine restarted from the same file agree."""
    sc = G.small_dem(n=250, seed=8)
    e = engine_for(sc)
    e.run(5)
    p1 = str(tmp_path / "a.bt")
    e.saveContactHistory(p1)
    f = engine_for(sc)
    g = engine_for(sc)
    f.loadContactHistory(p1)
    g.loadContactHistory(p1)
    f.run(4)
    g.run(4)
    np.testing.assert_array_equal(f.downloadParticleState()["pos"], g.downloadParticleState()["pos"])


@pytest.mark.parametrize("damage", ["truncated", "magic", "owners"])
def test_load_rejects_bad_files(tmp_path, damage):
    sc = G.small_dem(n=120, seed=6)
    e = engine_for(sc)
    e.run(2)
    p = str(tmp_path / "a.bt")
    e.saveContactHistory(p)
    raw = bytearray(open(p, "rb").read())
    if damage == "truncated":
        raw = raw[:-100]
    elif damage == "magic":
        raw[6] = ord("9")
    else:
        raw[16] ^= 1
    open(p, "wb").write(bytes(raw))
    f = engine_for(sc)
    with pytest.raises(RuntimeError):
        f.loadContactHistory(p)
