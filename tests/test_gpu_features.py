"""Features beyond the benchmark configs, checked against the reference's
own CUDA kernels (oracle/_ref/ref_engine.cubin through
oracle/ref_cuda_host.cu) and the CPU oracle:

* clump owners of 1 to 8 components (src/cuda_backend_cuda.cu:121-190,
  src/cuda/cuda_particle_backend.cu:103-147), their trajectories and a
  DMHIST2 round trip with clump topology;
* universal gravitation (src/cuda/cuda_contact_backend.cu:1095-1106);
* the diagnostic observers: regime counters, the 22-value microstate sums
  and the bodyParticle / bodyDetail outputs
  (src/cuda/cuda_contact_backend.cu:530-567,1226-1356, :820-842);
* the triangle grid (src/cuda/cuda_contact_backend.cu:409-476,1567-1610);
* history slots near the 64-slot capacity and its overflow error
  (src/cuda_backend_cuda.cu:500-502).
"""
import numpy as np
import pytest

import dmhist2
from gpu_helpers import close, compare_evaluation, engine_for, forces_of, state_of
from oracle import ref_cuda
from oracle.oracle import Oracle
from conftest import load_golden
from dem_mbd_cuda_gb300 import generate as G

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(), reason="reference device code not built")]


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def _first(x, sc):
    bodies = sc.body_states() if sc.n_bodies else None
    if hasattr(x, "computeForces"):
        return x.computeForces(0.0, bodies, True, True)
    return x.compute_forces(bodies)


def _trajectory_parity(sc, steps, runs):
    r = ref_cuda.RefCuda(sc)
    r.run(steps)
    sr = r.state()
    for x in runs:
        x.run(steps)
        sx = state_of(x)
        for k in ("pos", "vel", "quat"):
            close(sx[k], sr[k], what=k)
        close(sx["omega"], sr["omega"], atol=1e-6, what="omega")
        for kind in (0, 1):
            k1, l1, v1 = x.history(kind)
            k2, l2, v2 = r.history(kind)
            np.testing.assert_array_equal(k1, k2, err_msg=f"history keys kind {kind}")
            np.testing.assert_array_equal(l1, l2, err_msg=f"history last-seen kind {kind}")
            assert np.abs(v1 - v2).max() <= 1e-6 * max(np.abs(v2).max(), 1e-30) + 1e-15
    return r


def test_clumps_single_evaluation():
    sc = G.clumps()
    assert sc.n_components > 3 * sc.n
    r, o, e = ref_cuda.RefCuda(sc), Oracle(sc), engine_for(sc)
    for x in (r, o, e):
        _first(x, sc)
    cr = r.components()
    co = o.components()
    for k in ("pos", "vel", "offset"):
        close(co[k], cr[k], atol=1e-15, what="component " + k)
    compare_evaluation(o, r)
    compare_evaluation(e, r)


def test_clumps_trajectory():
    sc = G.clumps()
    _trajectory_parity(sc, 30, [Oracle(sc), engine_for(sc)])


def test_clump_checkpoint_roundtrip(tmp_path):
    """The engine's DMHIST2 file of a clump scene carries the reference's
    component topology (stable id, owner id, radius, body offset) and the
    reference kernels' history slots; load then save is byte-identical."""
    sc = G.clumps()
    e = engine_for(sc)
    e.run(12)
    r = ref_cuda.RefCuda(sc)
    r.run(12)
    p1 = str(tmp_path / "clumps.bt")
    e.saveContactHistory(p1)
    d = dmhist2.read(p1)
    assert d["owners"] == sc.n and d["comps"] == sc.n_components
    order = np.lexsort((sc.comp_id, sc.comp_owner))
    np.testing.assert_array_equal(d["topology"]["id"], sc.comp_id[order])
    np.testing.assert_array_equal(d["topology"]["owner"], sc.owner_id[sc.comp_owner[order]])
    np.testing.assert_array_equal(d["topology"]["geo"][:, 0], sc.comp_radius[order])
    np.testing.assert_array_equal(d["topology"]["geo"][:, 1:4], sc.comp_offset[order])
    for kind in (0, 1, 2):
        k2, _, v2 = r.history(kind)
        np.testing.assert_array_equal(d["keys"][kind], k2)
        assert np.abs(d["values"][kind] - v2).max() <= 1e-6 * max(np.abs(v2).max(), 1e-30) + 1e-15
    f = engine_for(sc)
    f.loadContactHistory(p1)
    p2 = str(tmp_path / "again.bt")
    f.saveContactHistory(p2)
    assert open(p1, "rb").read() == open(p2, "rb").read()


def test_universal_gravitation():
    sc = G.universal_gravity()
    r, o, e = ref_cuda.RefCuda(sc), Oracle(sc), engine_for(sc)
    for x in (r, o, e):
        _first(x, sc)
    fr = r.forces()["field"]
    assert np.abs(fr).max() > 1e-2                      # the attraction is on and above rounding
    compare_evaluation(o, r)
    compare_evaluation(e, r)
    _trajectory_parity(sc, 10, [Oracle(sc), engine_for(sc)])


@pytest.mark.parametrize("name,steps", [("small_mbd_nocap", 0), ("small_mbd_nocap", 6), ("data1_mbd", 0)])
def test_observers_and_body_outputs(name, steps):
    """Regime counters (exact), microstate sums, bodyParticle and bodyDetail
    of the engine and the oracle against the reference's kernels: the dt = 0
    start evaluation, and the reference's loop over a few steps on a scene
    whose manifolds stay below their caps (where a cap binds, the branch and
    with it the regime bits follow the last bit of a rounding)."""
    if name == "small_mbd_nocap":
        sc = G.small_mbd(caps=False)
    else:
        sc = load_golden(name)[0]
        sc.keep_body_particle, sc.keep_body_detail = 1, 1
    r, o, e = ref_cuda.RefCuda(sc), Oracle(sc), engine_for(sc)
    for x in (r, o, e):
        if steps:
            x.run(steps)
        else:
            _first(x, sc)
    dr = r.body_diagnostics()
    fr = r.forces()
    assert dr["regime_instant"].sum() > 0
    for who, x, dx in (("oracle", o, o.body_diagnostics()), ("engine", e, e.bodyDiagnostics())):
        np.testing.assert_array_equal(dx["regime_instant"], dr["regime_instant"], err_msg=who)
        np.testing.assert_array_equal(dx["regime_interval"], dr["regime_interval"], err_msg=who)
        for k in ("micro_instant", "micro_interval"):
            scale = max(np.abs(dr[k]).max(), 1e-30)
            assert np.abs(dx[k] - dr[k]).max() <= 1e-8 * scale + 1e-15, (who, k)
        fx = forces_of(x)
        for k in ("body_particle", "body_detail"):
            scale = max(np.abs(fr[k]).max(), 1e-30)
            assert np.abs(fx[k] - fr[k]).max() <= 1e-8 * scale + 1e-15, (who, k)


@pytest.mark.parametrize("name", ["small_mbd", "data1_mbd"])
def test_triangle_grid(name):
    """The oracle's triangle grid equals the reference kernels' bit for bit;
    the engine keeps exactly the reference's entries whose cell lies in the
    particles' cell box (the only cells ever looked up)."""
    sc = G.small_mbd() if name == "small_mbd" else load_golden(name)[0]
    r, o, e = ref_cuda.RefCuda(sc), Oracle(sc), engine_for(sc)
    for x in (r, o, e):
        _first(x, sc)
    kr, ir = r.triangle_grid()
    ko, io = o.triangle_grid()
    np.testing.assert_array_equal(ko, kr)
    np.testing.assert_array_equal(io, ir)
    tw_r, ab_r = r.world_triangles()
    tw_o, ab_o = o.world_triangles()
    close(tw_o, tw_r, atol=1e-15, what="world triangles")
    close(ab_o, ab_r, atol=1e-15, what="triangle boxes")

    def cells(keys):
        k = keys.astype(np.uint64)
        m = np.uint64((1 << 21) - 1)
        return np.stack([(k >> np.uint64(42)) & m, (k >> np.uint64(21)) & m, k & m], axis=1).astype(np.int64)

    pc = cells(r.grid()[0])
    tc = cells(kr)
    inside = np.all((tc >= pc.min(0)) & (tc <= pc.max(0)), axis=1)
    assert e.triangleGridEntryCount() == int(inside.sum())


def _crowded(counts=(60, 30)):
    """Large spheres each ringed by `counts` small touching spheres."""
    big, small, overlap = 4e-3, 0.6e-3, 1e-6
    pos, rad = [], []
    for k, m in enumerate(counts):
        c = np.array([0.03 * k - 0.03, 0.0, 0.02])
        pos.append(c)
        rad.append(big)
        i = np.arange(m) + 0.5
        th = np.arccos(1 - 2 * i / m)
        ph = np.pi * (1 + 5 ** 0.5) * i
        d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
        pos.extend(c + (big + small - overlap) * d)
        rad.extend([small] * m)
    kw = G.make_spheres(np.array(pos), np.array(rad), G.DENSITY)
    wo, wn = G.box_walls(np.array([-0.06, -0.03, 0.0]), np.array([0.06, 0.03, 0.06]))
    m = G.mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=0.1, muR=0.05, beta=0.5)
    return G.Scene(**kw, pp=m, pt=m, pw=m, dt=1e-6, gravity=(0.0, 0.0, -9.81), gravity_enabled=1, wall_origin=wo,
                   wall_normal=wn, name="crowded")


def test_history_near_capacity_and_overflow():
    """60 contacts on one component (slot high-water 60 of 64) match the
    reference kernels slot for slot; 80 is the reference's capacity error in
    the reference, the oracle and the engine."""
    sc = _crowded()
    r, e = ref_cuda.RefCuda(sc), engine_for(sc)
    r.run(4)
    e.run(4)
    assert r.stats()["particle_history_high_water"] == 60
    compare_evaluation(e, r)
    over = _crowded(counts=(80,))
    for make in (ref_cuda.RefCuda, Oracle, engine_for):
        with pytest.raises(Exception, match="capacity"):
            make(over).run(1)
