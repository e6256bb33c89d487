"""Speed settings change no result: the blocks per SM of the sweep, the
gathers and the particle law (grid-stride) leave the trajectory, the bodies
and the contact histories bit-identical, also where a component holds more
than a warp's width of contacts;
the autotuner returns a setting the engine accepts."""
import dataclasses

import numpy as np
import pytest

from gpu_helpers import compare_evaluation, engine_for
from oracle.oracle import Oracle
from dem_mbd_cuda_gb300 import generate as G

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("maker", ["small_dem", "small_mbd"])
def test_sweep_blocks_do_not_change_results(precision, maker):
    sc = getattr(G, maker)()
    runs = []
    for blocks in (0, 1, 3):
        e = engine_for(sc, precision=precision).set_sweep_blocks(blocks).set_gather_blocks(1 + blocks)
        e.set_pp_blocks(2 * blocks)
        e.run(15)
        runs.append(e)
    ref = runs[0]
    _assert_same_runs(sc, ref, runs[1:])


def _assert_same_runs(sc, ref, others):
    st0 = ref.downloadParticleState()
    for e in others:
        st = e.downloadParticleState()
        for k in ("pos", "vel", "omega", "quat"):
            np.testing.assert_array_equal(st[k], st0[k], err_msg=k)
        for kind in (0, 1, 2):
            k1, l1, v1 = e.history(kind)
            k2, l2, v2 = ref.history(kind)
            np.testing.assert_array_equal(k1, k2)
            np.testing.assert_array_equal(l1, l2)
            np.testing.assert_array_equal(v1, v2)
        if sc.n_bodies:
            np.testing.assert_array_equal(e.bodies()["loads"], ref.bodies()["loads"])


def crowded(counts=(60, 40, 20), big=8e-3, small=1e-3, overlap=2e-6):
    """Large spheres each covered by small ones that all touch it: a large
    component holds more than 32 contacts, and more than the 64 history
    slots where its count is above 64 (the reference's capacity error).
    The small spheres stand more than 3 mm apart, clear of one another."""
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
    pos, rad = np.array(pos), np.array(rad)
    kw = G.make_spheres(pos, rad, G.DENSITY)
    wo, wn = G.box_walls(np.array([-0.06, -0.03, 0.0]), np.array([0.06, 0.03, 0.06]))
    m = G.mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=0.1, muR=0.05, beta=0.5)
    return G.Scene(**kw, pp=m, pt=m, pw=m, dt=1e-6, gravity=(0.0, 0.0, -9.81), gravity_enabled=1, wall_origin=wo,
                   wall_normal=wn, name="crowded")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_crowded_components(precision):
    """Up to 60 contacts on one component: every sweep grid agrees bit for
    bit, and (FP64) with the oracle; 80 contacts on one component is the
    capacity error, as in the oracle."""
    sc = crowded()
    runs = [engine_for(sc, precision=precision).set_sweep_blocks(b) for b in (0, 1)]
    for e in runs:
        e.run(4)
    st = runs[0].stepStats()
    assert st["particle_history_overflows"] == 0 and st["particle_history_high_water"] == 60
    _assert_same_runs(sc, runs[0], runs[1:])
    if precision == "fp64":
        o = Oracle(sc)
        o.run(4)
        for e in runs:
            compare_evaluation(e, o, 4)
    over = crowded(counts=(80,))
    with pytest.raises(RuntimeError, match="capacity"):
        Oracle(over).run(1)
    with pytest.raises(Exception, match="capacity"):
        engine_for(over, precision=precision).run(1)


def test_autotune_returns_an_accepted_setting():
    from dem_mbd_cuda_gb300.autotune import autotune
    sc = G.small_mbd()
    out = autotune(sc, factors=(2.5, 3.0), sweep_blocks=(2, 4), gather_blocks=(1, 8), warp_items=(512,),
                   skins=(0, 500), steps=3, warmup=2)
    assert out["cell_factor"] in (2.5, 3.0)
    assert out["nl_skin"] in (None, 0, 500)
    assert out["sweep_blocks"] in (None, 2, 4)
    assert out["gather_blocks"] in (None, 1, 8)
    assert out["pt_warp_items"] in (None, 512)
    assert out["ms_per_step"] > 0 and out["default_ms_per_step"] > 0
    assert len(out["table"]) == 2 + 2 + 2 + 2 + 1
    e = engine_for(sc, precision="mixed", cell_factor=out["cell_factor"])
    if out["nl_skin"] is not None:
        e.set_neighbor_lists(out["nl_skin"] > 0, out["nl_skin"] or None)
    if out["sweep_blocks"] is not None:
        e.set_sweep_blocks(out["sweep_blocks"])
    if out["gather_blocks"] is not None:
        e.set_gather_blocks(out["gather_blocks"])
    if out["pt_warp_items"] is not None:
        e.set_pt_warp_items(out["pt_warp_items"])
    e.run(3)
    assert e.stepStats()["particle_contacts"] > 0


def test_candidate_counts_bound_the_contacts():
    """The engine-only step stats: the particle-triangle items the FP32
    probe kept cover every particle with a body contact, and the wall
    candidates every particle with a wall contact (FP32 tests reject only
    pairs that are certainly apart)."""
    sc = G.small_mbd()
    e = engine_for(sc, precision="mixed")
    e.run(5)
    st = e.stepStats()
    _, l_body, _ = e.history(2)
    _, l_wall, _ = e.history(1)
    step = max(int(l_body.max()), int(l_wall.max()))  # the last evaluation
    with_body = int((l_body == step).any(axis=1).sum())
    with_wall = int((l_wall == step).any(axis=1).sum())
    assert st["body_candidate_items"] >= with_body > 0
    assert st["wall_candidates"] >= with_wall


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("maker", ["plate_on_monolayer", "small_mbd", "clumps"])
def test_run_split_into_calls_gives_the_same_bits(maker, precision):
    """A run of 24 steps as one call, as 8 + 8 + 8, as 24 single steps and
    as 12 + 12 with the state read between the calls, and as 1 + 23 timed
    steps (whose last step runs the whole finish).  The first step of
    each call advances in other kernels than the steps inside a call; a call
    leaves its last quaternion rate to the next call's first advance, or to
    the read in between.  All round alike: the state and the half-step
    state (velocities, spins, quaternion rates, accelerations) are the same
    bits."""
    sc = getattr(G, maker)()
    runs = []
    for parts in ([24], [8, 8, 8], [1] * 24, [12, "read", 12], [1, "timed 23"]):
        e = engine_for(sc, precision=precision)
        for p in parts:
            if p == "read":
                e.downloadParticleState()
            elif p == "timed 23":
                e.time_steps(23)  # ends with the whole finish
            else:
                e.run(p)
        runs.append(e)
    ref = runs[0].downloadParticleState()
    ref_half = runs[0].downloadHalfState()
    for e in runs[1:]:
        st = e.downloadParticleState()
        for k in ("pos", "vel", "omega", "quat"):
            np.testing.assert_array_equal(st[k], ref[k], err_msg=k)
        half = e.downloadHalfState()
        for k in ("vh", "wh", "hdq", "acc", "aacc"):
            np.testing.assert_array_equal(half[k], ref_half[k], err_msg=k)
        np.testing.assert_array_equal(e.bodies()["center"], runs[0].bodies()["center"])
        np.testing.assert_array_equal(e.bodies()["quat"], runs[0].bodies()["quat"])


@pytest.mark.parametrize("maker", ["small_dem", "small_mbd", "plate_on_monolayer"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_neighbor_lists_give_the_cell_sweep_bits(maker, precision):
    """The sweep from neighbour lists takes the contacts in the cell sweep's
    order: trajectories, bodies and histories are bit-identical, with the
    default skin (few rebuilds) and with a skin so thin that the lists are
    rebuilt every few steps."""
    sc = getattr(G, maker)()
    runs = [engine_for(sc, precision=precision).set_neighbor_lists(False)]
    for permille in (500, 2):
        e = engine_for(sc, precision=precision).set_neighbor_lists(True, permille)
        runs.append(e)
    for e in runs:
        e.run(40)
    _assert_same_runs(sc, runs[0], runs[1:])


def test_neighbor_lists_with_crowded_components():
    """Up to 60 contacts on one component (lists of up to 32 partners
    overflow: those steps sweep the cells)."""
    sc = crowded()
    ref = engine_for(sc, precision="fp64").set_neighbor_lists(False)
    e = engine_for(sc, precision="fp64").set_neighbor_lists(True)
    for x in (ref, e):
        x.run(6)
    _assert_same_runs(sc, ref, [e])


def test_neighbor_lists_with_a_fast_mover():
    """One sphere thrown through a resting bed: it passes half the skin within
    a few steps, its neighbourhoods sweep the cells while every other
    component keeps its list (no global rebuild), and the run equals the
    cell sweep bit for bit."""
    sc = G.small_dem(n=400, seed=12, vel_std=0.0, omega_std=0.0)
    vel = np.zeros_like(sc.pos)
    k = int(np.argmax(sc.pos[:, 2]))
    vel[k] = [3.0, 0.0, -3.0]
    sc = dataclasses.replace(sc, vel=vel)
    ref = engine_for(sc, precision="fp64").set_neighbor_lists(False)
    e = engine_for(sc, precision="fp64").set_neighbor_lists(True)
    for x in (ref, e):
        x.run(60)
    st = e.neighbor_stats()
    assert st["builds"] == 1, st
    _assert_same_runs(sc, ref, [e])
