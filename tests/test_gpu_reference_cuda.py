"""The oracle and the engine against the reference's own CUDA engine.

The reference's kernels are compiled from its src/cuda/*.cu (the way its
CMakeLists.txt builds them) into oracle/_ref/ref_engine.cubin and run
through oracle/ref_cuda_host.cu, a restatement of its host glue
(src/cuda_backend_cuda.cu:302-524).  These tests pin the CPU oracle to the
reference's own FP64 results -- the tangential, twisting and rolling history
channels, the particle-triangle manifold and the integrator included -- and
check the engine against the reference directly.

Bars: sorted cell keys and ids, history keys and last-seen steps (the
contact lists) and the contact counters bit for bit; forces and history
values within 1e-9 of the largest value for one evaluation; states and body
loads over several steps within the reference's own bar 1e-8 + 1e-9 |ref|
(docs/CUDA_MIGRATION_VALIDATION.md:73).
"""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import close, compare_evaluation, engine_for, state_of
from oracle import ref_cuda
from oracle.oracle import Oracle
from dem_mbd_cuda_gb300 import generate as G

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(), reason="reference device code not built")]


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def scene(name):
    if name in ("wall_contact", "two_particle", "triangle_contact", "free_fall", "body_states",
                "data1_pure_dem", "data1_mbd"):
        return load_golden(name)[0]
    if name == "small_mbd_nocap":
        return G.small_mbd(caps=False)
    return getattr(G, name)()


def first_evaluation(x, sc):
    return x.compute_forces(sc.body_states() if sc.n_bodies else None) if not hasattr(x, "computeForces") else \
        x.computeForces(0.0, sc.body_states() if sc.n_bodies else None, True, True)


@pytest.mark.parametrize("name", ["wall_contact", "two_particle", "triangle_contact", "free_fall"])
def test_reference_kernels_give_the_reference_known_answers(name):
    """The launcher reproduces the reference's own analytic checks
    (tests/scenario_validator.cpp:80-113) with the reference's kernels."""
    sc = scene(name)
    r = ref_cuda.RefCuda(sc)
    loads = first_evaluation(r, sc)
    f = r.forces()
    if name == "wall_contact":
        assert abs(f["wall"][0, 2] - 100.0) <= 1e-9 and abs(f["total"][0, 2] - 100.0) <= 1e-9
    elif name == "two_particle":
        assert abs(f["contact"][0, 0] + 100) <= 1e-9 and abs(f["contact"][1, 0] - 100) <= 1e-9
        assert abs(f["contact"][0, 0] + f["contact"][1, 0]) <= 1e-12
    elif name == "triangle_contact":
        assert abs(f["total"][0, 2] - 100.0) <= 1e-8 and abs(loads[0, 2] + 100.0) <= 1e-8
    else:
        assert abs(f["total"][0, 2] + 9.8) <= 2e-12


@pytest.mark.parametrize("name", ["small_dem", "small_mbd", "data1_pure_dem", "data1_mbd", "triangle_contact"])
def test_oracle_single_evaluation_matches_reference_kernels(name):
    sc = scene(name)
    r = ref_cuda.RefCuda(sc)
    o = Oracle(sc)
    lr = first_evaluation(r, sc)
    lo = first_evaluation(o, sc)
    compare_evaluation(o, r)
    if sc.n_bodies:
        assert np.abs(lo - lr).max() <= 1e-9 * np.abs(lr).max() + 1e-12


@pytest.mark.parametrize("name", ["small_dem", "small_mbd", "data1_pure_dem", "data1_mbd"])
def test_engine_single_evaluation_matches_reference_kernels(name):
    sc = scene(name)
    r = ref_cuda.RefCuda(sc)
    e = engine_for(sc)
    lr = first_evaluation(r, sc)
    le = first_evaluation(e, sc)
    compare_evaluation(e, r)
    if sc.n_bodies:
        assert np.abs(le - lr).max() <= 1e-9 * np.abs(lr).max() + 1e-12


@pytest.mark.parametrize("name", ["small_dem", "small_mbd_nocap", "data1_pure_dem"])
def test_oracle_and_engine_trajectories_match_reference_kernels(name):
    """25 steps of the reference's loop: random velocities and spins load
    the tangential, twisting and rolling channels (small_dem), and the
    particle-triangle manifold history (small_mbd_nocap)."""
    sc = scene(name)
    steps = 25
    r = ref_cuda.RefCuda(sc)
    o = Oracle(sc)
    e = engine_for(sc)
    for x in (r, o, e):
        x.run(steps)
    sr = r.state()
    for other in (o, e):
        so = state_of(other)
        for k in ("pos", "vel", "quat"):
            close(so[k], sr[k], what=k)
        close(so["omega"], sr["omega"], atol=1e-6, what="omega")
        k1, l1, v1 = other.history(0)
        k2, l2, v2 = r.history(0)
        np.testing.assert_array_equal(k1, k2)
        np.testing.assert_array_equal(l1, l2)
        # history values integrate the state's rounding differences over the
        # steps through the contact stiffness
        assert np.abs(v1 - v2).max() <= 1e-6 * np.abs(v2).max() + 1e-15
        if sc.n_bodies:
            bo, br = other.bodies(), r.bodies()
            for k in ("center", "quat", "vel", "omega"):
                close(bo[k], br[k], what="body " + k)
            close(bo["loads"], br["loads"], atol=1e-8 + 1e-6 * np.abs(br["loads"]).max(), what="body loads")
            k1, l1, v1 = other.history(2)
            k2, l2, v2 = r.history(2)
            np.testing.assert_array_equal(k1, k2)
            assert np.abs(v1 - v2).max() <= 1e-6 * np.abs(v2).max() + 1e-15


def _config_scene(name):
    if name == "c0":
        return G.pure_dem()
    if name == "c1":
        return G.mbd_blade_plate()[0]
    return G.drum()[0]


@pytest.mark.parametrize("name,steps", [("c0", 3), ("c1", 1), ("drum", 3)])
def test_engine_matches_reference_kernels_at_config_size(name, steps):
    """The benchmark scenes at full size: config 0 (20,000 spheres, 5
    walls), config 1 (200,000 spheres, blade and plate, 2,216 triangles) and
    the 2M-sphere drum (19,520 triangles).  The start evaluation gives the
    reference's grid, contact lists and counters bit for bit and its forces
    and body loads within 1e-9; after a few steps the contact lists are still
    identical and the states within the reference's bar.  (Config 1 is held
    to one step: its blade manifolds slide at their Coulomb caps, where the
    reference's branch is decided by the last bit of a rounding -- see the
    knife-edge test below.)"""
    import gc
    sc = _config_scene(name)
    r = ref_cuda.RefCuda(sc)
    e = engine_for(sc)
    lr = first_evaluation(r, sc)
    le = first_evaluation(e, sc)
    compare_evaluation(e, r)
    if sc.n_bodies:
        assert np.abs(le - lr).max() <= 1e-9 * np.abs(lr).max() + 1e-12
    del r, e
    gc.collect()
    r = ref_cuda.RefCuda(sc)
    r.run(steps)
    sr = r.state()
    kr, lr_, _ = r.history(0)
    br = r.bodies() if sc.n_bodies else None
    del r
    gc.collect()
    e = engine_for(sc)
    e.run(steps)
    se = state_of(e)
    for k in ("pos", "vel", "quat"):
        close(se[k], sr[k], what=k)
    ke, le_, _ = e.history(0)
    np.testing.assert_array_equal(ke, kr)
    np.testing.assert_array_equal(le_, lr_)
    if br is not None:
        be = e.bodies()
        close(be["loads"], br["loads"], atol=1e-8 + 1e-6 * np.abs(br["loads"]).max(), what="body loads")


def test_batch_matches_reference_kernels_scene_by_scene():
    """Eight config-4 box scenes (2,000-40,000 spheres, their own friction
    and restitution) in one batched engine against each scene run alone by
    the reference's kernels: contact lists slot for slot and states within
    the reference's bar after 3 steps."""
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    scenes = G.batch(nscenes=8, settled=True)
    steps = 3
    b = CudaDemSolver().initialize(scenes, precision="fp64")
    b.run(steps)
    sb = b.downloadParticleState()
    hb = [b.history(kind) for kind in (0, 1)]
    off = 0
    for s in scenes:
        r = ref_cuda.RefCuda(s)
        r.run(steps)
        sr = r.state()
        for k in ("pos", "vel", "quat"):
            close(sb[k][off:off + s.n], sr[k], what=f"{s.name} {k}")
        for kind in (0, 1):
            kr, lr, _ = r.history(kind)
            np.testing.assert_array_equal(hb[kind][0][off:off + s.n], kr, err_msg=f"{s.name} keys {kind}")
            np.testing.assert_array_equal(hb[kind][1][off:off + s.n], lr, err_msg=f"{s.name} last-seen {kind}")
        off += s.n


def _loads_per_step(x, steps):
    out = []
    for _ in range(steps):
        x.run(1)
        out.append(x.bodies()["loads"].copy())
    return out


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("name,steps", [("small_mbd", 25), ("c1", 6)])
def test_cap_knife_edge_is_the_reference_model_s_own(name, steps):
    """Where particle-triangle manifolds slide at their Coulomb cap, the
    reference's body loads jump with the last bit of its inputs: the
    per-triangle pass re-tests the capped history against a limit equal to
    it up to rounding (src/cuda/cuda_contact_backend.cu:783-807 after
    :922-947), and the body loads it sums with atomicAdd change in their last
    bits with the order the atomics land in.  The reference's own spread --
    the reference run again, and the reference with one input moved by one
    ulp (the plate's initial height on the small scene, the blade's spin on
    config 1) -- reaches 1e-3 of the loads within the window, and the FP64
    engine's departure from the reference stays within three times that
    spread."""
    if name == "small_mbd":
        sc = G.small_mbd()
        ulp = sc.copy()
        ulp.body_center[0, 2] = np.nextafter(ulp.body_center[0, 2], np.inf)
    else:
        sc = _config_scene("c1")
        ulp = sc.copy()
        ulp.body_omega[0, 2] = np.nextafter(ulp.body_omega[0, 2], np.inf)
    ref = _loads_per_step(ref_cuda.RefCuda(sc), steps)
    again = _loads_per_step(ref_cuda.RefCuda(sc), steps)
    moved = _loads_per_step(ref_cuda.RefCuda(ulp), steps)
    eng = _loads_per_step(engine_for(sc), steps)
    rerun = max(_rel(a, r) for a, r in zip(again, ref))
    one_ulp = max(_rel(m, r) for m, r in zip(moved, ref))
    departure = max(_rel(x, r) for x, r in zip(eng, ref))
    print(f"{name}: reference rerun {rerun:.3g}, reference one ulp {one_ulp:.3g}, engine {departure:.3g}")
    envelope = max(rerun, one_ulp)
    assert envelope >= 1e-3, envelope
    assert departure <= 3 * envelope, (departure, envelope)
