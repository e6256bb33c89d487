"""Reverse-mode gradients of the FP64 step (dem_adjoint_forward / _backward)
against FP64 central differences of the engine's own forward run.

Loss L = mean particle height + 0.1 * mean x velocity after the run, on a few
hundred spheres with random velocities, spins and orientations in a walled
box (all three history channels active, contacts at their caps).  Gradients
with respect to the six materials of each contact class and to the initial
velocities (random directions) must match central differences with a
relative step of 1e-6 (1e-10 m for positions) to 1e-4 relative.
"""
import dataclasses

import numpy as np
import pytest

from gpu_helpers import engine_for
from dem_mbd_cuda_gb300 import generate as G

pytestmark = pytest.mark.gpu

STEPS, K = 30, 10
CV = 0.1  # weight of the mean x velocity in the loss


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def _scene():
    sc = G.small_dem(n=300, seed=11, vel_std=0.05)
    m = sc.pp
    # separate material objects per class so each can be perturbed alone
    return dataclasses.replace(sc, pp=dataclasses.replace(m), pw=dataclasses.replace(m), pt=dataclasses.replace(m))


def _loss(sc):
    e = engine_for(sc, precision="fp64")
    e.run(STEPS)
    st = e.downloadParticleState()
    return st["pos"][:, 2].mean() + CV * st["vel"][:, 0].mean()


def _adjoint(sc, fp32=False):
    e = engine_for(sc, precision="fp64").set_adjoint_fp32(fp32).adjoint_forward(STEPS, K)
    n = e.n
    dpos = np.zeros((n, 3)); dpos[:, 2] = 1.0 / n
    dvel = np.zeros((n, 3)); dvel[:, 0] = CV / n
    return e, e.adjoint_backward(dpos, dvel)


def _close(an, fd, what, scale):
    assert abs(an - fd) <= 1e-4 * max(abs(fd), abs(an)) + 1e-6 * scale, f"{what}: adjoint {an!r} vs fd {fd!r}"


def test_adjoint_forward_matches_plain_run():
    sc = _scene()
    e, _ = _adjoint(sc)
    st = e.downloadParticleState()
    ref = engine_for(sc, precision="fp64")
    ref.run(STEPS)
    rs = ref.downloadParticleState()
    for k in ("pos", "vel", "omega", "quat"):
        np.testing.assert_array_equal(st[k], rs[k], err_msg=k)


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("cls", ["pp", "pw"])
def test_material_gradients_match_central_differences(cls, fp32):
    """Both forms of the reverse law (FP64, and FP32 for the particle and
    wall contacts) against central differences of the FP64 forward run."""
    sc = _scene()
    _, g = _adjoint(sc, fp32)
    grads = g["dl_dparams"][cls]
    scale = max(abs(v) * abs(getattr(getattr(sc, cls), k)) for k, v in grads.items() if k != "epsS")
    for key, field in (("kN", "kN"), ("mu", "mu"), ("epsN", "epsN"), ("epsS", "epsS"), ("muT", "muT"), ("muR", "muR")):
        m = getattr(sc, cls)
        x0 = getattr(m, field)
        h = 1e-6 * abs(x0)
        lp = _loss(dataclasses.replace(sc, **{cls: dataclasses.replace(m, **{field: x0 + h})}))
        lm = _loss(dataclasses.replace(sc, **{cls: dataclasses.replace(m, **{field: x0 - h})}))
        fd = (lp - lm) / (2 * h)
        _close(grads[key] * x0, fd * x0, f"{cls}.{key}", scale)


@pytest.mark.parametrize("fp32", [False, True])
def test_initial_velocity_gradient_matches_central_differences(fp32):
    sc = _scene()
    _, g = _adjoint(sc, fp32)
    rng = np.random.default_rng(5)
    for trial in range(3):
        d = rng.normal(size=sc.vel.shape)
        an = float((g["dl_dvel0"] * d).sum())
        eps = 1e-6 * np.abs(sc.vel).max()
        lp = _loss(dataclasses.replace(sc, vel=sc.vel + eps * d))
        lm = _loss(dataclasses.replace(sc, vel=sc.vel - eps * d))
        _close(an, (lp - lm) / (2 * eps), f"v0 direction {trial}", abs(an))


def test_initial_position_and_spin_gradients_match_central_differences():
    sc = _scene()
    _, g = _adjoint(sc)
    rng = np.random.default_rng(6)
    d = rng.normal(size=sc.pos.shape)
    an = float((g["dl_dpos0"] * d).sum())
    # overlaps are micrometres and contacts near their caps change branch
    # within a nanometre: the position step has to be smaller than that
    eps = 1e-10
    lp = _loss(dataclasses.replace(sc, pos=sc.pos + eps * d))
    lm = _loss(dataclasses.replace(sc, pos=sc.pos - eps * d))
    _close(an, (lp - lm) / (2 * eps), "x0 direction", abs(an))
    d = rng.normal(size=sc.omega.shape)
    an = float((g["dl_domega0"] * d).sum())
    eps = 1e-6 * np.abs(sc.omega).max()
    lp = _loss(dataclasses.replace(sc, omega=sc.omega + eps * d))
    lm = _loss(dataclasses.replace(sc, omega=sc.omega - eps * d))
    _close(an, (lp - lm) / (2 * eps), "w0 direction", abs(an))


def test_fp32_reverse_stays_close_to_the_fp64_reverse():
    """The FP32 reverse law of the particle and wall contacts changes every
    gradient by less than 1e-5 of its size (material gradients, and the
    initial positions', velocities' and spins' gradients measured on their
    largest entry)."""
    sc = _scene()
    _, g64 = _adjoint(sc)
    _, g32 = _adjoint(sc, True)
    for cls in ("pp", "pw"):
        for key, a in g64["dl_dparams"][cls].items():
            b = g32["dl_dparams"][cls][key]
            assert abs(b - a) <= 1e-5 * abs(a) + 1e-12, (cls, key, a, b)
    for name in ("dl_dpos0", "dl_dvel0", "dl_domega0"):
        ref = g64[name]
        assert np.abs(g32[name] - ref).max() <= 1e-5 * np.abs(ref).max(), name


def _batch_scenes():
    """Three walled boxes of spheres (the same box, so their coordinates
    overlap) with their own materials and particle counts: a batch of the
    calibration workload's kind."""
    out = []
    for k, (n, mu, eps) in enumerate(((300, 0.4, 0.5), (200, 0.7, 0.3), (250, 0.2, 0.8))):
        sc = G.small_dem(n=n, seed=21 + k, vel_std=0.05)
        pp = dataclasses.replace(sc.pp, mu=mu, epsN=eps)
        pw = dataclasses.replace(sc.pp, mu=0.5 * mu, epsN=eps)
        out.append(dataclasses.replace(sc, pp=pp, pw=pw, pt=dataclasses.replace(pp)))
    return out


def test_batched_adjoint_matches_scene_by_scene():
    """One batched reverse sweep of the sum of the scenes' losses gives each
    scene's material and initial-state gradients as its own engine does
    (the scenes are independent; only the order of the atomic sums differs)."""
    scenes = _batch_scenes()
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    b = CudaDemSolver().initialize(scenes, precision="fp64").adjoint_forward(STEPS, K)
    dpos = np.zeros((b.n, 3))
    dvel = np.zeros((b.n, 3))
    off = 0
    for sc in scenes:
        dpos[off:off + sc.n, 2] = 1.0 / sc.n
        dvel[off:off + sc.n, 0] = CV / sc.n
        off += sc.n
    gb = b.adjoint_backward(dpos, dvel)
    assert len(gb["dl_dparams"]) == len(scenes)
    off = 0
    for k, sc in enumerate(scenes):
        _, g = _adjoint(sc)
        for cls in ("pp", "pw"):
            for key, a in g["dl_dparams"][cls].items():
                bk = gb["dl_dparams"][k][cls][key]
                assert abs(bk - a) <= 1e-9 * abs(a) + 1e-15, (k, cls, key, bk, a)
        for name in ("dl_dpos0", "dl_dvel0", "dl_domega0"):
            ref = g[name]
            got = gb[name][off:off + sc.n]
            assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max() + 1e-18, (k, name)
        off += sc.n


def test_batched_adjoint_with_a_rigid_body():
    """A batch of a walled box of spheres and the plate scene: the batched
    sweep gives each scene its own sweep's gradients, the plate's included
    (the body records and the manifold tapes are per body of the batch)."""
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    a = G.small_dem(n=200, seed=31, vel_std=0.05)
    scenes = [a, dataclasses.replace(_mbd_scene(), dt=a.dt)]
    b = CudaDemSolver().initialize(scenes, precision="fp64").adjoint_forward(STEPS, K)
    dpos = np.zeros((b.n, 3))
    off = 0
    for sc in scenes:
        dpos[off:off + sc.n, 2] = 1.0 / sc.n
        off += sc.n
    gb = b.adjoint_backward(dpos, None, dl_dbody_center=np.full((1, 3), CB))
    off = 0
    for k, sc in enumerate(scenes):
        e = engine_for(sc, precision="fp64").adjoint_forward(STEPS, K)
        d = np.zeros((sc.n, 3)); d[:, 2] = 1.0 / sc.n
        g = e.adjoint_backward(d, None, dl_dbody_center=np.full((1, 3), CB) if sc.n_bodies else None)
        for cls in ("pp", "pw", "pt"):
            for key, v in g["dl_dparams"][cls].items():
                bk = gb["dl_dparams"][k][cls][key]
                assert abs(bk - v) <= 1e-9 * abs(v) + 1e-15, (k, cls, key, bk, v)
        ref = g["dl_dvel0"]
        assert np.abs(gb["dl_dvel0"][off:off + sc.n] - ref).max() <= 1e-9 * np.abs(ref).max() + 1e-18
        off += sc.n


def test_batched_autograd_gradients():
    """simulate_batch returns per-scene material gradients equal to the
    engine's batched backward result."""
    torch = pytest.importorskip("torch")
    from dem_mbd_cuda_gb300.autograd import materials, simulate_batch
    scenes = _batch_scenes()
    pp = torch.stack([materials(s.pp) for s in scenes]).requires_grad_(True)
    pw = torch.stack([materials(s.pw) for s in scenes])
    v0 = torch.tensor(np.concatenate([s.vel for s in scenes]))
    pos, _ = simulate_batch(scenes, STEPS, pp, pw, v0, checkpoint_every=K)
    off, loss = 0, 0.0
    for s in scenes:
        loss = loss + pos[off:off + s.n, 2].mean()
        off += s.n
    loss.backward()
    assert pp.grad.shape == (len(scenes), 6)
    for k, s in enumerate(scenes):
        e = engine_for(s, precision="fp64").adjoint_forward(STEPS, K)
        dpos = np.zeros((s.n, 3)); dpos[:, 2] = 1.0 / s.n
        g = e.adjoint_backward(dpos, None)["dl_dparams"]["pp"]
        for f, key in enumerate(("kN", "mu", "epsN", "epsS", "muT", "muR")):
            assert abs(pp.grad[k, f].item() - g[key]) <= 1e-9 * abs(g[key]) + 1e-15, (k, key)


def test_anisotropic_inertia_gradients_match_central_differences():
    """Owners with three different principal inertias (Euler's equations with
    their gyroscopic terms): material gradients and random directions of the
    initial spins against central differences."""
    base = _scene()
    sc = dataclasses.replace(base, owner_inertia=base.owner_inertia * np.array([1.0, 1.35, 0.75]))
    _, g = _adjoint(sc)
    grads = g["dl_dparams"]["pp"]
    scale = max(abs(grads[k]) * abs(getattr(sc.pp, k)) for k in ("kN", "mu", "epsN"))
    for key in ("kN", "mu", "epsN", "muR"):
        x0 = getattr(sc.pp, key)
        h = 1e-6 * abs(x0)
        lp = _loss(dataclasses.replace(sc, pp=dataclasses.replace(sc.pp, **{key: x0 + h})))
        lm = _loss(dataclasses.replace(sc, pp=dataclasses.replace(sc.pp, **{key: x0 - h})))
        _close(grads[key] * x0, (lp - lm) / (2 * h) * x0, f"pp.{key}", scale)
    rng = np.random.default_rng(9)
    for trial in range(2):
        d = rng.normal(size=sc.omega.shape)
        an = float((g["dl_domega0"] * d).sum())
        eps = 1e-6 * np.abs(sc.omega).max()
        lp = _loss(dataclasses.replace(sc, omega=sc.omega + eps * d))
        lm = _loss(dataclasses.replace(sc, omega=sc.omega - eps * d))
        _close(an, (lp - lm) / (2 * eps), f"w0 direction {trial}", abs(an))


def test_adjoint_scope_errors():
    sc = _scene()
    e = engine_for(sc, precision="mixed")
    with pytest.raises(RuntimeError, match="FP64"):
        e.adjoint_forward(5, 5)


# ---- rigid bodies: a dynamic plate resting on a layer of spheres
CB = 0.5   # weight of the sum of the plate's final centre coordinates in the loss


def _mbd_scene():
    sc = G.plate_on_monolayer()
    return dataclasses.replace(sc, pp=dataclasses.replace(sc.pp), pw=dataclasses.replace(sc.pw),
                               pt=dataclasses.replace(sc.pt))


def _mbd_loss(sc):
    e = engine_for(sc, precision="fp64")
    e.run(STEPS)
    st = e.downloadParticleState()
    return st["pos"][:, 2].mean() + CV * st["vel"][:, 0].mean() + CB * float(e.bodies()["center"][0].sum())


def _mbd_adjoint(sc):
    e = engine_for(sc, precision="fp64").adjoint_forward(STEPS, K)
    n = e.n
    dpos = np.zeros((n, 3)); dpos[:, 2] = 1.0 / n
    dvel = np.zeros((n, 3)); dvel[:, 0] = CV / n
    return e, e.adjoint_backward(dpos, dvel, dl_dbody_center=np.full((1, 3), CB))


def test_rigid_body_forward_and_restore():
    """The checkpointed forward run equals a plain run (particles and the
    plate), and the backward run leaves the engine at its end."""
    sc = _mbd_scene()
    e, _ = _mbd_adjoint(sc)
    ref = engine_for(sc, precision="fp64")
    ref.run(STEPS)
    st, rs = e.downloadParticleState(), ref.downloadParticleState()
    for k in ("pos", "vel", "omega", "quat"):
        np.testing.assert_array_equal(st[k], rs[k], err_msg=k)
    np.testing.assert_array_equal(e.bodies()["center"], ref.bodies()["center"])
    e.run(3)
    ref.run(3)
    np.testing.assert_array_equal(e.downloadParticleState()["pos"], ref.downloadParticleState()["pos"])
    np.testing.assert_array_equal(e.bodies()["center"], ref.bodies()["center"])


@pytest.mark.parametrize("cls,keys", [("pt", ("kN", "epsN", "epsS")), ("pw", ("kN", "mu", "epsN"))])
def test_rigid_body_material_gradients_match_central_differences(cls, keys):
    """The loss includes the plate's final centre: gradients reach the
    particle-triangle materials through the plate's dynamics and the
    spheres under it."""
    sc = _mbd_scene()
    _, g = _mbd_adjoint(sc)
    grads = g["dl_dparams"][cls]
    scale = max(abs(grads[k]) * abs(getattr(getattr(sc, cls), k)) for k in keys)
    assert scale > 0
    for key in keys:
        m = getattr(sc, cls)
        x0 = getattr(m, key)
        h = 1e-6 * abs(x0)
        lp = _mbd_loss(dataclasses.replace(sc, **{cls: dataclasses.replace(m, **{key: x0 + h})}))
        lm = _mbd_loss(dataclasses.replace(sc, **{cls: dataclasses.replace(m, **{key: x0 - h})}))
        _close(grads[key] * x0, (lp - lm) / (2 * h) * x0, f"{cls}.{key}", scale)


def test_rigid_body_initial_state_gradients_match_central_differences():
    """dem_adjoint_body_gradients: the loss's gradient with respect to the
    dynamic plate's initial centre, velocity and body-frame spin (random
    directions) against central differences of the FP64 forward run."""
    sc = _mbd_scene()
    _, g = _mbd_adjoint(sc)
    assert g["dl_dbody_quat0"].shape == (1, 4)
    rng = np.random.default_rng(9)
    for name, field, eps in (("dl_dbody_center0", "body_center", 1e-10), ("dl_dbody_vel0", "body_vel", 1e-7),
                             ("dl_dbody_omega0", "body_omega", 1e-6)):
        d = rng.normal(size=getattr(sc, field).shape)
        an = float((g[name] * d).sum())
        lp = _mbd_loss(dataclasses.replace(sc, **{field: getattr(sc, field) + eps * d}))
        lm = _mbd_loss(dataclasses.replace(sc, **{field: getattr(sc, field) - eps * d}))
        _close(an, (lp - lm) / (2 * eps), name, abs(an))


def test_rigid_body_initial_velocity_gradient_matches_central_differences():
    sc = _mbd_scene()
    _, g = _mbd_adjoint(sc)
    rng = np.random.default_rng(8)
    for trial in range(3):
        d = rng.normal(size=sc.vel.shape)
        an = float((g["dl_dvel0"] * d).sum())
        eps = 1e-6 * np.abs(sc.vel).max()
        lp = _mbd_loss(dataclasses.replace(sc, vel=sc.vel + eps * d))
        lm = _mbd_loss(dataclasses.replace(sc, vel=sc.vel - eps * d))
        _close(an, (lp - lm) / (2 * eps), f"v0 direction {trial}", abs(an))


def test_autograd_function_and_calibration_step():
    """The torch.autograd.Function returns the engine's gradients, and one
    gradient step on the restitution reduces a calibration loss (final mean
    height against a target made with another restitution)."""
    torch = pytest.importorskip("torch")
    from dem_mbd_cuda_gb300.autograd import materials, simulate
    sc = _scene()
    pw = materials(sc.pw)
    v0 = torch.tensor(sc.vel)
    target_pp = materials(sc.pp)
    target_pp[2] = 0.6
    with torch.no_grad():
        target = simulate(sc, STEPS, target_pp, pw, v0)[0][:, 2].mean()

    def loss_of(pp):
        pos, _ = simulate(sc, STEPS, pp, pw, v0)
        return (pos[:, 2].mean() - target) ** 2

    pp = materials(sc.pp).requires_grad_(True)
    loss = loss_of(pp)
    loss.backward()
    # the autograd gradient is the engine's backward result
    e = engine_for(sc, precision="fp64").adjoint_forward(STEPS, 100)
    n = e.n
    z = torch.tensor(e.downloadParticleState()["pos"][:, 2]).mean()
    dpos = np.zeros((n, 3)); dpos[:, 2] = float(2.0 * (z - target)) / n
    g = e.adjoint_backward(dpos, None)
    assert pp.grad[2].item() == pytest.approx(g["dl_dparams"]["pp"]["epsN"], rel=1e-12)
    # half a Newton step on L = r^2 (d eps = -L / L') lowers the loss
    with torch.no_grad():
        pp2 = pp.detach().clone()
        pp2[2] -= float(loss.detach()) / pp.grad[2]
    assert float(loss_of(pp2)) < 0.5 * float(loss.detach())
