"""Helpers shared by the GPU parity tests."""
import numpy as np

from dem_mbd_cuda_gb300.engine import CudaDemSolver
from oracle.oracle import Oracle


def engine_for(scene, precision="fp64", **kw):
    e = CudaDemSolver()
    e.initialize(scene, precision=precision, **kw)
    return e


def close(a, b, atol=1e-8, rtol=1e-9, what=""):
    """The reference's own comparison bar, abs <= 1e-8 + 1e-9 |ref|
    (docs/CUDA_MIGRATION_VALIDATION.md:73)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    err = np.abs(a - b) - (atol + rtol * np.abs(b))
    assert np.all(err <= 0), f"{what}: max violation {err.max():.3e}, max abs diff {np.abs(a - b).max():.3e}"


def active_contacts(keys, last, step):
    """Set of (component, key) with last-seen == step: the contact list."""
    c, s = np.nonzero((keys != 0) & (last == step))
    return set(zip(c.tolist(), keys[c, s].tolist()))


def forces_of(x):
    """Force output of the engine, the oracle or the reference's CUDA engine."""
    return x.downloadForceOutput() if isinstance(x, CudaDemSolver) else x.forces()


def stats_of(x):
    return x.stepStats() if isinstance(x, CudaDemSolver) else x.stats()


def state_of(x):
    return x.downloadParticleState() if isinstance(x, CudaDemSolver) else x.state()


def compare_evaluation(e, o, step=None, tol=1e-9):
    """Bit-exact grid and history slots, tolerance on forces and values.
    `o` is the checker (oracle or the reference's CUDA engine); `e` is the
    run under test (engine, oracle or reference)."""
    ke, ie = e.grid()
    ko, io = o.grid()
    np.testing.assert_array_equal(ie, io)
    np.testing.assert_array_equal(ke, ko)
    for kind in (0, 1, 2):
        k1, l1, v1 = e.history(kind)
        k2, l2, v2 = o.history(kind)
        np.testing.assert_array_equal(k1, k2, err_msg=f"history keys kind {kind}")
        np.testing.assert_array_equal(l1, l2, err_msg=f"history last-seen kind {kind}")
        scale = max(np.abs(v2).max(), 1e-30)
        assert np.abs(v1 - v2).max() <= tol * scale + 1e-15, f"history values kind {kind}"
    fe, fo = forces_of(e), forces_of(o)
    for name in ("contact", "field", "wall", "total"):
        scale = max(np.abs(fo[name]).max(), 1e-30)
        assert np.abs(fe[name] - fo[name]).max() <= tol * scale + 1e-14, name
    se, so = stats_of(e), stats_of(o)
    for key in ("particle_contacts", "body_contacts", "particle_history_high_water", "body_history_high_water",
                "particle_history_overflows", "body_history_overflows"):
        assert se[key] == so[key], (key, se[key], so[key])
