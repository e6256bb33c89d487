"""Speed settings change no result: the blocks per SM of the sweep, the
gathers and the particle law (grid-stride) leave the trajectory, the bodies
and the contact histories bit-identical;
the autotuner returns a setting the engine accepts."""
import numpy as np
import pytest

from gpu_helpers import engine_for
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
    st0 = ref.downloadParticleState()
    for e in runs[1:]:
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


def test_autotune_returns_an_accepted_setting():
    from dem_mbd_cuda_gb300.autotune import autotune
    sc = G.small_mbd()
    out = autotune(sc, factors=(2.5, 3.0), sweep_blocks=(2, 4), gather_blocks=(1, 8), warp_items=(512,), steps=3,
                   warmup=2)
    assert out["cell_factor"] in (2.5, 3.0)
    assert out["sweep_blocks"] in (None, 2, 4)
    assert out["gather_blocks"] in (None, 1, 8)
    assert out["pt_warp_items"] in (None, 512)
    assert out["ms_per_step"] > 0 and out["default_ms_per_step"] > 0
    assert len(out["table"]) == 2 + 2 + 2 + 1
    e = engine_for(sc, precision="mixed", cell_factor=out["cell_factor"])
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
