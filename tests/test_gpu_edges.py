"""Edge cases of the engine against the oracle: particles exactly on cell
boundaries (the keys' floor at both signs), many spheres in one cell, a
scene without walls, a batch of very uneven scenes (one sphere next to
hundreds), and the reference's rejection of an empty scene.  Each case runs
with the neighbour lists on (the default) and off."""
import numpy as np
import pytest

from gpu_helpers import close, compare_evaluation, engine_for
from oracle.oracle import Oracle
from dem_mbd_cuda_gb300 import generate as G
from dem_mbd_cuda_gb300.engine import CudaDemSolver
from dem_mbd_cuda_gb300.scene import Scene

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def _scene(pos, rad, walls=True, vel=None, name="edge"):
    kw = G.make_spheres(np.asarray(pos, float), np.asarray(rad, float), G.DENSITY, vel=vel)
    m = G.mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=0.1, muR=0.05, beta=0.5)
    extra = {}
    if walls:
        wo, wn = G.box_walls([-0.05, -0.05, -0.05], [0.05, 0.05, 0.05])
        extra = dict(wall_origin=wo, wall_normal=wn)
    return Scene(**kw, pp=m, pt=m, pw=m, dt=1e-5, gravity=(0.0, 0.0, -9.81), gravity_enabled=1, name=name, **extra)


def _both(sc, steps, lists):
    e = engine_for(sc, precision="fp64").set_neighbor_lists(lists)
    o = Oracle(sc)
    e.run(steps)
    o.run(steps)
    return e, o


def _boundary_scene():
    """Pairs of touching spheres, the first centre of each exactly on a cell
    corner (multiples of the cell edge, both signs), the second across the
    boundary."""
    r = 2e-3
    mesh = 2.5 * r
    pos = []
    for i in range(-6, 7, 2):
        for j in (-2, 0, 2):
            a = np.array([i * mesh, j * mesh, 0.0])
            pos.append(a)
            pos.append(a + np.array([2 * r - 2e-6, 0.0, 0.0]))
    return _scene(np.array(pos), np.full(len(pos), r), walls=False)


def _dense_scene():
    """A slightly overlapping 4 x 4 x 4 lattice of small spheres (1 um
    overlaps, up to six contacts each) inside one cell of the grid a large,
    distant sphere sets."""
    big, small = 4e-3, 0.6e-3
    pos = [[0.05, 0.05, 0.05]]
    g = np.arange(4) * (2 * small - 1e-6) + 2e-3
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos += np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).tolist()
    rad = [big] + [small] * 64
    return _scene(np.array(pos), np.array(rad), walls=False)


@pytest.mark.parametrize("lists", [True, False])
def test_particles_on_cell_boundaries(lists):
    sc = _boundary_scene()
    e, o = _both(sc, 0, lists)
    assert o.stats()["particle_contacts"] == 2 * 21
    compare_evaluation(e, o, 0)
    e, o = _both(sc, 12, lists)
    compare_evaluation(e, o, 12)


@pytest.mark.parametrize("lists", [True, False])
def test_many_spheres_in_one_cell(lists):
    sc = _dense_scene()
    e, o = _both(sc, 0, lists)
    assert o.stats()["particle_contacts"] == 2 * 3 * 4 * 4 * 3
    compare_evaluation(e, o, 0)
    e, o = _both(sc, 4, lists)
    compare_evaluation(e, o, 4)


@pytest.mark.parametrize("lists", [True, False])
def test_scene_without_walls(lists):
    """Spheres in free flight (no walls, no contacts): the trajectory is the
    leapfrog's, step for step the oracle's."""
    rng = np.random.default_rng(8)
    pos = rng.uniform(-0.02, 0.02, size=(20, 3)) * np.array([1, 1, 1])
    pos[:, 0] = np.arange(20) * 0.006  # 6 mm apart: no contacts
    sc = _scene(pos, np.full(20, 2e-3), walls=False, vel=rng.normal(0, 0.1, size=(20, 3)))
    e, o = _both(sc, 30, lists)
    st = e.downloadParticleState()
    so = o.state()
    close(st["pos"], so["pos"], what="pos")
    close(st["vel"], so["vel"], what="vel")
    assert e.stepStats()["particle_contacts"] == 0


def test_uneven_batch_equals_individual_runs():
    """Scenes of 1, 2 and 500 spheres in one engine: each equals its own run
    bit for bit."""
    one = _scene([[0.0, 0.0, -0.045]], [2e-3])
    two = _scene([[0.0, 0.0, -0.0455], [0.0, 0.0, -0.0415]], [2e-3, 2e-3])
    big = G.small_dem(n=500, seed=4)
    big = Scene(**{**{k: getattr(big, k) for k in big.__dataclass_fields__}, "dt": 1e-5})
    scenes = [one, two, big]
    b = CudaDemSolver().initialize(scenes, precision="fp64")
    b.run(20)
    st = b.downloadParticleState()
    off = 0
    for sc in scenes:
        e = engine_for(sc, precision="fp64")
        e.run(20)
        si = e.downloadParticleState()
        for k in ("pos", "vel", "omega", "quat"):
            np.testing.assert_array_equal(st[k][off:off + sc.n], si[k], err_msg=f"{sc.n} {k}")
        off += sc.n


def test_empty_scene_is_rejected():
    sc = _scene(np.zeros((0, 3)), np.zeros(0))
    with pytest.raises(RuntimeError, match="requires particles"):
        CudaDemSolver().initialize(sc)


def test_scan_wait_runs_out_without_a_fault():
    """Failure detection of the single-pass scans: a look-back whose
    predecessor tile never publishes gives up at its bound, reports
    kErrScanWait (16) through its error word, and the context stays usable
    (the engine steps on)."""
    e = engine_for(G.small_dem(n=200, seed=2), precision="fp64")
    assert e.scan_wait_probe() & 16
    ref = engine_for(G.small_dem(n=200, seed=2), precision="fp64")
    e.run(5)
    ref.run(5)
    np.testing.assert_array_equal(e.downloadParticleState()["pos"], ref.downloadParticleState()["pos"])


@pytest.mark.parametrize("max_cells", [8, 40])
def test_cell_table_capacity_is_reported(max_cells):
    """A particle cell box larger than dem_options.max_cells is the
    reference's capacity error at a diagnostic evaluation.  The scene spans
    4 x 4 x 5 cells: 8 cells fail on the first two extents already, 40 on
    the full product."""
    sc = G.small_dem(n=200, seed=3)
    with pytest.raises(RuntimeError, match="dense cell-table capacity"):
        e = CudaDemSolver().initialize(sc, max_cells=max_cells)
        e.computeForces(0.0, None, False, True)


def test_key_range_is_reported():
    """A sphere beyond the signed 21-bit cell range (2^20 cells of 2.5 r_max,
    about 5.8 km here) is the reference's key-range error at a diagnostic
    evaluation; the other spheres still sort."""
    sc = G.small_dem(n=200, seed=3)
    mesh = 2.5 * float(sc.owner_radius.max())
    assert 1.0e4 / mesh > (1 << 20)
    sc.pos[7] = (1.0e4, 0.0, 0.0)
    with pytest.raises(RuntimeError, match="21-bit hash range"):
        e = CudaDemSolver().initialize(sc)
        e.computeForces(0.0, None, False, True)
