"""dem_cell_sort_static: the cell sort for callers that cannot allocate
device memory at the call site (memory owned by another pool or arena,
allocation-free loops, an exhausted quota).  Its working memory is a
built-in device array, so two calls in a row reuse (and must clear) the
previous call's contents.  Calls are checked against the engine's own sort
(dem_compute_forces + dem_download_grid), the oracle's grid, and a numpy
stable argsort of the reference's packed keys (packCell(floor(p * (1 /
mesh))), src/cuda/cuda_grid_backend.cu:19-71, sorted stably as
thrust::sort_by_key does) -- at the component limit, with a cell box at
the cell limit, across negative cell boundaries, with every component in
one cell, and on two streams ordered by an event.

The test allocates the caller's buffers with torch; the entry point itself
allocates nothing."""
import ctypes as C
import time

import numpy as np
import pytest

from dem_mbd_cuda_gb300 import generate as G
from dem_mbd_cuda_gb300.engine import CudaDemSolver
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

MAX_COMPONENTS = 262144
MAX_CELLS = 1048576


def numpy_sort(pos, mesh):
    """Stable sort of the reference's packed cell keys over input order."""
    c = np.floor(pos * (1.0 / mesh)).astype(np.int64) + (1 << 20)
    m = (1 << 21) - 1
    key = ((c[:, 0] & m) << 42) | ((c[:, 1] & m) << 21) | (c[:, 2] & m)
    order = np.argsort(key, kind="stable")
    return key[order].astype(np.uint64), order.astype(np.int32)


def engine_sort(scene):
    e = CudaDemSolver().initialize(scene)
    e.computeForces(0.0, None, False, False)
    return e.grid()


def static_sort(lib, torch, pos, mesh, stream=None):
    n = len(pos)
    dev = torch.device("cuda:0")
    x = torch.tensor(np.ascontiguousarray(pos[:, 0]), dtype=torch.float64, device=dev)
    y = torch.tensor(np.ascontiguousarray(pos[:, 1]), dtype=torch.float64, device=dev)
    z = torch.tensor(np.ascontiguousarray(pos[:, 2]), dtype=torch.float64, device=dev)
    keys = torch.zeros(n, dtype=torch.int64, device=dev)
    ids = torch.zeros(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    handle = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.dem_cell_sort_static(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()), n,
                                  float(mesh), C.c_void_p(keys.data_ptr()), C.c_void_p(ids.data_ptr()), handle)
    assert rc == 0, lib.dem_last_error()
    return keys.cpu().numpy().view(np.uint64), ids.cpu().numpy()


def test_static_sort_matches_engine_sort_twice(engine_lib):
    torch = pytest.importorskip("torch")
    a = G.small_dem(n=500, seed=31)
    b = G.pure_dem(n=3000, seed=32, box=(0.08, 0.08, 0.4))
    for scene in (a, b):
        keys_ref, ids_ref = engine_sort(scene)
        mesh = 2.5 * float(scene.owner_radius.max())
        keys, ids = static_sort(engine_lib, torch, scene.pos, mesh)
        np.testing.assert_array_equal(ids, ids_ref)
        np.testing.assert_array_equal(keys, keys_ref)


def test_static_sort_rejects_oversize(engine_lib):
    n = 262144 + 1
    rc = engine_lib.dem_cell_sort_static(None, None, None, n, 1e-3, None, None, None)
    assert rc != 0
    assert b"262144" in engine_lib.dem_last_error()


def test_static_sort_rejects_a_cell_box_spanning_the_hash_range(engine_lib):
    """Components at both ends of the signed 21-bit cell range on every axis:
    the cell box is 2^21 cells on each side (2^63 in all), which must come
    back as a capacity error, not wrap to an empty box and a silent success."""
    torch = pytest.importorskip("torch")
    lo, hi = -float(1 << 20), float(1 << 20) - 0.5
    pos = np.array([[lo, lo, lo], [hi, hi, hi], [0.25, 0.25, 0.25]])
    dev = torch.device("cuda:0")
    x, y, z = (torch.tensor(pos[:, k].copy(), dtype=torch.float64, device=dev) for k in range(3))
    keys = torch.zeros(3, dtype=torch.int64, device=dev)
    ids = torch.zeros(3, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = engine_lib.dem_cell_sort_static(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()),
                                         3, 1.0, C.c_void_p(keys.data_ptr()), C.c_void_p(ids.data_ptr()), None)
    assert rc == 4, engine_lib.dem_last_error()
    assert b"cell box exceeds" in engine_lib.dem_last_error()


def test_static_sort_matches_the_oracle_grid(engine_lib):
    torch = pytest.importorskip("torch")
    scene = G.small_dem(n=400, seed=33)
    o = Oracle(scene)
    o.compute_forces()
    keys_ref, ids_ref = o.grid()
    keys, ids = static_sort(engine_lib, torch, scene.pos, o.mesh_size())
    np.testing.assert_array_equal(ids, ids_ref)
    np.testing.assert_array_equal(keys, keys_ref)


def test_static_sort_at_the_component_limit(engine_lib):
    """262,144 components (the limit) spread over negative and positive
    cells, many of them exactly on cell faces."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(34)
    mesh = 5e-3
    pos = rng.uniform(-0.2, 0.2, size=(MAX_COMPONENTS, 3))
    on_face = rng.random(MAX_COMPONENTS) < 0.2
    pos[on_face] = np.round(pos[on_face] / mesh) * mesh
    keys, ids = static_sort(engine_lib, torch, pos, mesh)
    k_ref, i_ref = numpy_sort(pos, mesh)
    np.testing.assert_array_equal(ids, i_ref)
    np.testing.assert_array_equal(keys, k_ref)


def test_static_sort_with_the_cell_box_at_the_cell_limit(engine_lib):
    """An occupied cell box of 128 x 128 x 64 = 1,048,576 cells (the limit),
    its corners occupied, with components on both sides of zero."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(35)
    mesh = 1e-3
    lo = np.array([-64, -64, -32])
    ext = np.array([128, 128, 64])
    assert int(np.prod(ext)) == MAX_CELLS
    corners = np.array([[i, j, k] for i in (0, 1) for j in (0, 1) for k in (0, 1)]) * (ext - 1) + lo
    cells = np.concatenate([corners, lo + rng.integers(0, ext, size=(20000, 3))])
    pos = (cells + rng.uniform(0.05, 0.95, size=cells.shape)) * mesh
    keys, ids = static_sort(engine_lib, torch, pos, mesh)
    k_ref, i_ref = numpy_sort(pos, mesh)
    np.testing.assert_array_equal(ids, i_ref)
    np.testing.assert_array_equal(keys, k_ref)


def test_static_sort_with_every_component_in_one_cell(engine_lib):
    """The in-cell order is each member's count of members with a smaller
    index, O(m^2) in a cell of m members: 65,536 components in one cell
    still give the stable order (the time is printed)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(36)
    pos = rng.uniform(0.1, 0.9, size=(65536, 3)) * 1e-2
    t0 = time.perf_counter()
    keys, ids = static_sort(engine_lib, torch, pos, 1e-2)
    print("one cell of 65536 components: %.1f ms" % (1e3 * (time.perf_counter() - t0)))
    np.testing.assert_array_equal(ids, np.arange(65536, dtype=np.int32))
    assert np.all(keys == keys[0])


def test_static_sort_on_two_streams_in_order(engine_lib):
    """Two calls on different streams, the second ordered after the first by
    an event: each gives its own scene's sort (the shared scratch is reused
    in order, not raced)."""
    torch = pytest.importorskip("torch")
    a = G.small_dem(n=300, seed=37)
    b = G.small_dem(n=450, seed=38)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    mesh_a = 2.5 * float(a.owner_radius.max())
    mesh_b = 2.5 * float(b.owner_radius.max())
    ka, ia = static_sort(engine_lib, torch, a.pos, mesh_a, stream=s1)
    ev = torch.cuda.Event()
    ev.record(s1)
    s2.wait_event(ev)
    kb, ib = static_sort(engine_lib, torch, b.pos, mesh_b, stream=s2)
    for (k, i), (pos, mesh) in (((ka, ia), (a.pos, mesh_a)), ((kb, ib), (b.pos, mesh_b))):
        k_ref, i_ref = numpy_sort(pos, mesh)
        np.testing.assert_array_equal(i, i_ref)
        np.testing.assert_array_equal(k, k_ref)
