"""dem_cell_sort_static: the cell sort for callers that cannot allocate
device memory at the call site (memory owned by another pool or arena,
allocation-free loops, an exhausted quota).  Its working memory is a
built-in device array, so two calls in a row reuse (and must clear) the
previous call's contents.  Both calls are checked against the engine's own
sort (dem_compute_forces + dem_download_grid) on the same positions.

The test allocates the caller's buffers with torch; the entry point itself
allocates nothing."""
import ctypes as C

import numpy as np
import pytest

from dem_mbd_cuda_gb300 import generate as G
from dem_mbd_cuda_gb300.engine import CudaDemSolver

pytestmark = pytest.mark.gpu


def engine_sort(scene):
    e = CudaDemSolver().initialize(scene)
    e.computeForces(0.0, None, False, False)
    return e.grid()


def static_sort(lib, torch, pos, mesh):
    n = len(pos)
    dev = torch.device("cuda:0")
    x = torch.tensor(np.ascontiguousarray(pos[:, 0]), dtype=torch.float64, device=dev)
    y = torch.tensor(np.ascontiguousarray(pos[:, 1]), dtype=torch.float64, device=dev)
    z = torch.tensor(np.ascontiguousarray(pos[:, 2]), dtype=torch.float64, device=dev)
    keys = torch.zeros(n, dtype=torch.int64, device=dev)
    ids = torch.zeros(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = lib.dem_cell_sort_static(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()), n,
                                  float(mesh), C.c_void_p(keys.data_ptr()), C.c_void_p(ids.data_ptr()), None)
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
