"""The launcher of the reference's own CUDA kernels, without a GPU: it
builds, loads and exports its entry points, finds every kernel it launches in
the reference-built cubin's name table, and its restated argument structures
match the reference's headers field by field (checked where the reference
tree is present)."""
import ctypes as C

import pytest

from oracle import ref_cuda, reference_build

ENTRY_POINTS = ["rfc_error", "rfc_kernel_count", "rfc_kernel_short_name", "rfc_create", "rfc_destroy",
                "rfc_compute_forces", "rfc_leapfrog_init", "rfc_advance", "rfc_finish", "rfc_run", "rfc_time_run",
                "rfc_counts", "rfc_mesh_size", "rfc_get_state", "rfc_get_half", "rfc_get_forces", "rfc_get_grid",
                "rfc_get_triangle_grid", "rfc_get_world_triangles", "rfc_get_components", "rfc_get_history",
                "rfc_get_stats", "rfc_body_diagnostics", "rfc_get_regime_state", "rfc_get_microstate",
                "rfc_get_bodies", "rfc_device_bytes"]


def test_launcher_loads_and_exports_its_entry_points():
    lib = C.CDLL(ref_cuda.build())
    for name in ENTRY_POINTS:
        assert hasattr(lib, name), name
    L = ref_cuda.lib()
    shorts = [L.rfc_kernel_short_name(k).decode() for k in range(L.rfc_kernel_count())]
    assert len(shorts) == 13 and len(set(shorts)) == 13


@pytest.mark.skipif(not ref_cuda.available(), reason="reference device code not built")
def test_every_launched_kernel_is_in_the_reference_cubin():
    names = ref_cuda.kernel_names()
    assert len(names) == 13
    assert any("computeContactsKernel" in n for n in names)


@pytest.mark.skipif(reference_build.reference_root() is None, reason="reference tree not available")
def test_restated_layouts_match_the_reference_headers():
    reference_build.check_layout(reference_build.reference_root())
