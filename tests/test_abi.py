"""The C-ABI library builds for sm_103a, loads and exports every entry point
declared in include/dem_gb300.h (no compute calls: no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np

from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "dem_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dem_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_reference_surface():
    names = declared_functions()
    for required in ("dem_create", "dem_destroy", "dem_initialize", "dem_compute_forces", "dem_leapfrog_init",
                     "dem_leapfrog_advance", "dem_leapfrog_finish", "dem_save_history", "dem_load_history",
                     "dem_download_state", "dem_download_forces", "dem_stats", "dem_device_available",
                     "dem_device_description", "dem_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(engine_lib):
    missing = [n for n in declared_functions() if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_abi_version_and_error_path(engine_lib):
    assert engine_lib.dem_abi_version() == 1
    # NULL engine is rejected with a message, no crash, no device work
    rc = engine_lib.dem_compute_forces(None, 0.0, None, None, 0)
    assert rc != 0
    assert b"NULL" in engine_lib.dem_last_error()


def test_struct_layouts_match_header():
    """ctypes mirrors have the C sizes (x86-64 / AArch64 LP64)."""
    from dem_mbd_cuda_gb300.abi import COptions, CStepStats
    from dem_mbd_cuda_gb300.scene import CMech, CScene
    assert C.sizeof(CMech) == 8 * 8
    assert C.sizeof(COptions) == 32
    assert C.sizeof(CStepStats) == 64
    assert C.sizeof(CScene) % 8 == 0


def test_struct_sizes_match_compiled_header(tmp_path):
    """The ctypes mirrors against sizeof() of the header's structs as the C
    compiler lays them out."""
    import shutil
    import subprocess
    from pathlib import Path
    from dem_mbd_cuda_gb300.abi import COptions, CStepStats
    from dem_mbd_cuda_gb300.scene import CMech, CScene
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = Path(__file__).resolve().parents[1] / "include"
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "dem_gb300.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu\\n", sizeof(dem_mech), sizeof(dem_options),'
                   ' sizeof(dem_step_stats), sizeof(dem_scene));return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == [C.sizeof(CMech), C.sizeof(COptions), C.sizeof(CStepStats), C.sizeof(CScene)]


def test_scene_struct_roundtrip():
    from dem_mbd_cuda_gb300 import generate as G
    sc = G.small_mbd(n=50)
    cs, keep = sc.to_c()
    assert cs.n_owners == sc.n and cs.n_triangles == sc.n_triangles and cs.n_bodies == 1
    ids = np.ctypeslib.as_array(C.cast(cs.owner_id, C.POINTER(C.c_int)), shape=(sc.n,))
    np.testing.assert_array_equal(ids, sc.owner_id)
