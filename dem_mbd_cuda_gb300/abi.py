"""ctypes mirrors of the plain structs in include/dem_gb300.h."""
from __future__ import annotations

import ctypes as C

from .scene import CMech, CScene  # noqa: F401  (re-exported)

DEM_OK = 0
DEM_PRECISION_FP64 = 0
DEM_PRECISION_MIXED = 1


class COptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("cell_factor", C.c_double), ("max_cells", C.c_int), ("block_size", C.c_int),
                ("pt_fp32", C.c_int)]


class CBodyStates(C.Structure):
    _fields_ = [("center", C.c_void_p), ("quat", C.c_void_p), ("vel", C.c_void_p), ("omega", C.c_void_p)]


class CStepStats(C.Structure):
    _fields_ = [
        ("particle_contacts", C.c_int), ("body_contacts", C.c_int), ("body_max_depth", C.c_double),
        ("body_contact_fz", C.c_double), ("particle_history_overflows", C.c_int),
        ("body_history_overflows", C.c_int), ("particle_history_high_water", C.c_int),
        ("body_history_high_water", C.c_int), ("triangle_grid_overflows", C.c_int),
        ("cell_table_overflows", C.c_int), ("body_regime_interval_native_steps", C.c_uint64),
        ("body_candidate_items", C.c_int), ("wall_candidates", C.c_int),
    ]

    def to_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}
