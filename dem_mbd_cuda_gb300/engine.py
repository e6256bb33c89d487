"""Python mirror of the reference's ``CudaDemSolver`` over the C ABI.

``CudaDemSolver`` keeps the reference's member names and call order
(include/cuda_backend.h:40-72): ``initialize``, ``computeForces``,
``initializeParticleHalfStep``, ``advanceParticles``, ``finishParticleStep``,
``saveContactHistory`` / ``loadContactHistory``, ``downloadParticleState``,
``downloadForceOutput``, ``stepStats``.  Errors raise ``RuntimeError`` with the
library's message, as the reference throws ``std::runtime_error``.  There is
no CPU fallback: without the CUDA library or a device every call fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import CBodyStates, COptions, CStepStats, DEM_PRECISION_FP64, DEM_PRECISION_MIXED  # noqa: F401
from .scene import Scene

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdemgb300.so")

_lib = None

_SIGS = {
    "dem_abi_version": ([], C.c_int),
    "dem_last_error": ([], C.c_char_p),
    "dem_device_available": ([], C.c_int),
    "dem_device_description": ([], C.c_char_p),
    "dem_create": ([C.c_void_p], C.c_int),
    "dem_destroy": ([C.c_void_p], C.c_int),
    "dem_default_options": ([C.c_void_p], None),
    "dem_initialize": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "dem_initialize_batch": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "dem_compute_forces": ([C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int], C.c_int),
    "dem_leapfrog_init": ([C.c_void_p, C.c_double], C.c_int),
    "dem_leapfrog_advance": ([C.c_void_p, C.c_double], C.c_int),
    "dem_leapfrog_finish": ([C.c_void_p, C.c_double, C.c_double], C.c_int),
    "dem_run_steps": ([C.c_void_p, C.c_int], C.c_int),
    "dem_get_bodies": ([C.c_void_p] + [C.c_void_p] * 5, C.c_int),
    "dem_save_history": ([C.c_void_p, C.c_char_p], C.c_int),
    "dem_load_history": ([C.c_void_p, C.c_char_p], C.c_int),
    "dem_has_restored_leapfrog_state": ([C.c_void_p, C.c_void_p], C.c_int),
    "dem_download_state": ([C.c_void_p] + [C.c_void_p] * 4, C.c_int),
    "dem_download_forces": ([C.c_void_p] + [C.c_void_p] * 6, C.c_int),
    "dem_stats": ([C.c_void_p, C.c_void_p], C.c_int),
    "dem_body_diagnostics": ([C.c_void_p] + [C.c_void_p] * 4, C.c_int),
    "dem_grid_entry_counts": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "dem_device_memory_bytes": ([C.c_void_p, C.c_void_p], C.c_int),
    "dem_counts": ([C.c_void_p] + [C.c_void_p] * 5, C.c_int),
    "dem_download_grid": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "dem_download_history": ([C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "dem_last_phase_times": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "dem_cell_sort_static": ([C.c_void_p] * 3 + [C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "dem_x_compute_forces_timed": ([C.c_void_p, C.c_int], C.c_int),
    "dem_x_time_steps": ([C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "dem_x_download_half": ([C.c_void_p] + [C.c_void_p] * 5, C.c_int),
    "dem_x_synchronize": ([C.c_void_p], C.c_int),
    "dem_x_set_pt_warp_items": ([C.c_void_p, C.c_int], C.c_int),
    "dem_x_set_launch": ([C.c_void_p, C.c_int, C.c_int], C.c_int),
    "dem_adjoint_forward": ([C.c_void_p, C.c_int, C.c_int], C.c_int),
    "dem_adjoint_backward": ([C.c_void_p] + [C.c_void_p] * 6, C.c_int),
    "dem_adjoint_backward_mbd": ([C.c_void_p] + [C.c_void_p] * 8, C.c_int),
    "dem_x_neighbor_stats": ([C.c_void_p] + [C.c_void_p] * 4, C.c_int),
    "dem_x_adjoint_bytes": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "dem_x_set_adjoint_fp32": ([C.c_void_p, C.c_int], C.c_int),
    "dem_adjoint_body_gradients": ([C.c_void_p] * 5, C.c_int),
    "dem_x_scan_wait_probe": ([C.c_void_p, C.c_void_p], C.c_int),
}


def load_library(path=LIB_PATH):
    """Load libdemgb300.so (built by ``dem_mbd_cuda_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA engine library missing: {path}; run dem_mbd_cuda_gb300.build.build()")
        lib = C.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def options(precision="fp64", cell_factor=2.5, max_cells=0, block_size=0, pt_fp32=False):
    o = COptions()
    o.pt_fp32 = int(bool(pt_fp32))
    o.precision = DEM_PRECISION_MIXED if precision in ("mixed", "fp32", DEM_PRECISION_MIXED) else DEM_PRECISION_FP64
    o.cell_factor = float(cell_factor)
    o.max_cells = int(max_cells)
    o.block_size = int(block_size)
    return o


class CudaDemSolver:
    """GB300 engine with the reference's CudaDemSolver call surface."""

    def __init__(self):
        self.lib = load_library()
        h = C.c_void_p()
        self._check(self.lib.dem_create(C.byref(h)))
        self.h = h
        self._keep = []
        self.n = self.nc = self.nb = self.nt = self.nw = 0
        self.scenes = 1

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.dem_last_error().decode() or f"dem error {rc}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.dem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ lifecycle
    def initialize(self, scene, opts=None, **kw):
        """CudaDemSolver::initialize; ``scene`` is a Scene or a list (batch)."""
        o = opts if opts is not None else options(**kw)
        if isinstance(scene, (list, tuple)):
            cs = (self._scene_struct() * len(scene))()
            for k, s in enumerate(scene):
                c, keep = s.to_c()
                cs[k] = c
                self._keep.append(keep)
            self._keep.append(cs)
            self._check(self.lib.dem_initialize_batch(self.h, C.cast(cs, C.c_void_p), len(scene), C.byref(o)))
            self.scenes = len(scene)
        else:
            self.scenes = 1
            c, keep = scene.to_c()
            self._keep += [c, keep]
            self._check(self.lib.dem_initialize(self.h, C.byref(c), C.byref(o)))
        vals = [C.c_int() for _ in range(5)]
        self._check(self.lib.dem_counts(self.h, *[C.byref(v) for v in vals]))
        self.n, self.nc, self.nb, self.nt, self.nw = (v.value for v in vals)
        return self

    @staticmethod
    def _scene_struct():
        from .scene import CScene
        return CScene

    def computeForces(self, time=0.0, bodies=None, body_forces=True, collect_diagnostics=False):
        """Returns the [nb, 6] body loads (contact + m g) when requested."""
        bs = None
        if bodies is not None and self.nb > 0:
            arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in bodies]
            self._keep_bs = arrs
            bs = CBodyStates(*[a.ctypes.data for a in arrs])
        out = np.zeros((max(self.nb, 1), 6)) if (body_forces and self.nb > 0) else None
        self._check(self.lib.dem_compute_forces(self.h, float(time), C.byref(bs) if bs is not None else None, _p(out),
                                                int(bool(collect_diagnostics))))
        return None if out is None else out[:self.nb]

    def initializeParticleHalfStep(self, half_dt):
        self._check(self.lib.dem_leapfrog_init(self.h, float(half_dt)))

    def advanceParticles(self, dt):
        self._check(self.lib.dem_leapfrog_advance(self.h, float(dt)))
        return 0.0

    def finishParticleStep(self, dt, half_dt=None):
        self._check(self.lib.dem_leapfrog_finish(self.h, float(dt), float(0.5 * dt if half_dt is None else half_dt)))

    def run(self, steps):
        """Reference integration loop (pure DEM or DEM-MBD) for ``steps`` steps."""
        self._check(self.lib.dem_run_steps(self.h, int(steps)))

    def saveContactHistory(self, path):
        self._check(self.lib.dem_save_history(self.h, os.fsencode(path)))

    def loadContactHistory(self, path):
        self._check(self.lib.dem_load_history(self.h, os.fsencode(path)))

    def hasRestoredParticleLeapfrogState(self):
        r = C.c_int()
        self._check(self.lib.dem_has_restored_leapfrog_state(self.h, C.byref(r)))
        return bool(r.value)

    # -------------------------------------------------------------- outputs
    def downloadParticleState(self):
        n = self.n
        pos, vel, omg, q = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4))
        self._check(self.lib.dem_download_state(self.h, _p(pos), _p(vel), _p(omg), _p(q)))
        return dict(pos=pos, vel=vel, omega=omg, quat=q)

    def downloadHalfState(self):
        n = self.n
        vh, wh, hdq, acc, aacc = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 3))
        self._check(self.lib.dem_x_download_half(self.h, _p(vh), _p(wh), _p(hdq), _p(acc), _p(aacc)))
        return dict(vh=vh, wh=wh, hdq=hdq, acc=acc, aacc=aacc)

    def downloadForceOutput(self, particle_forces=True, body_forces=True):
        n, nb = self.n, self.nb
        c, f, w, t = (np.zeros((n, 6)) for _ in range(4))
        bp = np.zeros((nb, n, 6)) if (nb and particle_forces) else None
        bd = np.zeros((nb, n, 19)) if (nb and body_forces) else None
        self._check(self.lib.dem_download_forces(self.h, _p(c), _p(f), _p(w), _p(t), _p(bp), _p(bd)))
        return dict(contact=c, field=f, wall=w, total=t, body_particle=bp, body_detail=bd)

    def stepStats(self):
        s = CStepStats()
        self._check(self.lib.dem_stats(self.h, C.byref(s)))
        return s.to_dict()

    def bodyDiagnostics(self):
        nb = max(self.nb, 1)
        ri = np.zeros((nb, 7), dtype=np.uint64)
        rv = np.zeros((nb, 7), dtype=np.uint64)
        mi = np.zeros((nb, 22))
        mv = np.zeros((nb, 22))
        self._check(self.lib.dem_body_diagnostics(self.h, _p(ri), _p(rv), _p(mi), _p(mv)))
        k = self.nb
        return dict(regime_instant=ri[:k], regime_interval=rv[:k], micro_instant=mi[:k], micro_interval=mv[:k])

    def bodies(self):
        nb = max(self.nb, 1)
        c, q, v, w, l = np.zeros((nb, 3)), np.zeros((nb, 4)), np.zeros((nb, 3)), np.zeros((nb, 3)), np.zeros((nb, 6))
        self._check(self.lib.dem_get_bodies(self.h, _p(c), _p(q), _p(v), _p(w), _p(l)))
        k = self.nb
        return dict(center=c[:k], quat=q[:k], vel=v[:k], omega=w[:k], loads=l[:k])

    def particleGridEntryCount(self):
        a, b = C.c_size_t(), C.c_size_t()
        self._check(self.lib.dem_grid_entry_counts(self.h, C.byref(a), C.byref(b)))
        return a.value

    def triangleGridEntryCount(self):
        a, b = C.c_size_t(), C.c_size_t()
        self._check(self.lib.dem_grid_entry_counts(self.h, C.byref(a), C.byref(b)))
        return b.value

    def deviceMemoryBytes(self):
        b = C.c_size_t()
        self._check(self.lib.dem_device_memory_bytes(self.h, C.byref(b)))
        return b.value

    # ------------------------------------------------- parity introspection
    def grid(self):
        k = np.zeros(self.nc, dtype=np.uint64)
        i = np.zeros(self.nc, dtype=np.int32)
        self._check(self.lib.dem_download_grid(self.h, _p(k), _p(i)))
        return k, i

    def history(self, kind):
        slots = (64, 16, 64)[kind]
        s = self.nc * slots
        keys = np.zeros(s, dtype=np.uint64)
        last = np.zeros(s, dtype=np.int32)
        val = np.zeros((s, 9))
        self._check(self.lib.dem_download_history(self.h, int(kind), _p(keys), _p(last), _p(val)))
        return keys.reshape(self.nc, slots), last.reshape(self.nc, slots), val.reshape(self.nc, slots, 9)

    def compute_forces_timed(self, diag=False):
        self._check(self.lib.dem_x_compute_forces_timed(self.h, int(diag)))
        ms = (C.c_float * 16)()
        cnt = C.c_int()
        self._check(self.lib.dem_last_phase_times(self.h, ms, 16, C.byref(cnt)))
        return [ms[k] for k in range(cnt.value)]

    def adjoint_forward(self, steps, checkpoint_every=100):
        """The reference's step sequence from a fresh engine (first
        evaluation, leapfrog start, `steps` steps) with checkpoints for the
        reverse sweep (FP64 form, spheres; rigid bodies included)."""
        self._check(self.lib.dem_adjoint_forward(self.h, int(steps), int(checkpoint_every)))
        return self

    def adjoint_backward(self, dl_dpos=None, dl_dvel=None, dl_dbody_center=None, dl_dbody_vel=None):
        """Gradient of a scalar loss given its adjoint w.r.t. the final
        positions / velocities ([n, 3]) and, with rigid bodies, the dynamic
        bodies' final centres / velocities ([nb, 3]).  Returns a dict with
        dl_dpos0, dl_dvel0, dl_domega0 ([n, 3]) and dl_dparams ({"pp", "pw",
        "pt"}: each {kN, mu, epsN, epsS, muT, muR}; for a batch, a list of
        those, one per scene)."""
        n = self.n

        def arr(x, rows):
            return None if x is None else np.ascontiguousarray(x, dtype=np.float64).reshape(rows, 3)
        a, b = arr(dl_dpos, n), arr(dl_dvel, n)
        bc, bv = arr(dl_dbody_center, max(self.nb, 1)), arr(dl_dbody_vel, max(self.nb, 1))
        x0, v0, w0 = (np.zeros((n, 3)) for _ in range(3))
        p = np.zeros(18 * self.scenes)
        opt = [None if x is None else _p(x) for x in (a, b, bc, bv)]
        self._check(self.lib.dem_adjoint_backward_mbd(self.h, *opt, _p(x0), _p(v0), _p(w0), _p(p)))
        keys = ("kN", "mu", "epsN", "epsS", "muT", "muR")
        per = [{"pp": dict(zip(keys, q[:6])), "pw": dict(zip(keys, q[6:12])), "pt": dict(zip(keys, q[12:]))}
               for q in p.reshape(self.scenes, 18)]
        out = {"dl_dpos0": x0, "dl_dvel0": v0, "dl_domega0": w0,
               "dl_dparams": per[0] if self.scenes == 1 else per}
        if self.nb > 0:
            nb = self.nb
            bc, bq, bv, bw = np.zeros((nb, 3)), np.zeros((nb, 4)), np.zeros((nb, 3)), np.zeros((nb, 3))
            self._check(self.lib.dem_adjoint_body_gradients(self.h, _p(bc), _p(bq), _p(bv), _p(bw)))
            out.update(dl_dbody_center0=bc, dl_dbody_quat0=bq, dl_dbody_vel0=bv, dl_dbody_omega0=bw)
        return out

    def set_pt_warp_items(self, n):
        """Crossover of the two particle-triangle kernels: up to n contact
        items one warp per item, above one thread per item (tests force
        either path with 1 << 30 or -1)."""
        self._check(self.lib.dem_x_set_pt_warp_items(self.h, int(n)))
        return self

    def set_sweep_blocks(self, blocks_per_sm):
        """Blocks per SM of the particle sweep (grid-stride); 0 launches one
        thread per component.  Changes only the speed."""
        self._check(self.lib.dem_x_set_launch(self.h, 0, int(blocks_per_sm)))
        return self

    def set_gather_blocks(self, blocks_per_sm):
        """Blocks of 256 per SM of the record gathers.  Changes only the speed."""
        self._check(self.lib.dem_x_set_launch(self.h, 1, int(blocks_per_sm)))
        return self

    def set_neighbor_lists(self, on, skin_permille=None):
        """Sweep particle pairs from per-component neighbour lists (rebuilt by
        the cell sweep when a component has moved half the skin) instead of
        the 27 cells every step.  skin_permille: the skin as a share of the
        room the cell edge leaves beyond the largest pair (default 500).
        Changes only the speed."""
        if skin_permille is not None:
            self._check(self.lib.dem_x_set_launch(self.h, 4, int(skin_permille)))
        self._check(self.lib.dem_x_set_launch(self.h, 3, 1 if on else 0))
        return self

    def scan_wait_probe(self):
        """Run out the single-pass scans' bounded wait on purpose (a tile
        that never publishes) and return the error word it sets."""
        v = C.c_uint()
        self._check(self.lib.dem_x_scan_wait_probe(self.h, C.byref(v)))
        return v.value

    def neighbor_stats(self):
        """Neighbour-list builds so far, the mean and longest list, and
        whether the last build overflowed a list (those steps sweep the
        cells)."""
        b, m, x, o = C.c_int(), C.c_double(), C.c_int(), C.c_int()
        self._check(self.lib.dem_x_neighbor_stats(self.h, C.byref(b), C.byref(m), C.byref(x), C.byref(o)))
        return {"builds": b.value, "mean_length": m.value, "max_length": x.value, "overflowed": bool(o.value)}

    def set_adjoint_fp32(self, on=True):
        """Run the reverse law of the particle and wall contacts in FP32 (the
        forward run, its recompute and the rest of the reverse sweep stay
        FP64); its gradients carry FP32 rounding, stated against the FP64
        reverse by the tests and the bench."""
        self._check(self.lib.dem_x_set_adjoint_fp32(self.h, 1 if on else 0))
        return self

    def adjoint_memory(self):
        """Device bytes of the reverse mode's checkpoints (occupied history
        prefixes only) and of its two segment tapes."""
        a, b = C.c_size_t(), C.c_size_t()
        self._check(self.lib.dem_x_adjoint_bytes(self.h, C.byref(a), C.byref(b)))
        return {"checkpoint_bytes": a.value, "tape_bytes": b.value}

    def set_pp_blocks(self, blocks_per_sm):
        """Blocks of 256 per SM of the particle law (0: 16).  Changes only the speed."""
        self._check(self.lib.dem_x_set_launch(self.h, 2, int(blocks_per_sm)))
        return self

    def time_steps(self, steps):
        ms = C.c_float()
        self._check(self.lib.dem_x_time_steps(self.h, int(steps), C.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check(self.lib.dem_x_synchronize(self.h))


def device_available():
    try:
        return bool(load_library().dem_device_available())
    except Exception:
        return False
