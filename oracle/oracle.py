"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (oracle/dem_oracle.c) restates the reference's FP64 DEM step on
the CPU.  Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of bench.py use this module, as the checker; the engine never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "dem_oracle.c")


def build(force=False):
    """Compile the oracle with gcc (no contraction, OpenMP)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC", "-o", LIB, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [P, C.c_int]
        L.orc_destroy.argtypes = [P]
        L.orc_error.restype = C.c_char_p
        L.orc_compute_forces.argtypes = [P, P, P, P, P, P, C.c_int]
        L.orc_leapfrog_init.argtypes = [P, C.c_double]
        L.orc_advance.argtypes = [P, C.c_double]
        L.orc_finish.argtypes = [P, C.c_double]
        L.orc_run.argtypes = [P, C.c_int, C.c_double]
        for name in ("orc_counts", "orc_get_state", "orc_set_state", "orc_get_half", "orc_get_forces",
                     "orc_get_body_result", "orc_get_bodies", "orc_get_grid", "orc_get_triangle_grid",
                     "orc_get_world_triangles", "orc_get_components", "orc_update_components", "orc_set_half",
                     "orc_get_history", "orc_get_stats", "orc_get_regime_state", "orc_body_diagnostics"):
            getattr(L, name).restype = None
        L.orc_get_history.argtypes = [P, C.c_int, P, P, P]
        L.orc_mesh_size.restype = C.c_double
        L.orc_mesh_size.argtypes = [P]
        L.orc_step_index.argtypes = [P]
        L.orc_circle_triangle_area.restype = C.c_double
        L.orc_circle_triangle_area.argtypes = [P, P, P, P, P, C.c_double]
        L.orc_counts.argtypes = [P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Oracle:
    """FP64 CPU restatement of the reference solver (one scene)."""

    def __init__(self, scene, threads=1):
        self.scene = scene
        cs, self._keep = scene.to_c()
        self._cs = cs
        L = lib()
        self.h = L.orc_create(C.byref(cs), int(threads))
        if not self.h:
            raise RuntimeError("oracle: " + L.orc_error().decode())
        counts = np.zeros(6, dtype=np.int32)
        L.orc_counts(C.c_void_p(self.h), _p(counts))
        self.n, self.nc, self.nb, self.nt, self.nw = (int(x) for x in counts[:5])

    def close(self):
        if self.h:
            lib().orc_destroy(C.c_void_p(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle error {rc}: " + lib().orc_error().decode())

    # reference call surface
    def compute_forces(self, bodies=None, diag=True):
        nb = self.nb
        out = np.zeros((max(nb, 1), 6))
        if bodies is not None:
            c, q, v, w = (np.ascontiguousarray(x, dtype=np.float64) for x in bodies)
            self._check(lib().orc_compute_forces(C.c_void_p(self.h), _p(c), _p(q), _p(v), _p(w), _p(out), int(diag)))
        else:
            self._check(lib().orc_compute_forces(C.c_void_p(self.h), None, None, None, None, _p(out), int(diag)))
        return out[:nb]

    def leapfrog_init(self, half_dt):
        self._check(lib().orc_leapfrog_init(C.c_void_p(self.h), half_dt))

    def advance(self, dt):
        self._check(lib().orc_advance(C.c_void_p(self.h), dt))

    def finish(self, dt):
        self._check(lib().orc_finish(C.c_void_p(self.h), dt))

    def run(self, steps, dt=None):
        self._check(lib().orc_run(C.c_void_p(self.h), int(steps), float(self.scene.dt if dt is None else dt)))

    # accessors
    def state(self):
        n = self.n
        pos, vel, omg, q = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4))
        lib().orc_get_state(C.c_void_p(self.h), _p(pos), _p(vel), _p(omg), _p(q))
        return dict(pos=pos, vel=vel, omega=omg, quat=q)

    def half(self):
        n = self.n
        vh, wh, hdq, acc, aacc = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 3))
        lib().orc_get_half(C.c_void_p(self.h), _p(vh), _p(wh), _p(hdq), _p(acc), _p(aacc))
        return dict(vh=vh, wh=wh, hdq=hdq, acc=acc, aacc=aacc)

    def forces(self):
        n, nb = self.n, self.nb
        c, f, w, t = (np.zeros((n, 6)) for _ in range(4))
        bp = np.zeros((nb, n, 6)) if (nb and self.scene.keep_body_particle) else None
        bd = np.zeros((nb, n, 19)) if (nb and self.scene.keep_body_detail) else None
        lib().orc_get_forces(C.c_void_p(self.h), _p(c), _p(f), _p(w), _p(t), _p(bp), _p(bd))
        return dict(contact=c, field=f, wall=w, total=t, body_particle=bp, body_detail=bd)

    def body_result(self):
        r = np.zeros((max(self.nb, 1), 6))
        lib().orc_get_body_result(C.c_void_p(self.h), _p(r))
        return r[:self.nb]

    def bodies(self):
        nb = max(self.nb, 1)
        c, q, v, w, l = np.zeros((nb, 3)), np.zeros((nb, 4)), np.zeros((nb, 3)), np.zeros((nb, 3)), np.zeros((nb, 6))
        lib().orc_get_bodies(C.c_void_p(self.h), _p(c), _p(q), _p(v), _p(w), _p(l))
        k = self.nb
        return dict(center=c[:k], quat=q[:k], vel=v[:k], omega=w[:k], loads=l[:k])

    def grid(self):
        k = np.zeros(self.nc, dtype=np.uint64)
        i = np.zeros(self.nc, dtype=np.int32)
        lib().orc_get_grid(C.c_void_p(self.h), _p(k), _p(i))
        return k, i

    def triangle_grid(self):
        counts = np.zeros(6, dtype=np.int32)
        lib().orc_counts(C.c_void_p(self.h), _p(counts))
        e = int(counts[5])
        k = np.zeros(max(e, 1), dtype=np.uint64)
        i = np.zeros(max(e, 1), dtype=np.int32)
        lib().orc_get_triangle_grid(C.c_void_p(self.h), _p(k), _p(i))
        return k[:e], i[:e]

    def world_triangles(self):
        tw = np.zeros((max(self.nt, 1), 15))
        ab = np.zeros((max(self.nt, 1), 6))
        lib().orc_get_world_triangles(C.c_void_p(self.h), _p(tw), _p(ab))
        return tw[:self.nt], ab[:self.nt]

    def components(self):
        nc = self.nc
        a = [np.zeros((nc, 3)) for _ in range(4)]
        lib().orc_get_components(C.c_void_p(self.h), *[_p(x) for x in a])
        return dict(pos=a[0], vel=a[1], vh=a[2], offset=a[3])

    def history(self, kind):
        slots = (64, 16, 64)[kind]
        s = self.nc * slots
        keys = np.zeros(s, dtype=np.uint64)
        last = np.zeros(s, dtype=np.int32)
        val = np.zeros((s, 9))
        lib().orc_get_history(C.c_void_p(self.h), kind, _p(keys), _p(last), _p(val))
        return keys.reshape(self.nc, slots), last.reshape(self.nc, slots), val.reshape(self.nc, slots, 9)

    def stats(self):
        from dem_mbd_cuda_gb300.abi import CStepStats
        s = CStepStats()
        lib().orc_get_stats(C.c_void_p(self.h), C.byref(s))
        return s.to_dict()

    def body_diagnostics(self):
        nb = max(self.nb, 1)
        ri = np.zeros((nb, 7), dtype=np.uint64)
        rv = np.zeros((nb, 7), dtype=np.uint64)
        mi = np.zeros((nb, 22))
        mv = np.zeros((nb, 22))
        lib().orc_body_diagnostics(C.c_void_p(self.h), _p(ri), _p(rv), _p(mi), _p(mv))
        k = self.nb
        return dict(regime_instant=ri[:k], regime_interval=rv[:k], micro_instant=mi[:k], micro_interval=mv[:k])

    def mesh_size(self):
        return lib().orc_mesh_size(C.c_void_p(self.h))


def circle_triangle_area(center, normal, a, b, c, radius):
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (center, normal, a, b, c)]
    return lib().orc_circle_triangle_area(*[_p(x) for x in arrs], float(radius))
