"""ctypes binding of the reference's own CUDA engine (TEST INFRASTRUCTURE ONLY).

``RefCuda`` runs the reference's kernels -- device code compiled from the
reference's src/cuda/*.cu into oracle/_ref/ref_engine.cubin by
oracle/reference_build.py -- through oracle/ref_cuda_host.cu, which restates
the reference's host glue (src/cuda_backend_cuda.cu:302-524 and the gpu*
launch wrappers).  It has the accessors of ``oracle.oracle.Oracle``, so the
same comparisons pin the oracle and check the engine against the reference
itself.  Only tests/ and the baseline leg of bench.py use it; the engine
never imports it.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libref_cuda.so")
SRC = os.path.join(HERE, "ref_cuda_host.cu")
DEPS = [SRC, os.path.join(HERE, "ref_cuda_layout.h"), os.path.join(ROOT, "include", "dem_gb300.h")]
CUBIN = os.path.join(HERE, "_ref", "ref_engine.cubin")
KERNELS = os.path.join(HERE, "_ref", "ref_engine_kernels.json")


def available():
    """True when the reference's device code has been built (it is built
    where the reference tree exists and travels with the repository)."""
    return os.path.exists(CUBIN) and os.path.exists(KERNELS)


def build(force=False):
    """Compile the launcher with nvcc (sm_103a, for the Thrust calls it makes)."""
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(p) for p in DEPS):
        return LIB
    cmd = ["nvcc", "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-gencode",
           "arch=compute_103a,code=sm_103a", SRC, "-o", LIB + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for ref_cuda_host.cu:\n" + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.rfc_error.restype = C.c_char_p
        L.rfc_kernel_count.restype = C.c_int
        L.rfc_kernel_short_name.restype = C.c_char_p
        L.rfc_kernel_short_name.argtypes = [C.c_int]
        L.rfc_create.restype = P
        L.rfc_create.argtypes = [C.c_char_p, P, P]
        L.rfc_destroy.argtypes = [P]
        L.rfc_compute_forces.argtypes = [P, P, P, P, P, P, C.c_int]
        L.rfc_leapfrog_init.argtypes = [P, C.c_double]
        L.rfc_advance.argtypes = [P, C.c_double]
        L.rfc_finish.argtypes = [P, C.c_double]
        L.rfc_run.argtypes = [P, C.c_int]
        L.rfc_time_run.argtypes = [P, C.c_int, P]
        L.rfc_counts.argtypes = [P, P]
        L.rfc_mesh_size.restype = C.c_double
        L.rfc_mesh_size.argtypes = [P]
        for name in ("rfc_get_state", "rfc_get_components"):
            getattr(L, name).argtypes = [P, P, P, P, P]
        L.rfc_get_half.argtypes = [P, P, P, P, P, P]
        L.rfc_get_forces.argtypes = [P, P, P, P, P, P, P]
        L.rfc_get_grid.argtypes = [P, P, P]
        L.rfc_get_triangle_grid.argtypes = [P, P, P]
        L.rfc_get_world_triangles.argtypes = [P, P, P]
        L.rfc_get_history.argtypes = [P, C.c_int, P, P, P]
        L.rfc_get_stats.argtypes = [P, P]
        L.rfc_get_stats.restype = None
        L.rfc_body_diagnostics.argtypes = [P, P, P, P, P]
        L.rfc_body_diagnostics.restype = None
        L.rfc_get_regime_state.argtypes = [P, P]
        L.rfc_get_microstate.argtypes = [P, P]
        L.rfc_get_bodies.argtypes = [P, P, P, P, P, P]
        L.rfc_get_bodies.restype = None
        L.rfc_device_bytes.restype = C.c_size_t
        L.rfc_device_bytes.argtypes = [P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def kernel_names():
    """Entry names of the launcher's kernels, in its order."""
    with open(KERNELS) as f:
        table = json.load(f)
    L = lib()
    out = []
    for k in range(L.rfc_kernel_count()):
        short = L.rfc_kernel_short_name(k).decode()
        if short not in table:
            raise RuntimeError("reference cubin lacks " + short)
        out.append(table[short])
    return out


class RefCuda:
    """The reference's FP64 CUDA engine on one scene (the current device)."""

    def __init__(self, scene):
        if not available():
            raise RuntimeError("reference device code not built (oracle/reference_build.py)")
        if scene.n_triangles and np.any(np.diff(np.asarray(scene.tri_body)) < 0):
            raise ValueError("the reference lists triangles body by body; sort the scene's triangles by body")
        self.scene = scene
        cs, self._keep = scene.to_c()
        self._cs = cs
        names = kernel_names()
        self._names = (C.c_char_p * len(names))(*[n.encode() for n in names])
        L = lib()
        self.h = L.rfc_create(CUBIN.encode(), C.cast(self._names, C.c_void_p), C.byref(cs))
        if not self.h:
            raise RuntimeError("reference CUDA engine: " + L.rfc_error().decode())
        counts = np.zeros(6, dtype=np.int32)
        L.rfc_counts(C.c_void_p(self.h), _p(counts))
        self.n, self.nc, self.nb, self.nt, self.nw = (int(x) for x in counts[:5])

    def close(self):
        if getattr(self, "h", None):
            lib().rfc_destroy(C.c_void_p(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"reference CUDA engine error {rc}: " + lib().rfc_error().decode())

    # reference call surface
    def compute_forces(self, bodies=None, diag=True):
        out = np.zeros((max(self.nb, 1), 6))
        if bodies is not None and self.nb:
            c, q, v, w = (np.ascontiguousarray(x, dtype=np.float64) for x in bodies)
            rc = lib().rfc_compute_forces(C.c_void_p(self.h), _p(c), _p(q), _p(v), _p(w), _p(out), int(diag))
        else:
            rc = lib().rfc_compute_forces(C.c_void_p(self.h), None, None, None, None,
                                          _p(out) if self.nb else None, int(diag))
        self._check(rc)
        return out[:self.nb]

    def leapfrog_init(self, half_dt):
        self._check(lib().rfc_leapfrog_init(C.c_void_p(self.h), half_dt))

    def advance(self, dt):
        self._check(lib().rfc_advance(C.c_void_p(self.h), dt))

    def finish(self, dt):
        self._check(lib().rfc_finish(C.c_void_p(self.h), dt))

    def run(self, steps):
        """The reference's step loop with its host MBD step (dt of the scene)."""
        self._check(lib().rfc_run(C.c_void_p(self.h), int(steps)))

    def time_run(self, steps):
        """Seconds of wall clock for `steps` steps of the reference's loop."""
        sec = C.c_double(0.0)
        self._check(lib().rfc_time_run(C.c_void_p(self.h), int(steps), C.byref(sec)))
        return sec.value

    # accessors (as oracle.oracle.Oracle)
    def state(self):
        n = self.n
        pos, vel, omg, q = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4))
        self._check(lib().rfc_get_state(C.c_void_p(self.h), _p(pos), _p(vel), _p(omg), _p(q)))
        return dict(pos=pos, vel=vel, omega=omg, quat=q)

    def half(self):
        n = self.n
        vh, wh, hdq, acc, aacc = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 3))
        self._check(lib().rfc_get_half(C.c_void_p(self.h), _p(vh), _p(wh), _p(hdq), _p(acc), _p(aacc)))
        return dict(vh=vh, wh=wh, hdq=hdq, acc=acc, aacc=aacc)

    def forces(self):
        n, nb = self.n, self.nb
        c, f, w, t = (np.zeros((n, 6)) for _ in range(4))
        bp = np.zeros((nb, n, 6)) if (nb and self.scene.keep_body_particle) else None
        bd = np.zeros((nb, n, 19)) if (nb and self.scene.keep_body_detail) else None
        self._check(lib().rfc_get_forces(C.c_void_p(self.h), _p(c), _p(f), _p(w), _p(t), _p(bp), _p(bd)))
        return dict(contact=c, field=f, wall=w, total=t, body_particle=bp, body_detail=bd)

    def bodies(self):
        nb = max(self.nb, 1)
        c, q, v, w, l = np.zeros((nb, 3)), np.zeros((nb, 4)), np.zeros((nb, 3)), np.zeros((nb, 3)), np.zeros((nb, 6))
        lib().rfc_get_bodies(C.c_void_p(self.h), _p(c), _p(q), _p(v), _p(w), _p(l))
        k = self.nb
        return dict(center=c[:k], quat=q[:k], vel=v[:k], omega=w[:k], loads=l[:k])

    def grid(self):
        k = np.zeros(self.nc, dtype=np.uint64)
        i = np.zeros(self.nc, dtype=np.int32)
        self._check(lib().rfc_get_grid(C.c_void_p(self.h), _p(k), _p(i)))
        return k, i

    def triangle_grid(self):
        counts = np.zeros(6, dtype=np.int32)
        lib().rfc_counts(C.c_void_p(self.h), _p(counts))
        e = int(counts[5])
        k = np.zeros(max(e, 1), dtype=np.uint64)
        i = np.zeros(max(e, 1), dtype=np.int32)
        self._check(lib().rfc_get_triangle_grid(C.c_void_p(self.h), _p(k), _p(i)))
        return k[:e], i[:e]

    def world_triangles(self):
        tw = np.zeros((max(self.nt, 1), 15))
        ab = np.zeros((max(self.nt, 1), 6))
        self._check(lib().rfc_get_world_triangles(C.c_void_p(self.h), _p(tw), _p(ab)))
        return tw[:self.nt], ab[:self.nt]

    def components(self):
        nc = self.nc
        a = [np.zeros((nc, 3)) for _ in range(4)]
        self._check(lib().rfc_get_components(C.c_void_p(self.h), *[_p(x) for x in a]))
        return dict(pos=a[0], vel=a[1], vh=a[2], offset=a[3])

    def history(self, kind):
        slots = (64, 16, 64)[kind]
        s = self.nc * slots
        keys = np.zeros(s, dtype=np.uint64)
        last = np.zeros(s, dtype=np.int32)
        val = np.zeros((s, 9))
        self._check(lib().rfc_get_history(C.c_void_p(self.h), kind, _p(keys), _p(last), _p(val)))
        return keys.reshape(self.nc, slots), last.reshape(self.nc, slots), val.reshape(self.nc, slots, 9)

    def stats(self):
        from dem_mbd_cuda_gb300.abi import CStepStats
        s = CStepStats()
        lib().rfc_get_stats(C.c_void_p(self.h), C.byref(s))
        return s.to_dict()

    def body_diagnostics(self):
        nb = max(self.nb, 1)
        ri = np.zeros((nb, 7), dtype=np.uint64)
        rv = np.zeros((nb, 7), dtype=np.uint64)
        mi = np.zeros((nb, 22))
        mv = np.zeros((nb, 22))
        lib().rfc_body_diagnostics(C.c_void_p(self.h), _p(ri), _p(rv), _p(mi), _p(mv))
        k = self.nb
        return dict(regime_instant=ri[:k], regime_interval=rv[:k], micro_instant=mi[:k], micro_interval=mv[:k])

    def regime_state(self):
        st = np.zeros((max(self.nb, 1), self.nc), dtype=np.int32)
        self._check(lib().rfc_get_regime_state(C.c_void_p(self.h), _p(st)))
        return st[:self.nb]

    def microstate(self):
        m = np.zeros((max(self.nb, 1), self.nc, 22))
        self._check(lib().rfc_get_microstate(C.c_void_p(self.h), _p(m)))
        return m[:self.nb]

    def mesh_size(self):
        return lib().rfc_mesh_size(C.c_void_p(self.h))
