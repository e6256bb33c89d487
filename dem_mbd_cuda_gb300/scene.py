"""Scene description shared by the engine binding, the generators and tests.

A ``Scene`` holds, as numpy arrays, exactly what the reference's
``CudaDemSolver::initialize`` reads from PARTICLE, BODYSET, CONTROL, the three
MECH blocks and ODE (src/cuda_backend_cuda.cu:302-381).  ``to_c`` turns it into
the ``dem_scene`` struct of include/dem_gb300.h; the returned keep-alive list
must outlive any call that uses the struct.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, replace

import numpy as np


@dataclass
class Mech:
    """Contact material: the MECH fields the GPU path reads
    (include/simulation.h:48-64).  The reference's defaults are dangerous
    (cohesion 1, no damping); every generator sets each field explicitly."""
    epsS: float = 1.0
    mu: float = 0.5
    epsN: float = 1.0
    cohesion: float = 1.0
    beta: float = 1.0
    muT: float = 1.3
    muR: float = 1.0
    kN: float = 1.0


class CMech(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("epsS", "mu", "epsN", "cohesion", "beta", "muT", "muR", "kN")]


_P = C.c_void_p


class CScene(C.Structure):
    _fields_ = [
        ("n_owners", C.c_int), ("owner_id", _P), ("owner_status", _P), ("owner_mass", _P),
        ("owner_radius", _P), ("owner_inertia", _P), ("owner_pos", _P), ("owner_vel", _P),
        ("owner_omega", _P), ("owner_quat", _P),
        ("n_components", C.c_int), ("comp_owner", _P), ("comp_id", _P), ("comp_radius", _P),
        ("comp_offset", _P),
        ("n_walls", C.c_int), ("wall_origin", _P), ("wall_normal", _P),
        ("n_bodies", C.c_int), ("body_mass", _P), ("body_center", _P), ("body_quat", _P),
        ("body_vel", _P), ("body_omega", _P), ("body_inertia", _P), ("body_state", _P),
        ("n_triangles", C.c_int), ("tri_body", _P), ("tri_local", _P),
        ("pp", CMech), ("pt", CMech), ("pw", CMech),
        ("dt", C.c_double), ("gravity", C.c_double * 3), ("gravity_enabled", C.c_int),
        ("universal_gravity_enabled", C.c_int), ("keep_body_particle", C.c_int),
        ("keep_body_detail", C.c_int),
    ]


def _f64(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


@dataclass
class Scene:
    owner_id: np.ndarray
    owner_status: np.ndarray
    owner_mass: np.ndarray
    owner_radius: np.ndarray
    owner_inertia: np.ndarray          # (n, 3)
    pos: np.ndarray                    # (n, 3)
    vel: np.ndarray                    # (n, 3)
    omega: np.ndarray                  # (n, 3) body frame
    quat: np.ndarray                   # (n, 4) w, x, y, z
    pp: Mech = field(default_factory=Mech)
    pt: Mech = field(default_factory=Mech)
    pw: Mech = field(default_factory=Mech)
    dt: float = 1e-5
    gravity: tuple = (0.0, 0.0, 0.0)
    gravity_enabled: int = 0
    universal_gravity_enabled: int = 0
    comp_owner: np.ndarray | None = None
    comp_id: np.ndarray | None = None
    comp_radius: np.ndarray | None = None
    comp_offset: np.ndarray | None = None
    wall_origin: np.ndarray | None = None
    wall_normal: np.ndarray | None = None
    body_mass: np.ndarray | None = None
    body_center: np.ndarray | None = None
    body_quat: np.ndarray | None = None
    body_vel: np.ndarray | None = None
    body_omega: np.ndarray | None = None
    body_inertia: np.ndarray | None = None
    body_state: np.ndarray | None = None
    tri_body: np.ndarray | None = None
    tri_local: np.ndarray | None = None    # (nt, 15): v1, v2, v3, v4, normal
    keep_body_particle: int = 0
    keep_body_detail: int = 0
    name: str = "scene"

    # ------------------------------------------------------------- helpers
    @property
    def n(self) -> int:
        return int(len(self.owner_id))

    @property
    def n_walls(self) -> int:
        return 0 if self.wall_origin is None else int(len(self.wall_origin))

    @property
    def n_bodies(self) -> int:
        return 0 if self.body_mass is None else int(len(self.body_mass))

    @property
    def n_triangles(self) -> int:
        return 0 if self.tri_body is None else int(len(self.tri_body))

    @property
    def n_components(self) -> int:
        return self.n if self.comp_owner is None else int(len(self.comp_owner))

    def copy(self) -> "Scene":
        out = replace(self)
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                setattr(out, k, v.copy())
        return out

    def body_states(self):
        return (self.body_center.copy(), self.body_quat.copy(), self.body_vel.copy(), self.body_omega.copy())

    def to_c(self):
        """Return (CScene, keep_alive)."""
        keep = []

        def ptr(a, conv):
            if a is None:
                return None
            a = conv(a)
            keep.append(a)
            return a.ctypes.data

        s = CScene()
        s.n_owners = self.n
        s.owner_id = ptr(self.owner_id, _i32)
        s.owner_status = ptr(self.owner_status, _i32)
        s.owner_mass = ptr(self.owner_mass, _f64)
        s.owner_radius = ptr(self.owner_radius, _f64)
        s.owner_inertia = ptr(self.owner_inertia, _f64)
        s.owner_pos = ptr(self.pos, _f64)
        s.owner_vel = ptr(self.vel, _f64)
        s.owner_omega = ptr(self.omega, _f64)
        s.owner_quat = ptr(self.quat, _f64)
        if self.comp_owner is not None:
            s.n_components = int(len(self.comp_owner))
            s.comp_owner = ptr(self.comp_owner, _i32)
            s.comp_id = ptr(self.comp_id, _i32)
            s.comp_radius = ptr(self.comp_radius, _f64)
            s.comp_offset = ptr(self.comp_offset, _f64)
        s.n_walls = self.n_walls
        if self.n_walls:
            s.wall_origin = ptr(self.wall_origin, _f64)
            s.wall_normal = ptr(self.wall_normal, _f64)
        s.n_bodies = self.n_bodies
        if self.n_bodies:
            s.body_mass = ptr(self.body_mass, _f64)
            s.body_center = ptr(self.body_center, _f64)
            s.body_quat = ptr(self.body_quat, _f64)
            s.body_vel = ptr(self.body_vel, _f64)
            s.body_omega = ptr(self.body_omega, _f64)
            s.body_inertia = ptr(self.body_inertia, _f64)
            s.body_state = ptr(self.body_state, _i32)
            s.n_triangles = self.n_triangles
            if self.n_triangles:
                s.tri_body = ptr(self.tri_body, _i32)
                s.tri_local = ptr(self.tri_local, _f64)
        for name in ("pp", "pt", "pw"):
            m = getattr(self, name)
            setattr(s, name, CMech(m.epsS, m.mu, m.epsN, m.cohesion, m.beta, m.muT, m.muR, m.kN))
        s.dt = float(self.dt)
        for k in range(3):
            s.gravity[k] = float(self.gravity[k])
        s.gravity_enabled = int(self.gravity_enabled)
        s.universal_gravity_enabled = int(self.universal_gravity_enabled)
        s.keep_body_particle = int(self.keep_body_particle)
        s.keep_body_detail = int(self.keep_body_detail)
        return s, keep


def sphere_inertia(mass, radius):
    """0.4 m r^2 on every axis, as PARTICLE::LoadParticles does
    (src/particle.cpp:86-90)."""
    m = np.asarray(mass, dtype=np.float64)
    r = np.asarray(radius, dtype=np.float64)
    i = 0.4 * m * r * r
    return np.stack([i, i, i], axis=1)


def make_spheres(pos, radius, density=2500.0, vel=None, ids=None, status=None) -> dict:
    """Owner arrays for plain spheres with mass rho * 4/3 pi r^3."""
    pos = _f64(pos).reshape(-1, 3)
    n = len(pos)
    radius = _f64(radius).reshape(n)
    mass = density * (4.0 / 3.0) * np.pi * radius ** 3
    return dict(
        owner_id=_i32(np.arange(n) if ids is None else ids),
        owner_status=_i32(np.zeros(n) if status is None else status),
        owner_mass=mass,
        owner_radius=radius,
        owner_inertia=sphere_inertia(mass, radius),
        pos=pos,
        vel=np.zeros((n, 3)) if vel is None else _f64(vel).reshape(n, 3),
        omega=np.zeros((n, 3)),
        quat=np.tile(np.array([1.0, 0.0, 0.0, 0.0]), (n, 1)),
    )


def mesh_to_triangles(vertices, faces):
    """Body-frame triangle records as BODYSET::LoadBodys builds them
    (src/multibody.cpp:121-145): v2, v3, v4 are the face vertices, the normal
    is normalize((v3-v2) x (v4-v2)) and v1 = centroid - normal * mean edge.
    Faces are 1-based as in the mesh .bt file.  Operations are evaluated in
    the reference's order so the records are bit-identical."""
    V = _f64(vertices).reshape(-1, 3)
    F = np.asarray(faces, dtype=np.int64).reshape(-1, 3) - 1
    v2, v3, v4 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    a1 = v3 - v2
    a2 = v4 - v2
    a3 = v3 - v4

    def nrm(a):
        return np.sqrt(a[:, 0] * a[:, 0] + a[:, 1] * a[:, 1] + a[:, 2] * a[:, 2])

    center = (v2 + v3 + v4) / 3
    mean_size = (nrm(a1) + nrm(a2) + nrm(a3)) / 3
    cr = np.stack([a1[:, 1] * a2[:, 2] - a1[:, 2] * a2[:, 1],
                   a1[:, 2] * a2[:, 0] - a1[:, 0] * a2[:, 2],
                   a1[:, 0] * a2[:, 1] - a1[:, 1] * a2[:, 0]], axis=1)
    ln = nrm(cr)
    inv = np.where(ln > 1e-14, 1.0 / np.where(ln > 1e-14, ln, 1.0), 0.0)
    normal = np.where((ln > 1e-14)[:, None], cr * inv[:, None], 0.0)
    v1 = center - normal * mean_size[:, None]
    return np.concatenate([v1, v2, v3, v4, normal], axis=1)


def concat_scenes(scenes):
    """Concatenated owner/body/triangle arrays in scene order (the numbering
    used by the batched engine)."""
    out = {}
    for key in ("owner_id", "owner_status", "owner_mass", "owner_radius", "owner_inertia", "pos", "vel", "omega", "quat"):
        out[key] = np.concatenate([getattr(s, key) for s in scenes])
    return out
