"""Reference input files: world.par, Particles.bt, Wall.bt, the body CSV and
mesh .bt, read into a ``Scene`` and written back out.

Formats follow the reference's loaders:
  * world.par  -- ``KEY = value`` with ``#`` comments (src/simulation.cpp:158-307);
    ``MECH_`` keys set all three contact classes, ``MECH_PP_/PT_/PW_`` one.
  * Particles.bt -- 17 columns: id status mass radius x y z vx vy vz
    qw qx qy qz wx wy wz (src/particle.cpp:65-73).
  * Wall.bt -- count, then origin and inward normal per wall (src/wall.cpp:8-38).
  * body CSV -- count row, header row, then name, mass, centre, velocity,
    angular velocity, quaternion (w first), 9 inertia entries, optional state
    (src/multibody.cpp:295-435).
  * mesh .bt -- "nverts ntris", vertices, 1-based faces (src/multibody.cpp:41-147).
"""
from __future__ import annotations

import os
import re

import numpy as np

from .scene import Mech, Scene, mesh_to_triangles, sphere_inertia

_MECH_KEYS = {"epsS": "epsS", "mu": "mu", "epsN": "epsN", "cohesive": "cohesion", "beta": "beta",
              "mu_T": "muT", "mu_R": "muR", "kN": "kN"}


def read_world_par(path):
    values = {}
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        for line in f:
            line = line.split("#", 1)[0].strip()
            if not line or "=" not in line:
                continue
            k, v = line.split("=", 1)
            values[k.strip()] = v.strip()
    return values


def _resolve(case_dir, legacy_path):
    """Map the reference's ``Data\\DATA\\InputFile\\...`` paths onto the case
    directory (include/file_utils.h:19-80 redirects them the same way)."""
    p = legacy_path.replace("\\", "/")
    m = re.search(r"InputFile/(.*)$", p)
    if m:
        return os.path.join(case_dir, "InputFile", m.group(1))
    return os.path.join(case_dir, p)


def mechs_from_par(values):
    out = {"pp": Mech(), "pt": Mech(), "pw": Mech()}
    for key, val in values.items():
        if not key.startswith("MECH_"):
            continue
        rest = key[5:]
        targets = ["pp", "pt", "pw"]
        for prefix, t in (("PP_", "pp"), ("PT_", "pt"), ("PW_", "pw")):
            if rest.startswith(prefix):
                targets = [t]
                rest = rest[len(prefix):]
        if rest not in _MECH_KEYS:
            continue
        for t in targets:
            setattr(out[t], _MECH_KEYS[rest], float(val))
    return out


def read_particles(path):
    rows = np.loadtxt(path, ndmin=2)
    if rows.shape[1] != 17:
        raise ValueError(f"{path}: expected 17 columns, got {rows.shape[1]}")
    mass = rows[:, 2].copy()
    radius = rows[:, 3].copy()
    return dict(owner_id=rows[:, 0].astype(np.int32), owner_status=rows[:, 1].astype(np.int32),
                owner_mass=mass, owner_radius=radius, owner_inertia=sphere_inertia(mass, radius),
                pos=rows[:, 4:7].copy(), vel=rows[:, 7:10].copy(), quat=rows[:, 10:14].copy(),
                omega=rows[:, 14:17].copy())


def write_particles(path, scene: Scene):
    data = np.column_stack([scene.owner_id, scene.owner_status, scene.owner_mass, scene.owner_radius, scene.pos,
                            scene.vel, scene.quat, scene.omega])
    fmt = ["%d", "%d"] + ["%.17g"] * 15
    np.savetxt(path, data, fmt=fmt)


def read_walls(path):
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    vals = np.array([float(t) for t in tok[1:1 + 6 * n]]).reshape(n, 6)
    return vals[:, :3].copy(), vals[:, 3:].copy()


def write_walls(path, origin, normal):
    with open(path, "w") as f:
        f.write(f"{len(origin)}\n")
        for o, nn in zip(origin, normal):
            f.write(" ".join("%.17g" % v for v in list(o) + list(nn)) + "\n")


def read_mesh(path):
    with open(path) as f:
        tok = f.read().split()
    nv, nt = int(tok[0]), int(tok[1])
    v = np.array([float(t) for t in tok[2:2 + 3 * nv]]).reshape(nv, 3)
    faces = np.array([int(t) for t in tok[2 + 3 * nv:2 + 3 * nv + 3 * nt]]).reshape(nt, 3)
    return v, faces


def write_mesh(path, vertices, faces):
    with open(path, "w") as f:
        f.write(f"{len(vertices)} {len(faces)}\n")
        for v in vertices:
            f.write("%.17g %.17g %.17g\n" % tuple(v))
        for t in faces:
            f.write("%d %d %d\n" % tuple(t))


def read_bodies(path, case_dir):
    with open(path, encoding="utf-8", errors="replace") as f:
        lines = f.read().splitlines()
    n = int(lines[0].split(",")[0].strip())
    bodies = []
    for i in range(n):
        tok = [t.strip() for t in lines[2 + i].split(",") if t.strip() != ""]
        if len(tok) < 24:
            raise ValueError(f"{path}: body {i + 1} has {len(tok)} columns")
        vals = [float(t) for t in tok[1:24]]
        state = int(tok[24]) if len(tok) >= 25 else 0
        mesh_path = _resolve(case_dir, tok[0])
        v, faces = read_mesh(mesh_path)
        b = dict(mass=vals[0], center=vals[1:4], vel=vals[4:7], omega=vals[7:10], quat=vals[10:14],
                 inertia=vals[14:23], state=state, vertices=v, faces=faces)
        if state == 1:
            b["vel"] = [0.0, 0.0, 0.0]
            b["omega"] = [0.0, 0.0, 0.0]
        bodies.append(b)
    return bodies


def write_bodies(path, bodies, mesh_names):
    with open(path, "w") as f:
        f.write(f"{len(bodies)}" + "," * 24 + "\n")
        f.write("filepath,mass,x,y,z,vx,vy,vz,omega_x,omega_y,omega_z,lambda_x,lambda_y,lambda_z,lambda_w,"
                "I1,I2,I3,I4,I5,I6,I7,I8,I9,state\n")
        for b, name in zip(bodies, mesh_names):
            vals = [b["mass"], *b["center"], *b["vel"], *b["omega"], *b["quat"], *b["inertia"]]
            f.write(name + "," + ",".join("%.17g" % v for v in vals) + ",%d\n" % b["state"])


def attach_bodies(scene_kw, bodies):
    nb = len(bodies)
    tris, tb = [], []
    for i, b in enumerate(bodies):
        t = mesh_to_triangles(b["vertices"], b["faces"])
        tris.append(t)
        tb.append(np.full(len(t), i, dtype=np.int32))
    scene_kw.update(
        body_mass=np.array([b["mass"] for b in bodies], dtype=np.float64),
        body_center=np.array([b["center"] for b in bodies], dtype=np.float64).reshape(nb, 3),
        body_quat=np.array([b["quat"] for b in bodies], dtype=np.float64).reshape(nb, 4),
        body_vel=np.array([b["vel"] for b in bodies], dtype=np.float64).reshape(nb, 3),
        body_omega=np.array([b["omega"] for b in bodies], dtype=np.float64).reshape(nb, 3),
        body_inertia=np.array([b["inertia"] for b in bodies], dtype=np.float64).reshape(nb, 9),
        body_state=np.array([b["state"] for b in bodies], dtype=np.int32),
        tri_body=np.concatenate(tb), tri_local=np.concatenate(tris))
    return scene_kw


def read_case(case_dir):
    """Read a reference case directory (``<case>/InputFile/...``) into a Scene
    plus its ODE settings."""
    par = read_world_par(os.path.join(case_dir, "InputFile", "SettingData", "world.par"))
    kw = read_particles(_resolve(case_dir, par.get("CONTROL_PARTICLES_FILE", "InputFile/Particles/Particles.bt")))
    mechs = mechs_from_par(par)
    kw.update(mechs)
    kw["dt"] = float(par.get("ODE_StepSize", "1e-5"))
    kw["gravity_enabled"] = int(par.get("CONTROL_GRAVITY_FLAG", "0"))
    kw["gravity"] = tuple(float(par.get(k, "0")) for k in ("CONTROL_GRAVITY_X", "CONTROL_GRAVITY_Y", "CONTROL_GRAVITY_Z"))
    kw["universal_gravity_enabled"] = int(par.get("CONTROL_UNIVERSAL_GRAVITATION_FLAG", "0"))
    if int(par.get("CONTROL_WALL_FLAG", "0")):
        o, n = read_walls(_resolve(case_dir, par["CONTROL_WALL_FILE"]))
        kw["wall_origin"], kw["wall_normal"] = o, n
    if int(par.get("CONTROL_MULTIBODY_FLAG", "0")):
        bodies = read_bodies(_resolve(case_dir, par["CONTROL_MULTIBODY_FILE"]), case_dir)
        attach_bodies(kw, bodies)
    kw["keep_body_particle"] = int(par.get("CONTROL_OUTPUT_PARTICLE_FORCE", "1"))
    kw["keep_body_detail"] = int(par.get("CONTROL_OUTPUT_BODY_FORCE", "1"))
    ode = dict(start=int(par.get("ODE_StartStep", "0")), end=int(par.get("ODE_EndStep", "0")),
               output_interval=int(par.get("ODE_OutputInterval", "1")), dt=kw["dt"],
               multibody=int(par.get("CONTROL_MULTIBODY_FLAG", "0")))
    return Scene(**kw, name=os.path.basename(os.path.normpath(case_dir))), ode


def write_case(case_dir, scene: Scene, end_step: int, output_interval: int, body_meshes=None):
    """Write a Scene as a reference case (all MECH_ keys explicit, outputs off)."""
    inp = os.path.join(case_dir, "InputFile")
    for sub in ("SettingData", "Particles", "Environment", "BodySet"):
        os.makedirs(os.path.join(inp, sub), exist_ok=True)
    write_particles(os.path.join(inp, "Particles", "Particles.bt"), scene)
    lines = ["ODE_Option = 1", f"ODE_StepSize = {scene.dt!r}", f"ODE_EndStep = {end_step}", "ODE_StartStep = 0",
             f"ODE_OutputInterval = {output_interval}"]
    for prefix, m in (("PP", scene.pp), ("PT", scene.pt), ("PW", scene.pw)):
        for key, attr in _MECH_KEYS.items():
            lines.append(f"MECH_{prefix}_{key} = {getattr(m, attr)!r}")
    lines += [f"CONTROL_GRAVITY_FLAG = {scene.gravity_enabled}"]
    lines += [f"CONTROL_GRAVITY_{a} = {g!r}" for a, g in zip("XYZ", scene.gravity)]
    lines.append(f"CONTROL_WALL_FLAG = {1 if scene.n_walls else 0}")
    if scene.n_walls:
        write_walls(os.path.join(inp, "Environment", "Wall.bt"), scene.wall_origin, scene.wall_normal)
        lines.append("CONTROL_WALL_FILE = Data\\DATA\\InputFile\\Environment\\Wall.bt")
    lines.append(f"CONTROL_MULTIBODY_FLAG = {1 if scene.n_bodies else 0}")
    if scene.n_bodies and body_meshes is not None:
        names = []
        bodies = []
        for i, (v, faces) in enumerate(body_meshes):
            fname = f"body{i + 1}.bt"
            write_mesh(os.path.join(inp, "BodySet", fname), v, faces)
            names.append("Data\\DATA\\InputFile\\BodySet\\" + fname)
            bodies.append(dict(mass=scene.body_mass[i], center=scene.body_center[i], vel=scene.body_vel[i],
                               omega=scene.body_omega[i], quat=scene.body_quat[i], inertia=scene.body_inertia[i],
                               state=int(scene.body_state[i])))
        write_bodies(os.path.join(inp, "BodySet", "bodies.csv"), bodies, names)
        lines.append("CONTROL_MULTIBODY_FILE = Data\\DATA\\InputFile\\BodySet\\bodies.csv")
    lines += ["CONTROL_UNIVERSAL_GRAVITATION_FLAG = 0",
              "CONTROL_PARTICLES_FILE = Data\\DATA\\InputFile\\Particles\\Particles.bt",
              "CONTROL_OUTPUT_PARTICLE_STATE = 0", "CONTROL_OUTPUT_PARTICLE_FORCE = 0",
              "CONTROL_OUTPUT_BODY_STATE = 0", "CONTROL_OUTPUT_BODY_FORCE = 0", "CONTROL_OUTPUT_SUMMARY = 0"]
    with open(os.path.join(inp, "SettingData", "world.par"), "w") as f:
        f.write("\n".join(lines) + "\n")
