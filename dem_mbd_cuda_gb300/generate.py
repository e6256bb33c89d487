"""Seeded synthetic scenes in the reference's units and conventions.

The reference ships no benchmark inputs beyond its 1704-particle validation
cases, so every workload is generated here from a fixed seed.  Beds are built
either on a jittered simple-cubic lattice (``bed``: radii drawn from the
stated distribution and clipped, in lattice-wavefront order, so that no pair
overlaps by more than ``overlap`` metres; layers start apart and the bed
falls) or as vertical columns in force balance (``column_bed``: every sphere
rests on the one below with the overlap its load needs, so the bed is
settled at step 0).
All MECH fields are set explicitly (the reference's defaults enable cohesion).

Meshes follow the reference's convention: faces are 1-based vertex triples
whose normal (v3 - v2) x (v4 - v2) points toward the particles
(src/multibody.cpp:123-135), with vertices in the body frame.
"""
from __future__ import annotations

import numpy as np

from .scene import Mech, Scene, make_spheres, mesh_to_triangles

DENSITY = 2500.0


def mech(kN=1e5, epsN=0.5, epsS=0.5, mu=0.3, muT=0.0, muR=0.0, beta=0.5, cohesion=0.0):
    return Mech(epsS=epsS, mu=mu, epsN=epsN, cohesion=cohesion, beta=beta, muT=muT, muR=muR, kN=kN)


def box_walls(lo, hi, top=False):
    """Floor and four side walls of an axis-aligned box, normals inward
    (Wall.bt convention, src/wall.cpp:13-35)."""
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    o, n = [], []
    o.append([0, 0, lo[2]]); n.append([0, 0, 1])
    if top:
        o.append([0, 0, hi[2]]); n.append([0, 0, -1])
    o.append([lo[0], 0, 0]); n.append([1, 0, 0])
    o.append([hi[0], 0, 0]); n.append([-1, 0, 0])
    o.append([0, lo[1], 0]); n.append([0, 1, 0])
    o.append([0, hi[1], 0]); n.append([0, -1, 0])
    return np.array(o, float), np.array(n, float)


def lattice_sites(counts, pitch, origin, jitter, rng):
    nx, ny, nz = counts
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    idx = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1)
    pos = np.asarray(origin, float) + idx * pitch
    pos = pos + rng.uniform(-jitter, jitter, size=pos.shape)
    return idx, pos


def clip_radii(idx, pos, radius, counts, overlap, keep=None):
    """Clip radii in wavefront order (ix+iy+iz) against the six face
    neighbours assigned before, so every pair overlaps by at most
    ``overlap``; pairs that would have overlapped more end up in contact."""
    nx, ny, nz = counts
    r = radius.copy()
    lin = (idx[:, 0] * ny + idx[:, 1]) * nz + idx[:, 2]
    grid = -np.ones(nx * ny * nz, dtype=np.int64)
    grid[lin] = np.arange(len(lin))
    if keep is not None:
        grid[lin[~keep]] = -1
    wave = idx.sum(axis=1)
    order = np.argsort(wave, kind="stable")
    bounds = np.searchsorted(wave[order], np.arange(wave.max() + 2))
    for k in range(len(bounds) - 1):
        sel = order[bounds[k]:bounds[k + 1]]
        if keep is not None:
            sel = sel[keep[sel]]
        if len(sel) == 0:
            continue
        for d in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
            nb = idx[sel] - np.array(d)
            ok = (nb >= 0).all(axis=1)
            nl = (nb[:, 0] * ny + nb[:, 1]) * nz + nb[:, 2]
            j = np.where(ok, grid[np.where(ok, nl, 0)], -1)
            has = j >= 0
            if not has.any():
                continue
            s, jj = sel[has], j[has]
            dist = np.linalg.norm(pos[s] - pos[jj], axis=1)
            r[s] = np.minimum(r[s], dist - r[jj] + overlap)
    return r


def bed(n, rmin, rmax, pitch, origin, aspect=(1, 1, None), seed=0, jitter=0.2e-3, overlap=1e-7, radius_fn=None,
        inside=None, center_xy=True, nxy=None):
    """Lattice bed of about ``n`` spheres; ``inside(pos) -> bool mask`` removes
    sites (e.g. the volume of a body).  With ``center_xy`` the lattice is
    centred on x = y = 0 and ``origin`` only sets its lowest z."""
    rng = np.random.default_rng(seed)
    ax, ay = aspect[0], aspect[1]
    base = (n / (ax * ay)) ** (1.0 / 3.0)
    nx = max(1, int(round(base * ax))) if nxy is None else nxy
    ny = max(1, int(round(base * ay))) if nxy is None else nxy
    nz = max(1, int(np.ceil(n / (nx * ny))))
    counts = (nx, ny, nz)
    origin = np.array(origin, float)
    if center_xy:
        origin[0] = -(nx - 1) * pitch / 2
        origin[1] = -(ny - 1) * pitch / 2
    while True:
        counts = (nx, ny, nz)
        idx, pos = lattice_sites(counts, pitch, origin, jitter, np.random.default_rng(seed))
        keep = np.ones(len(pos), bool)
        if inside is not None:
            keep &= ~inside(pos)
        if keep.sum() >= n:
            break
        nz += max(1, int(np.ceil((n - keep.sum()) / (nx * ny))))
    # trim to exactly n kept sites, lowest layers first
    order = np.lexsort((idx[:, 1], idx[:, 0], idx[:, 2]))
    kept = order[keep[order]][:n]
    keep = np.zeros(len(pos), bool)
    keep[kept] = True
    if radius_fn is None:
        radius = rng.uniform(rmin, rmax, size=len(pos))
    else:
        radius = radius_fn(rng, len(pos))
    radius = clip_radii(idx, pos, radius, counts, overlap, keep=keep)
    radius = np.maximum(radius, 0.25 * rmin)
    sel = np.nonzero(keep)[0]
    return pos[sel], radius[sel], rng


def box_mesh(half, subdiv):
    """Closed box centred at the origin, faces subdivided (na, nb, nc) along
    x, y, z; outward normals."""
    hx, hy, hz = half
    na, nb, nc = subdiv
    verts, faces = [], []

    def face(origin, u, v, nu, nv, normal):
        o = np.asarray(origin, float)
        u = np.asarray(u, float)
        v = np.asarray(v, float)
        base = len(verts)
        for a in range(nu + 1):
            for b in range(nv + 1):
                verts.append(o + u * (a / nu) + v * (b / nv))
        for a in range(nu):
            for b in range(nv):
                p00 = base + a * (nv + 1) + b
                p10 = p00 + (nv + 1)
                p01 = p00 + 1
                p11 = p10 + 1
                tri = [(p00, p10, p11), (p00, p11, p01)]
                for t in tri:
                    vv = [verts[k] for k in t]
                    nrm = np.cross(vv[1] - vv[0], vv[2] - vv[0])
                    if np.dot(nrm, normal) < 0:
                        t = (t[0], t[2], t[1])
                    faces.append([k + 1 for k in t])

    face([hx, -hy, -hz], [0, 2 * hy, 0], [0, 0, 2 * hz], nb, nc, [1, 0, 0])
    face([-hx, -hy, -hz], [0, 2 * hy, 0], [0, 0, 2 * hz], nb, nc, [-1, 0, 0])
    face([-hx, hy, -hz], [2 * hx, 0, 0], [0, 0, 2 * hz], na, nc, [0, 1, 0])
    face([-hx, -hy, -hz], [2 * hx, 0, 0], [0, 0, 2 * hz], na, nc, [0, -1, 0])
    face([-hx, -hy, hz], [2 * hx, 0, 0], [0, 2 * hy, 0], na, nb, [0, 0, 1])
    face([-hx, -hy, -hz], [2 * hx, 0, 0], [0, 2 * hy, 0], na, nb, [0, 0, -1])
    return np.array(verts), np.array(faces, dtype=np.int64)


def cylinder_mesh(radius, length, ntheta, nx, nrings):
    """Closed cylinder along x centred at the origin with INWARD normals (a
    drum: particles are inside)."""
    verts, faces = [], []
    th = np.linspace(0, 2 * np.pi, ntheta, endpoint=False)
    xs = np.linspace(-length / 2, length / 2, nx + 1)

    def tri(a, b, c, want):
        va, vb, vc = verts[a], verts[b], verts[c]
        nrm = np.cross(vb - va, vc - va)
        if np.dot(nrm, want) < 0:
            b, c = c, b
        faces.append([a + 1, b + 1, c + 1])

    base = len(verts)
    for x in xs:
        for t in th:
            verts.append(np.array([x, radius * np.cos(t), radius * np.sin(t)]))
    for i in range(nx):
        for j in range(ntheta):
            a = base + i * ntheta + j
            b = base + i * ntheta + (j + 1) % ntheta
            c = base + (i + 1) * ntheta + j
            d = base + (i + 1) * ntheta + (j + 1) % ntheta
            mid = (verts[a] + verts[d]) / 2
            want = -np.array([0, mid[1], mid[2]])
            tri(a, b, d, want)
            tri(a, d, c, want)
    for side, x in ((-1, -length / 2), (1, length / 2)):
        want = np.array([-side, 0, 0], float)
        center = len(verts)
        verts.append(np.array([x, 0.0, 0.0]))
        rings = [center]
        for k in range(1, nrings + 1):
            rk = radius * k / nrings
            start = len(verts)
            for t in th:
                verts.append(np.array([x, rk * np.cos(t), rk * np.sin(t)]))
            rings.append(start)
        for j in range(ntheta):
            tri(center, rings[1] + j, rings[1] + (j + 1) % ntheta, want)
        for k in range(1, nrings):
            for j in range(ntheta):
                a = rings[k] + j
                b = rings[k] + (j + 1) % ntheta
                c = rings[k + 1] + j
                d = rings[k + 1] + (j + 1) % ntheta
                tri(a, b, d, want)
                tri(a, d, c, want)
    return np.array(verts), np.array(faces, dtype=np.int64)


def _attach(kw, bodies):
    nb = len(bodies)
    tris, tb = [], []
    for i, b in enumerate(bodies):
        t = mesh_to_triangles(b["vertices"], b["faces"])
        tris.append(t)
        tb.append(np.full(len(t), i, dtype=np.int32))
    kw.update(body_mass=np.array([b["mass"] for b in bodies], float),
              body_center=np.array([b["center"] for b in bodies], float).reshape(nb, 3),
              body_quat=np.array([b.get("quat", [1, 0, 0, 0]) for b in bodies], float).reshape(nb, 4),
              body_vel=np.array([b.get("vel", [0, 0, 0]) for b in bodies], float).reshape(nb, 3),
              body_omega=np.array([b.get("omega", [0, 0, 0]) for b in bodies], float).reshape(nb, 3),
              body_inertia=np.array([b["inertia"] for b in bodies], float).reshape(nb, 9),
              body_state=np.array([b["state"] for b in bodies], np.int32),
              tri_body=np.concatenate(tb), tri_local=np.concatenate(tris))
    return kw


def pure_dem(n=20000, seed=1000, rmin=1.8e-3, rmax=2.2e-3, box=(0.2, 0.2, 0.4), dt=1e-5, kN=1e5, epsN=0.5, mu=0.3,
             pitch=None, name="c0_pure_dem", fill_width=False, jitter=0.2e-3):
    """Config 0: spheres r ~ U[rmin, rmax] on a jittered lattice in a box of 5
    walls (floor + 4 sides), kN 1e5, restitution 0.5, friction 0.3."""
    pitch = pitch if pitch is not None else 2.0 * rmin + 0.1e-3
    lo = np.array([-box[0] / 2, -box[1] / 2, 0.0])
    hi = np.array([box[0] / 2, box[1] / 2, box[2]])
    width = box[0] - 2 * rmax
    per = int(width // pitch)
    origin = lo + np.array([rmax, rmax, rmax]) + (width - (per - 1) * pitch) / 2 * np.array([1, 1, 0])
    origin[2] = rmax + 0.3e-3
    pos, rad, _ = bed(n, rmin, rmax, pitch, origin, aspect=(1, 1, None), seed=seed, nxy=per if fill_width else None,
                      jitter=jitter)
    assert pos[:, 0].max() + rad.max() < hi[0] and pos[:, 1].max() + rad.max() < hi[1], "bed exceeds the box"
    kw = make_spheres(pos, rad, DENSITY)
    wo, wn = box_walls(lo, hi)
    m = mech(kN=kN, epsN=epsN, epsS=epsN, mu=mu)
    return Scene(**kw, pp=m, pt=m, pw=m, dt=dt, gravity=(0.0, 0.0, -9.81), gravity_enabled=1, wall_origin=wo,
                 wall_normal=wn, name=name)


def column_bed(n, col_xy, base_z, radius_fn, rng, cap, g, kN, kN_base, density=DENSITY, kmax=None):
    """A bed of vertical sphere columns in static equilibrium under gravity.

    Column c stands at ``col_xy[c]``; its lowest sphere rests on the support
    ``base_z(xy, r) -> z`` (centre height of a sphere of radius r touching
    the support, vectorised over columns) and every sphere rests on the one
    below it.  Radii come from ``radius_fn`` capped at ``cap`` (half the
    smallest lateral gap between column axes), so spheres of neighbouring
    columns never touch.  The n lowest spheres (by top height) are kept, and
    each contact is then given the overlap that carries the weight above it
    (g * sum of masses above / kN, kN_base for the support): every particle
    starts at rest in force balance with its contacts closed, which a plain
    lattice (gaps between layers) does not give.  Returns positions, radii
    and the column index of every sphere."""
    m = len(col_xy)
    kmax = kmax or int(np.ceil(3.0 * n / max(m, 1))) + 8
    r = np.minimum(radius_fn(rng, m * kmax).reshape(m, kmax), cap)
    z0 = base_z(col_xy, r[:, 0])
    ok = np.isfinite(z0)
    z = np.empty_like(r)
    z[:, 0] = z0
    z[:, 1:] = z0[:, None] + np.cumsum(r[:, :-1] + r[:, 1:], axis=1)
    top = z + r
    top[~ok] = np.inf
    flat = np.argsort(top, axis=None, kind="stable")[:n]
    if not np.isfinite(top.flat[flat[-1]]):
        raise ValueError("column bed: not enough room for %d spheres" % n)
    keep = np.zeros(m * kmax, bool)
    keep[flat] = True
    keep = keep.reshape(m, kmax)
    # a column keeps a contiguous run from its base (top heights increase
    # along a column), so the counts give the kept spheres directly
    cnt = keep.sum(axis=1)
    assert np.array_equal(keep, np.arange(kmax)[None, :] < cnt[:, None])
    mass = density * (4.0 / 3.0) * np.pi * r ** 3 * keep
    above = np.cumsum(mass[:, ::-1], axis=1)[:, ::-1]   # weight carried by each sphere's lower contact
    delta = g * above / kN
    delta[:, 0] = g * above[:, 0] / kN_base
    z = z - np.cumsum(delta, axis=1)
    sel = keep.ravel()
    cols = np.repeat(np.arange(m), kmax)[sel]
    pos = np.column_stack([col_xy[cols, 0], col_xy[cols, 1], z.ravel()[sel]])
    return pos, r.ravel()[sel], cols


def column_grid(lo, hi, pitch, jitter, rng, hexagonal=False):
    """Column axes on a square lattice covering [lo, hi] (2-D), jittered;
    or (``hexagonal``) on staggered rows ``pitch * sqrt(3) / 2`` apart, every
    other row shifted by half a pitch, which keeps the nearest axes
    ``pitch`` apart with 15% more columns per area."""
    if hexagonal:
        dy = pitch * np.sqrt(3.0) / 2.0
        ny = int(np.floor((hi[1] - lo[1]) / dy)) + 1
        oy = lo[1] + 0.5 * ((hi[1] - lo[1]) - (ny - 1) * dy)
        rows = []
        for j in range(ny):
            shift = 0.5 * pitch * (j % 2)
            nx = int(np.floor((hi[0] - lo[0] - shift) / pitch)) + 1
            ox = lo[0] + shift + 0.5 * ((hi[0] - lo[0] - shift) - (nx - 1) * pitch)
            rows.append(np.column_stack([ox + pitch * np.arange(nx), np.full(nx, oy + j * dy)]))
        xy = np.concatenate(rows)
        return xy + rng.uniform(-jitter, jitter, size=xy.shape)
    nx = int(np.floor((hi[0] - lo[0]) / pitch)) + 1
    ny = int(np.floor((hi[1] - lo[1]) / pitch)) + 1
    ox = lo[0] + 0.5 * ((hi[0] - lo[0]) - (nx - 1) * pitch)
    oy = lo[1] + 0.5 * ((hi[1] - lo[1]) - (ny - 1) * pitch)
    gx, gy = np.meshgrid(ox + pitch * np.arange(nx), oy + pitch * np.arange(ny), indexing="ij")
    xy = np.column_stack([gx.ravel(), gy.ravel()])
    return xy + rng.uniform(-jitter, jitter, size=xy.shape)


def mbd_blade_plate(n=200000, seed=1001, rmin=1.5e-3, rmax=2.5e-3, box=0.4, dt=5e-6, name="c1_dem_mbd"):
    """Config 1: spheres r ~ U[1.5, 2.5] mm in a 0.4 m box with a rotating
    blade (prescribed, omega_z = 3) buried in the bed and a 1 kg dynamic
    plate (inertia 1e-3 I) resting on it; wall/triangle friction 0.4.

    The bed is the settled state of the dropped spheres: vertical columns
    in force balance (``column_bed``) on the floor, and on the blade's top
    face where a column stands over the blade."""
    rng = np.random.default_rng(seed)
    g = 9.81
    pitch, jitter = 2.0 * rmax + 0.3e-3, 0.1e-3
    cap = 0.5 * pitch - jitter - 1e-6
    lo = np.array([-box / 2, -box / 2, 0.0])
    hi = np.array([box / 2, box / 2, box])
    edge = rmax + 0.3e-3
    xy = column_grid(lo[:2] + edge, hi[:2] - edge, pitch, jitter, rng)
    blade_half = (0.12, 0.006, 0.05)
    blade_center = np.array([0.0, 0.0, 0.06])
    blade_v, blade_f = box_mesh(blade_half, (32, 2, 13))
    blade_top = blade_center[2] + blade_half[2]
    on_blade = (np.abs(xy[:, 0]) < blade_half[0]) & (np.abs(xy[:, 1]) < blade_half[1])
    near_blade = (np.abs(xy[:, 0]) < blade_half[0] + rmax + 0.5e-3) & \
                 (np.abs(xy[:, 1]) < blade_half[1] + rmax + 0.5e-3)
    xy = xy[on_blade | ~near_blade]
    on_blade = (np.abs(xy[:, 0]) < blade_half[0]) & (np.abs(xy[:, 1]) < blade_half[1])

    def base_z(p, r):
        return np.where(on_blade, blade_top + r, r)

    pos, rad, _ = column_bed(n, xy, base_z, lambda rg, k: rg.uniform(rmin, rmax, size=k), rng, cap, g, 1e5, 1e5)
    plate_half = (0.05, 0.05, 0.002)
    plate_xy = np.array([0.08, 0.08])
    under = (np.abs(pos[:, 0] - plate_xy[0]) < plate_half[0]) & (np.abs(pos[:, 1] - plate_xy[1]) < plate_half[1])
    top = float((pos[under, 2] + rad[under]).max())
    plate_v, plate_f = box_mesh(plate_half, (6, 6, 1))
    plate_center = np.array([plate_xy[0], plate_xy[1], top + plate_half[2] - 2e-7])
    kw = make_spheres(pos, rad, DENSITY)
    wo, wn = box_walls(lo, hi)
    pp = mech(kN=1e5, epsN=0.5, epsS=0.5, mu=0.3)
    pt = mech(kN=1e5, epsN=0.5, epsS=0.5, mu=0.4)
    bodies = [dict(vertices=blade_v, faces=blade_f, mass=5.0, center=blade_center, omega=[0, 0, 3.0],
                   inertia=[1, 0, 0, 0, 1, 0, 0, 0, 1], state=2),
              dict(vertices=plate_v, faces=plate_f, mass=1.0, center=plate_center,
                   inertia=[1e-3, 0, 0, 0, 1e-3, 0, 0, 0, 1e-3], state=0)]
    _attach(kw, bodies)
    return Scene(**kw, pp=pp, pt=pt, pw=pt, dt=dt, gravity=(0.0, 0.0, -g), gravity_enabled=1, wall_origin=wo,
                 wall_normal=wn, name=name), [(blade_v, blade_f), (plate_v, plate_f)]


def drum(n=2000000, seed=1002, radius=0.3, length=0.5, omega=2.0, dt=2e-6, name="c2_drum", ntheta=160, nx=50,
         nrings=6, pitch=4.11e-3):
    """Config 2: lognormal radii (median 1 mm, sigma 0.25, clipped to
    [0.5, 2] mm) in a rotating closed cylinder (axis x, inward normals,
    prescribed omega_x), friction 0.5, restitution 0.3, kN 1e5.

    The bed is settled and turning with the drum: vertical columns in force
    balance (``column_bed``) standing on the cylinder's facets, every
    sphere moving with the drum's rigid rotation (v = omega x p, spin =
    omega), so the wall does not slip under the bed at the start.  Columns
    stand on a hexagonal lattice 4.11 mm apart, which admits every radius up
    to the 2 mm clip; 2,000,000 spheres then fill 45% of the drum (solid
    fraction 0.17 below the bed surface).  A 40% fill with 2M spheres would
    need a solid fraction of 0.2, denser than columns that admit 2 mm
    spheres pack."""
    rng = np.random.default_rng(seed)
    g = 9.81

    def radius_fn(rg, k):
        return np.clip(np.exp(np.log(1e-3) + 0.25 * rg.standard_normal(k)), 0.5e-3, 2.0e-3)

    jitter = 0.05e-3
    cap = 0.5 * pitch - jitter - 1e-6
    half_len = length / 2 - cap - 0.5e-3
    inner = radius * np.cos(np.pi / ntheta)          # facet plane distance from the axis
    reach = np.sqrt((inner - cap) ** 2 - (0.5 * inner) ** 2)
    xy = column_grid(np.array([-half_len, -reach]), np.array([half_len, reach]), pitch, jitter, rng, hexagonal=True)
    # facets of the lower half: plane (cos a, sin a) . (y, z) = inner at the
    # facet's mid angle a (sin a < 0); a sphere of radius r inside has
    # (cos a, sin a) . (y, z) <= inner - r for every facet, so on the
    # vertical line at y its lowest centre is the largest of the bounds.
    mids = (np.arange(ntheta) + 0.5) * (2 * np.pi / ntheta)
    lower = mids[np.sin(mids) < -0.3]
    ca, sa = np.cos(lower), np.sin(lower)

    def base_z(p, r):
        y = p[:, 1][:, None]
        zc = ((inner - r[:, None]) - ca[None, :] * y) / sa[None, :]
        return zc.max(axis=1)

    pos, rad, _ = column_bed(n, xy, base_z, radius_fn, rng, cap, g, 1e5, 1e5)
    w = np.array([omega, 0.0, 0.0])
    vel = np.cross(w[None, :], pos)
    kw = make_spheres(pos, rad, DENSITY, vel=vel)
    kw["omega"] = np.tile(w, (len(pos), 1))
    v, f = cylinder_mesh(radius, length, ntheta, nx, nrings)
    m = mech(kN=1e5, epsN=0.3, epsS=0.3, mu=0.5)
    bodies = [dict(vertices=v, faces=f, mass=100.0, center=[0, 0, 0], omega=[omega, 0, 0],
                   inertia=[10, 0, 0, 0, 10, 0, 0, 0, 10], state=2)]
    _attach(kw, bodies)
    return Scene(**kw, pp=m, pt=m, pw=m, dt=dt, gravity=(0.0, 0.0, -g), gravity_enabled=1, name=name), [(v, f)]


def box_columns(n, seed, rmin=1.8e-3, rmax=2.2e-3, box=(0.1, 0.1, 0.4), dt=1e-5, kN=1e5, epsN=0.5, mu=0.3,
                name="box_columns"):
    """A settled bed of n spheres r ~ U[rmin, rmax] in a box of 5 walls
    (floor + 4 sides): vertical columns in force balance on the floor
    (``column_bed``)."""
    rng = np.random.default_rng(seed)
    g = 9.81
    pitch, jitter = 2.0 * rmax + 0.2e-3, 0.05e-3
    cap = 0.5 * pitch - jitter - 1e-6
    lo = np.array([-box[0] / 2, -box[1] / 2, 0.0])
    hi = np.array([box[0] / 2, box[1] / 2, box[2]])
    edge = rmax + 0.2e-3
    xy = column_grid(lo[:2] + edge, hi[:2] - edge, pitch, jitter, rng)
    pos, rad, _ = column_bed(n, xy, lambda p, r: r, lambda rg, k: rg.uniform(rmin, rmax, size=k), rng, cap, g, kN, kN)
    if (pos[:, 2] + rad).max() > hi[2]:
        raise ValueError("column bed exceeds the box height")
    kw = make_spheres(pos, rad, DENSITY)
    wo, wn = box_walls(lo, hi)
    m = mech(kN=kN, epsN=epsN, epsS=epsN, mu=mu)
    return Scene(**kw, pp=m, pt=m, pw=m, dt=dt, gravity=(0.0, 0.0, -g), gravity_enabled=1, wall_origin=wo,
                 wall_normal=wn, name=name)


def batch(nscenes=256, seed=1004, nmin=2000, nmax=40000, dt=1e-5, settled=False):
    """Config 4: independent box scenes with N_s ~ U[2k, 40k], per-scene
    friction ~ U[0.1, 0.7] and restitution ~ U[0.2, 0.8], in 0.1 x 0.1 x
    0.4 m boxes of 5 walls: jittered lattices at rest (``settled=False``;
    4.5 mm apart, so every radius of U[1.8, 2.2] mm fits and the layers fall
    onto each other and settle during the run) or settled column beds."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(nscenes):
        ns = int(rng.integers(nmin, nmax + 1))
        mu = float(rng.uniform(0.1, 0.7))
        e = float(rng.uniform(0.2, 0.8))
        if settled:
            sc = box_columns(ns, seed * 1000 + s, dt=dt, epsN=e, mu=mu, name=f"c4_scene{s}")
        else:
            sc = pure_dem(n=ns, seed=seed * 1000 + s, box=(0.1, 0.1, 0.4), dt=dt, epsN=e, mu=mu, name=f"c4_scene{s}",
                          fill_width=True, pitch=4.5e-3, jitter=0.05e-3)
        out.append(sc)
    return out


def adjoint_settle(n=50000, seed=1003, dt=1e-5, vel_std=0.05, plate=True, name="c3_adjoint"):
    """Config 3: spheres r ~ U[1.8, 2.2] mm on a lattice in a 0.1 m box of 5
    walls (open top, walls 0.6 m high), seeded normal initial velocities (std
    0.05 m/s); the bed settles during the run.  With ``plate`` the config-1
    plate (1 kg, 100 x 100 x 4 mm, 192 triangles, inertia 1e-3 I, dynamic)
    rests on the highest sphere, centred over the box."""
    sc = pure_dem(n=n, seed=seed, box=(0.1, 0.1, 0.6), dt=dt, name=name, fill_width=True)
    rng = np.random.default_rng(seed + 1)
    sc.vel = rng.normal(0.0, vel_std, size=sc.vel.shape)
    if not plate:
        return sc
    kw = {f: getattr(sc, f) for f in ("owner_id", "owner_status", "owner_mass", "owner_radius", "owner_inertia", "pos",
                                      "vel", "omega", "quat")}
    half = (0.05, 0.05, 0.002)
    plate_v, plate_f = box_mesh(half, (6, 6, 1))
    top = float((sc.pos[:, 2] + sc.owner_radius).max())
    bodies = [dict(vertices=plate_v, faces=plate_f, mass=1.0, center=[0.0, 0.0, top + half[2] - 2e-7],
                   inertia=[1e-3, 0, 0, 0, 1e-3, 0, 0, 0, 1e-3], state=0)]
    _attach(kw, bodies)
    return Scene(**kw, pp=sc.pp, pt=sc.pw, pw=sc.pw, dt=sc.dt, gravity=sc.gravity, gravity_enabled=sc.gravity_enabled,
                 wall_origin=sc.wall_origin, wall_normal=sc.wall_normal, name=name)


def small_mbd(n=400, seed=7, dt=2e-5, caps=True, name="small_mbd"):
    """A few hundred spheres on a tilted plate body plus walls, for tests.

    With ``caps=False`` the particle-triangle material cannot reach its
    Coulomb cap (mu = 1e20) and has zero twisting and rolling limits
    (mu_T = mu_R = 0, always capped to zero): the
    reference's per-triangle re-check of a capped manifold history compares
    two numbers equal up to rounding, so trajectories that hit a cap are not
    reproducible bit for bit between any two builds."""
    rmin, rmax = 1.8e-3, 2.2e-3
    pitch = 3.9e-3
    k = int(np.ceil(np.sqrt(n / 4)))
    origin = np.array([-(k - 1) * pitch / 2, -(k - 1) * pitch / 2, 0.004])
    pos, rad, rng = bed(n, rmin, rmax, pitch, origin, aspect=(1, 1, None), seed=seed, overlap=5e-6)
    kw = make_spheres(pos, rad, DENSITY, vel=rng.normal(0, 0.01, size=(len(pos), 3)))
    kw["omega"] = rng.normal(0, 5.0, size=(len(pos), 3))
    half = k * pitch / 2 + 0.01
    plate_v, plate_f = box_mesh((half, half, 0.001), (8, 8, 1))
    th = 0.05
    qp = [np.cos(th / 2), np.sin(th / 2), 0.0, 0.0]
    wo, wn = box_walls([-half, -half, -0.05], [half, half, 0.2])
    m = mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=0.1, muR=0.05, beta=0.5, cohesion=0.0)
    mt = m if caps else mech(kN=1e5, epsN=0.5, epsS=0.6, mu=1e20, muT=0.0, muR=0.0, beta=0.5)
    bodies = [dict(vertices=plate_v, faces=plate_f, mass=0.5, center=[0.0, 0.0, 0.0011], quat=qp,
                   omega=[0.0, 0.0, 0.5], inertia=[1e-3, 0, 0, 0, 1e-3, 0, 0, 0, 2e-3], state=0)]
    _attach(kw, bodies)
    return Scene(**kw, pp=m, pt=mt, pw=m, dt=dt, gravity=(0.0, 0.0, -9.81), gravity_enabled=1, wall_origin=wo,
                 wall_normal=wn, keep_body_particle=1, keep_body_detail=1, name=name)


def plate_on_monolayer(nx=4, ny=4, r=2e-3, gap=0.4e-3, plate_mass=0.01, seed=11, vel_std=1e-3, omega_std=2.0,
                       dt=1e-5, name="plate_on_monolayer"):
    """A dynamic plate resting on one layer of equal spheres on the floor of
    a walled box (tests of the rigid-body reverse mode): every sphere under
    the plate touches it from the first step, with the small overlap the
    plate's weight needs.  The particle-triangle material has no Coulomb,
    twisting or rolling cap (mu = 1e20, mu_T = mu_R = 0), so no contact
    sits on a cap."""
    rng = np.random.default_rng(seed)
    g = 9.81
    pitch = 2 * r + gap
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    m1 = DENSITY * 4.0 / 3.0 * np.pi * r ** 3
    n = nx * ny
    load = (m1 + plate_mass / n) * g
    zc = r - load / 1e5          # the floor overlap that carries sphere and plate share
    pos = np.stack([X.ravel(), Y.ravel(), np.full(n, zc)], axis=1)
    rad = np.full(n, r)
    kw = make_spheres(pos, rad, DENSITY, vel=rng.normal(0, vel_std, size=(n, 3)))
    kw["omega"] = rng.normal(0, omega_std, size=(n, 3))
    half = (nx * pitch / 2, ny * pitch / 2, 1e-3)
    plate_v, plate_f = box_mesh(half, (nx, ny, 1))
    top = zc + r
    plate_center = [0.0, 0.0, top + half[2] - (plate_mass / n) * g / 1e5]
    ix = plate_mass * (half[1] ** 2 + half[2] ** 2) / 3
    iy = plate_mass * (half[0] ** 2 + half[2] ** 2) / 3
    iz = plate_mass * (half[0] ** 2 + half[1] ** 2) / 3
    bodies = [dict(vertices=plate_v, faces=plate_f, mass=plate_mass, center=plate_center,
                   inertia=[ix, 0, 0, 0, iy, 0, 0, 0, iz], state=0)]
    _attach(kw, bodies)
    lo = [-half[0] - 5e-3, -half[1] - 5e-3, 0.0]
    hi = [half[0] + 5e-3, half[1] + 5e-3, 0.05]
    wo, wn = box_walls(lo, hi)
    m = mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=0.1, muR=0.05, beta=0.5)
    mt = mech(kN=1e5, epsN=0.5, epsS=0.6, mu=1e20, muT=0.0, muR=0.0, beta=0.5)
    return Scene(**kw, pp=m, pt=mt, pw=m, dt=dt, gravity=(0.0, 0.0, -g), gravity_enabled=1, wall_origin=wo,
                 wall_normal=wn, name=name)


def small_dem(n=500, seed=3, dt=1e-5, rmin=1.8e-3, rmax=2.2e-3, vel_std=0.01, omega_std=5.0, muT=0.1, muR=0.05,
              overlap=5e-6, name="small_dem"):
    """A few hundred spheres in a small box with random velocities and spins,
    all history channels active (tests)."""
    box = (0.04, 0.04, 0.1)
    pitch = 3.9e-3
    lo = np.array([-box[0] / 2, -box[1] / 2, 0.0])
    hi = np.array([box[0] / 2, box[1] / 2, box[2]])
    per = int((box[0] - 2 * rmax) // pitch)
    span = (per - 1) * pitch
    origin = np.array([-span / 2, -span / 2, rmax + 0.1e-3])
    pos, rad, rng = bed(n, rmin, rmax, pitch, origin, aspect=(1, 1, None), seed=seed, overlap=overlap)
    kw = make_spheres(pos, rad, DENSITY, vel=rng.normal(0, vel_std, size=(len(pos), 3)))
    kw["omega"] = rng.normal(0, omega_std, size=(len(pos), 3))
    q = rng.normal(size=(len(pos), 4))
    kw["quat"] = q / np.linalg.norm(q, axis=1, keepdims=True)
    wo, wn = box_walls(lo, hi)
    m = mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=muT, muR=muR, beta=0.5)
    return Scene(**kw, pp=m, pt=m, pw=m, dt=dt, gravity=(0.0, 0.0, -9.81), gravity_enabled=1, wall_origin=wo,
                 wall_normal=wn, name=name)


def clumps(n_owners=216, seed=5, dt=1e-5, rc=1.0e-3, vel_std=1e-5, omega_std=0.01, overlap=5e-9, name="clumps"):
    """A pile of rigid multi-sphere owners (clumps) of 1 to 8 components in a
    walled box, for tests of the clump path (src/cuda_backend_cuda.cu:121-190,
    src/particle.cpp:170-278).  Each owner's components sit on random
    directions at 0 to 1.2 component radii from the owner's mass centre
    (body frame), so they overlap one another; component ids are unique and
    the components are listed in shuffled order.  Owners are dropped one by
    one (unrotated) at random (x, y) onto the floor or the owners below and
    stop where a component first touches, overlapping by ``overlap``, so
    every owner rests on something from the first step; small random
    velocities and spins and anisotropic principal inertia exercise every
    history channel and the offset torques."""
    rng = np.random.default_rng(seed)
    width = 2.6 * rc * np.sqrt(n_owners / 6.0)
    comp_owner, comp_radius, comp_offset = [], [], []
    mass, inertia, radius, pos = [], [], [], []
    placed_p = np.zeros((0, 3))
    placed_r = np.zeros(0)
    for i in range(n_owners):
        k = int(rng.integers(1, 9))
        d = rng.normal(size=(k, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        off = d * rng.uniform(0.0, 1.2 * rc, size=(k, 1))
        rr = rng.uniform(0.8 * rc, 1.2 * rc, size=k)
        mk = DENSITY * 4.0 / 3.0 * np.pi * rr ** 3
        m = float(mk.sum())
        off = off - (mk[:, None] * off).sum(0) / m        # offsets about the owner's mass centre
        I = np.zeros(3)
        for a in range(3):
            b, cc = (a + 1) % 3, (a + 2) % 3
            I[a] = float((mk * (0.4 * rr ** 2 + off[:, b] ** 2 + off[:, cc] ** 2)).sum())
        xy = rng.uniform(-width / 2, width / 2, size=2)
        cxy = xy[None, :] + off[:, :2]
        z = float((rr - off[:, 2]).max())                 # resting on the floor
        if len(placed_r):
            h2 = ((cxy[:, None, :] - placed_p[None, :, :2]) ** 2).sum(-1)
            s2 = (rr[:, None] + placed_r[None, :]) ** 2
            touch = h2 < s2
            if touch.any():
                zc = placed_p[None, :, 2] + np.sqrt(np.where(touch, s2 - h2, 0.0)) - off[:, 2:3]
                z = max(z, float(zc[touch].max()))
        z -= overlap
        centre = np.array([xy[0], xy[1], z])
        placed_p = np.concatenate([placed_p, centre + off])
        placed_r = np.concatenate([placed_r, rr])
        comp_owner += [i] * k
        comp_radius += rr.tolist()
        comp_offset += off.tolist()
        mass.append(m)
        inertia.append(I)
        radius.append(float((np.linalg.norm(off, axis=1) + rr).max()))
        pos.append(centre)
    own = np.array(comp_owner)
    nc = len(own)
    kw = dict(owner_id=np.arange(n_owners, dtype=np.int32) * 3 + 1,
              owner_status=np.zeros(n_owners, np.int32), owner_mass=np.array(mass),
              owner_radius=np.array(radius), owner_inertia=np.array(inertia), pos=np.array(pos),
              vel=rng.normal(0, vel_std, size=(n_owners, 3)), omega=rng.normal(0, omega_std, size=(n_owners, 3)),
              quat=np.tile([1.0, 0.0, 0.0, 0.0], (n_owners, 1)))
    perm = rng.permutation(nc)                            # input order need not be owner order
    ids = rng.permutation(nc).astype(np.int32) + 100
    span = width / 2 + 3 * rc
    wo, wn = box_walls([-span, -span, 0.0], [span, span, 0.2])
    m = mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=0.1, muR=0.05, beta=0.5)
    return Scene(**kw, comp_owner=own.astype(np.int32)[perm], comp_id=ids,
                 comp_radius=np.array(comp_radius)[perm], comp_offset=np.array(comp_offset)[perm],
                 pp=m, pt=m, pw=m, dt=dt, gravity=(0.0, 0.0, -9.81), gravity_enabled=1, wall_origin=wo,
                 wall_normal=wn, name=name)


def universal_gravity(n=2000, seed=9, dt=1e-5, name="universal_gravity"):
    """Spheres in a loose cloud with mutual gravitation on
    (CONTROL universal gravitation, src/cuda/cuda_contact_backend.cu:1095-1106)
    and a few contacts, no walls.  The density is 1e9 kg/m^3 so the pairwise
    attraction (constant 6.674e-11) is about 1% of the contact forces, well
    above their rounding."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(n ** (1 / 3)))
    pitch = 4.1e-3
    idx = np.stack(np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 3)[:n]
    pos = idx * pitch + rng.uniform(-0.1e-3, 0.1e-3, size=(n, 3))
    rad = rng.uniform(1.8e-3, 2.1e-3, size=n)
    kw = make_spheres(pos, rad, 1e9, vel=rng.normal(0, 0.01, size=(n, 3)))
    kw["omega"] = rng.normal(0, 5.0, size=(n, 3))
    m = mech(kN=1e5, epsN=0.5, epsS=0.6, mu=0.4, muT=0.1, muR=0.05, beta=0.5)
    return Scene(**kw, pp=m, pt=m, pw=m, dt=dt, gravity=(0.0, 0.0, 0.0), gravity_enabled=0,
                 universal_gravity_enabled=1, name=name)
