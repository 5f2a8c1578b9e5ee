"""Synthetic scenes for the device-resident simulator.

A scene is a box of walls (thick slabs, like the reference's ``Plane_maker_3D`` walls,
``MWDiem.py:143-537``) plus convex particles.  Rows are ordered walls first, then particles, as in
the reference (``MWDiem.py:403-408``: ids below ``num_particles_wall`` are walls).  The cell grid
and the fly-away box follow ``MWDiem.py:549-580``: the box is the bounding box of the wall
vertices, ``numcells = int(extent / max_particlesize)``, ``cellsize = extent / numcells``.

Initial orientations are baked into the vertices and every quaternion starts at identity, as the
reference does (``MWDiem.py:622-629``).  The contact configs name a damping ratio zeta; the reference
takes a restitution coefficient, mapped as ``en = exp(-pi zeta / sqrt(1 - zeta^2))`` (which inverts
the reference's ``Gn = -2 m ln(en) / tc``), with ``et = en``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import shapes

G = 9.81


def restitution_from_damping(zeta: float) -> float:
    return math.exp(-math.pi * zeta / math.sqrt(1.0 - zeta * zeta))


@dataclass
class Body:
    vertices: np.ndarray      # (n,3) body-frame offsets from the centre (orientation baked in)
    inertia_bf: np.ndarray    # (3,) principal moments (diag of the reference's eig)
    inertia_size: float
    mass: float


@dataclass
class CompactBodies:
    """Particles drawn from a pool of shapes: particle k is pool[pick[k]] rotated by quats[k]
    (orientation baked into its vertices, quaternion state starting at identity).  Builds large
    scenes without one Python object per particle."""
    pool: list
    pick: np.ndarray
    quats: np.ndarray

    def __len__(self):
        return int(len(self.pick))

    def expand(self):
        out = []
        for k in range(len(self.pick)):
            b = self.pool[int(self.pick[k])]
            out.append(Body(vertices=b.vertices @ shapes.quat_to_matrix(self.quats[k]).T, inertia_bf=b.inertia_bf,
                            inertia_size=b.inertia_size, mass=b.mass))
        return out


@dataclass
class SceneSpec:
    """Host description of one scene (rows: walls, then particles)."""
    walls: list = field(default_factory=list)          # list of (Body, centre (3,), normal (3,))
    bodies: list = field(default_factory=list)         # list of Body
    centres: np.ndarray = None                         # (n_particles, 3)
    velocities: np.ndarray = None                      # (n_particles, 3) initial v = v_1/2
    Kn: float = 1e5
    en: float = 0.372
    et: float = 0.372
    mu: float = 0.5
    Kn_wall: float = 1e5
    en_wall: float = 0.372
    et_wall: float = 0.372
    mu_wall: float = 0.5
    dt: float = 5e-5
    gravity: tuple = (0.0, 0.0, -G)
    max_particlesize: float = 2.4
    name: str = "scene"
    law: str = "reference"   # contact law: "reference" (as the reference computes it) or "physical"

    @property
    def n_walls(self) -> int:
        return len(self.walls)

    @property
    def n_particles(self) -> int:
        return len(self.bodies)

    def body_list(self):
        return self.bodies.expand() if isinstance(self.bodies, CompactBodies) else list(self.bodies)

    def principal_bodies(self):
        """The particles re-expressed in the principal axes of their inertia, as the physical contact
        law integrates them: (bodies, q0) where bodies holds the same shapes with body-frame vertices
        r_p along the principal axes and diagonal moments, and q0 (n_particles, 4) is each particle's
        starting orientation, R(q0) r_p = its world-oriented vertices.  (The reference keeps the
        world-oriented vertices as the body frame and takes the eigenvalues of the inertia tensor as
        body-frame moments, Particle_class.py:125-156, which is exact only for shapes whose principal
        axes lie along x, y, z.)"""
        cb = self.bodies
        if isinstance(cb, CompactBodies):
            pool, qp = [], []
            for b in cb.pool:
                r, lam, q = shapes.principal_frame(b.vertices, b.mass)
                pool.append(Body(vertices=r, inertia_bf=lam, inertia_size=b.inertia_size, mass=b.mass))
                qp.append(q)
            pick = np.asarray(cb.pick, dtype=np.int64)
            quats = np.asarray(cb.quats, dtype=np.float64)
            q0 = np.array([shapes.quat_mul(quats[k], qp[pick[k]]) for k in range(len(pick))]).reshape(-1, 4)
            ident = np.tile([1.0, 0.0, 0.0, 0.0], (len(pick), 1))
            return CompactBodies(pool=pool, pick=pick, quats=ident), q0
        out, q0 = [], []
        for b in cb:
            r, lam, q = shapes.principal_frame(b.vertices, b.mass)
            out.append(Body(vertices=r, inertia_bf=lam, inertia_size=b.inertia_size, mass=b.mass))
            q0.append(q)
        return out, np.array(q0).reshape(-1, 4)

    def wall_bbox(self):
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        for b, c, _ in self.walls:
            v = b.vertices + c
            lo = np.minimum(lo, v.min(0))
            hi = np.maximum(hi, v.max(0))
        return lo, hi

    def grid(self):
        """numcells, cellsize per axis (MWDiem.py:575-580)."""
        lo, hi = self.wall_bbox()
        ext = hi - lo
        n = np.array([int(e / self.max_particlesize) for e in ext], dtype=np.int64)
        n = np.maximum(n, 1)
        return n, ext / n

    def box(self):
        lo, hi = self.wall_bbox()
        return (hi[0], lo[0], hi[1], lo[1], hi[2], lo[2])


def body_from_shape(s: shapes.Shape, q=None) -> Body:
    v = s.vertices if q is None else s.vertices @ shapes.quat_to_matrix(q).T
    return Body(vertices=np.ascontiguousarray(v), inertia_bf=np.real(np.diag(s.inertia_bf)).copy(),
                inertia_size=float(s.inertia_size), mass=float(s.mass))


def fast_hull_body(rng, n_min, n_max, r_min, r_max, density=1.0):
    """Hull of n ~ U{n_min..n_max} points uniform on a sphere of radius U[r_min, r_max]; vectorised
    inertia (same closed form as shapes.inertia_tensor)."""
    from scipy.spatial import ConvexHull
    while True:
        n = int(rng.integers(n_min, n_max + 1))
        p = rng.normal(size=(n, 3))
        p /= np.sqrt((p ** 2).sum(1, keepdims=True))
        p *= rng.uniform(r_min, r_max)
        try:
            h = ConvexHull(p)
        except Exception:
            continue
        verts = p[h.vertices]
        remap = np.full(n, -1)
        remap[h.vertices] = np.arange(len(h.vertices))
        faces = remap[h.simplices]
        c = verts.mean(0)
        verts = verts - c
        D, E, F = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
        nrm = np.cross(E - D, F - E)
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        flip = (nrm * D).sum(1) < 0
        nrm[flip] *= -1
        dv = (D * nrm).sum(1) / 6.0
        P = np.zeros((3, 3))
        for i in range(3):
            for j in range(3):
                P[i, j] = (density * dv / 20.0 * (2 * D[:, i] * D[:, j] + 2 * E[:, i] * E[:, j] + 2 * F[:, i] * F[:, j]
                                                  + D[:, i] * E[:, j] + D[:, j] * E[:, i] + D[:, i] * F[:, j]
                                                  + D[:, j] * F[:, i] + E[:, i] * F[:, j] + E[:, j] * F[:, i])).sum()
        I = np.array([[P[1, 1] + P[2, 2], -P[0, 1], -P[0, 2]], [-P[0, 1], P[0, 0] + P[2, 2], -P[1, 2]],
                      [-P[0, 2], -P[1, 2], P[0, 0] + P[1, 1]]])
        eig = np.real(np.linalg.eig(I)[0])
        if verts.shape[0] < 4 or np.any(eig <= 0):
            continue
        return Body(vertices=np.ascontiguousarray(verts), inertia_bf=eig, inertia_size=float(np.trace(I) / 3),
                    mass=float(density * h.volume))


def box_walls(inner_x, inner_y, height, thickness, density=1.0):
    """Floor (top face at z = 0) and four side walls around [-inner_x/2, inner_x/2] x [-inner_y/2, inner_y/2]."""
    t = thickness
    out = []
    floor = shapes.slab(inner_x + 2 * t, inner_y + 2 * t, t, density)
    out.append((body_from_shape(floor), np.array([0.0, 0.0, -t / 2]), np.array([0.0, 0.0, 1.0])))
    for sgn in (1, -1):
        w = shapes.slab(t, inner_y + 2 * t, height, density)
        out.append((body_from_shape(w), np.array([sgn * (inner_x / 2 + t / 2), 0.0, height / 2]),
                    np.array([1.0, 0.0, 0.0])))
    for sgn in (1, -1):
        w = shapes.slab(inner_x, t, height, density)
        out.append((body_from_shape(w), np.array([0.0, sgn * (inner_y / 2 + t / 2), height / 2]),
                    np.array([0.0, 1.0, 0.0])))
    return out


def lattice(n, inner_x, inner_y, spacing, jitter, rng, z0=None):
    nx = max(1, int(inner_x // spacing))
    ny = max(1, int(inner_y // spacing))
    per_layer = nx * ny
    layers = (n + per_layer - 1) // per_layer
    idx = np.arange(n)
    k, r = idx // per_layer, idx % per_layer
    i, j = r % nx, r // nx
    x = -inner_x / 2 + spacing / 2 + i * spacing
    y = -inner_y / 2 + spacing / 2 + j * spacing
    z = (z0 if z0 is not None else spacing / 2) + k * spacing
    c = np.stack([x, y, z], 1).astype(np.float64)
    c += rng.uniform(-jitter, jitter, size=c.shape)
    return c, layers


def pour_walls(n, box=40.0, spacing=2.6, r_max=1.2, density=1.0):
    """Walls of the pour scene; they depend on the sizes only (height = lattice layers + margin)."""
    maxsize = 2 * r_max
    per_layer = max(1, int(box // spacing)) ** 2
    layers = (n + per_layer - 1) // per_layer
    height = float(spacing / 2 + layers * spacing + 2 * maxsize)
    return box_walls(box, box, height, 10 * maxsize, density)


def pour_scene(n=20000, seed=0, box=40.0, spacing=2.6, jitter=0.1, n_min=12, n_max=32, r_min=0.8, r_max=1.2,
               zeta=0.3, kn=1e5, mu=0.5, dt=5e-5, density=1.0, pool=None, name="pour"):
    """Random hulls on a jittered lattice in a box, random orientations, at rest, under gravity."""
    rng = np.random.default_rng(seed)
    en = restitution_from_damping(zeta)
    maxsize = 2 * r_max
    centres, layers = lattice(n, box, box, spacing, jitter, rng)
    walls = pour_walls(n, box, spacing, r_max, density)
    if pool:
        base = [fast_hull_body(rng, n_min, n_max, r_min, r_max, density) for _ in range(pool)]
        pick = rng.integers(pool, size=n)
        bodies = []
        for k in range(n):
            b = base[pick[k]]
            q = shapes.random_quaternion(rng)
            bodies.append(Body(vertices=b.vertices @ shapes.quat_to_matrix(q).T, inertia_bf=b.inertia_bf,
                               inertia_size=b.inertia_size, mass=b.mass))
    else:
        bodies = []
        for k in range(n):
            b = fast_hull_body(rng, n_min, n_max, r_min, r_max, density)
            q = shapes.random_quaternion(rng)
            b.vertices = np.ascontiguousarray(b.vertices @ shapes.quat_to_matrix(q).T)
            bodies.append(b)
    return SceneSpec(walls=walls, bodies=bodies, centres=centres, velocities=np.zeros((n, 3)), Kn=kn, en=en,
                     et=en, mu=mu, Kn_wall=kn, en_wall=en, et_wall=en, mu_wall=mu, dt=dt, max_particlesize=maxsize,
                     name=name)


def packed_scene(n=16, seed=0, box=8.0, spacing=2.2, z0=1.0, jitter=0.05, vel=0.5, n_min=12, n_max=32,
                 r_min=0.8, r_max=1.2, zeta=0.3, kn=1e5, mu=0.5, dt=5e-5, density=1.0, name="packed"):
    """Random hulls on a lattice closer than their diameters (neighbours and the floor overlap from
    the first step), random orientations and velocities: a small scene whose contacts are active
    from step 0 (the differentiable step's finite-difference case)."""
    rng = np.random.default_rng(seed)
    en = restitution_from_damping(zeta)
    centres, layers = lattice(n, box, box, spacing, jitter, rng, z0=z0)
    height = float(z0 + layers * spacing + 4 * r_max)
    walls = box_walls(box, box, height, 20 * r_max, density)
    bodies = []
    for _ in range(n):
        b = fast_hull_body(rng, n_min, n_max, r_min, r_max, density)
        q = shapes.random_quaternion(rng)
        b.vertices = np.ascontiguousarray(b.vertices @ shapes.quat_to_matrix(q).T)
        bodies.append(b)
    v = rng.normal(size=(n, 3)) * vel
    return SceneSpec(walls=walls, bodies=bodies, centres=centres, velocities=v, Kn=kn, en=en, et=en, mu=mu,
                     Kn_wall=kn, en_wall=en, et_wall=en, mu_wall=mu, dt=dt, max_particlesize=2 * r_max, name=name)


def settling_scene(seed=0, n_side=5, edge=1.0, spacing=1.5, jitter=0.1, zeta=0.3, kn=1e5, mu=0.5, dt=1e-4,
                   floor=10.0):
    """125 unit cubes (density 1) on a 5x5x5 lattice, random orientations, onto a 10 x 10 floor."""
    rng = np.random.default_rng(seed)
    en = restitution_from_damping(zeta)
    cube = shapes.cube(edge)
    maxsize = float(2 * cube.radius)
    n = n_side ** 3
    idx = np.arange(n)
    i, j, k = idx % n_side, (idx // n_side) % n_side, idx // (n_side * n_side)
    off = (n_side - 1) * spacing / 2
    centres = np.stack([i * spacing - off, j * spacing - off, maxsize / 2 + 0.2 + k * spacing], 1).astype(float)
    centres += rng.uniform(-jitter, jitter, size=centres.shape)
    height = float(centres[:, 2].max() + 4 * maxsize)
    walls = box_walls(floor, floor, height, 10 * maxsize)
    bodies = [body_from_shape(cube, shapes.random_quaternion(rng)) for _ in range(n)]
    return SceneSpec(walls=walls, bodies=bodies, centres=centres, velocities=np.zeros((n, 3)), Kn=kn, en=en, et=en,
                     mu=mu, Kn_wall=kn, en_wall=en, et_wall=en, mu_wall=mu, dt=dt, max_particlesize=maxsize,
                     name="settling")


def mixed_shape_pool(rng, pool, r_min=0.8, r_max=1.2, n_min=12, n_max=32, density=1.0):
    """1/3 cubes, 1/3 regular tetrahedra, 1/3 random hulls, sizes matched to the hull radius range."""
    out = []
    for k in range(pool):
        kind = k % 3
        r = rng.uniform(r_min, r_max)
        if kind == 0:
            out.append(body_from_shape(shapes.cube(2 * r / math.sqrt(3), density)))
        elif kind == 1:
            out.append(body_from_shape(shapes.tetrahedron(2 * r * math.sqrt(8.0 / 3.0) / 2, density)))
        else:
            out.append(fast_hull_body(rng, n_min, n_max, r_min, r_max, density))
    return out


def batched_scenes(n_scenes=256, total=2_000_000, n_lo=100, n_hi=50_000, seed=0, pool=3072, dt=5e-5, zeta=0.3,
                   kn=1e5, mu=0.5, spacing=2.6, jitter=0.1):
    """Independent boxes with log-uniform particle counts in [n_lo, n_hi] (scaled to ~total)."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), size=n_scenes))
    counts = np.clip(np.round(counts * total / counts.sum()), n_lo, n_hi).astype(int)
    base = mixed_shape_pool(rng, pool)
    en = restitution_from_damping(zeta)
    scenes = []
    for s, n in enumerate(counts):
        side = max(8.0, spacing * math.ceil(math.sqrt(n / 40.0)))
        centres, _ = lattice(int(n), side, side, spacing, jitter, rng)
        height = float(centres[:, 2].max() + spacing + 4.8)
        walls = box_walls(side, side, height, 24.0)
        pick = rng.integers(len(base), size=int(n))
        q = rng.normal(size=(int(n), 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        bodies = CompactBodies(pool=base, pick=pick, quats=q)
        scenes.append(SceneSpec(walls=walls, bodies=bodies, centres=centres, velocities=np.zeros((int(n), 3)),
                                Kn=kn, en=en, et=en, mu=mu, Kn_wall=kn, en_wall=en, et_wall=en, mu_wall=mu, dt=dt,
                                max_particlesize=2.4, name=f"batch{s}"))
    return scenes


def reference_arrays(spec: SceneSpec, V=None, bodies=None, q0=None):
    """The state a scene gives the reference's per-step loop: its FP64 arrays (MWDiem.py:603-646),
    walls first, vertices in world coordinates padded with zeros to V, plus what the loop reads
    beside them.  `bodies`/`q0` replace the scene's bodies and starting orientations (the physical
    contact law's principal-axes frames).  Returns (state, aux): state holds v, v12, w12bf, wbf, w,
    F, T, com, dxall, q12, q, qall, verts, mass, Iinv, I; aux holds nv (vertex counts), Is
    (moment_of_inertia_size, Particle_class.py:151), ext (external force: gravity), wall_n, wall_c,
    wall_range (6 max_particlesize, MWDiem.py:808-811), the cell grid (nx, ny, cs) and the box."""
    W = spec.n_walls
    parts = spec.body_list() if bodies is None else list(bodies)
    all_bodies = [b for b, _, _ in spec.walls] + parts
    centres = np.concatenate([np.array([c for _, c, _ in spec.walls]).reshape(-1, 3), np.asarray(spec.centres)], 0)
    N = len(all_bodies)
    nv = np.array([b.vertices.shape[0] for b in all_bodies], dtype=np.int32)
    V = int(V or nv.max())
    verts = np.zeros((N, V, 3))
    for i, b in enumerate(all_bodies):
        verts[i, :nv[i]] = centres[i] + b.vertices
    mass = np.array([b.mass for b in all_bodies])
    I = np.zeros((N, 3, 3))
    Iinv = np.zeros((N, 3, 3))
    for i, b in enumerate(all_bodies):
        I[i] = np.diag(b.inertia_bf)
        Iinv[i] = np.diag(1.0 / np.asarray(b.inertia_bf))
    if q0 is None:
        q0 = np.tile([1.0, 0.0, 0.0, 0.0], (N, 1))

    def z():
        return np.zeros((N, 3))

    st = dict(v=z(), v12=z(), w12bf=z(), wbf=z(), w=z(), F=z(), T=z(), com=centres.copy(), dxall=z(),
              q12=q0.copy(), q=q0.copy(), qall=np.tile([1.0, 0.0, 0.0, 0.0], (N, 1)), verts=verts, mass=mass,
              Iinv=Iinv, I=I)
    if spec.velocities is not None:
        st["v"][W:] = spec.velocities
        st["v12"][W:] = spec.velocities
    ext = np.zeros((N, 3))
    ext[W:] = mass[W:, None] * np.asarray(spec.gravity)[None, :]
    ncell, cs = spec.grid()
    aux = dict(nv=nv, V=V, Is=np.array([b.inertia_size for b in all_bodies]), ext=ext,
               wall_n=np.array([n for _, _, n in spec.walls]).reshape(-1, 3), wall_c=centres[:W].copy(),
               wall_range=6.0 * spec.max_particlesize, nx=int(ncell[0]), ny=int(ncell[1]), cs=cs, box=spec.box(),
               W=W, N=N)
    return st, aux
