"""Convex polyhedron shapes: vertices, faces, volume, mass and inertia.

Host-side set-up code (runs once per scene).  The construction follows the reference's particle
makers:

* a shape is the convex hull (scipy's Qhull) of a point set; its vertices are listed in
  ``hull.vertices`` order and its faces are the hull's triangles (``CLASSES/Particle_class.py:62-115``);
* the shape is centred on the mean of its vertices, not on its volume centroid
  (``Particle_class.py:264-282``);
* the inertia tensor is the polyhedron formula of Dobrovolskis (Icarus 124, 1996), summed over the
  triangles with outward normals (``Particle_class.py:125-156``);
* the body-frame inertia is the diagonal of the tensor's eigenvalues as ``np.linalg.eig`` returns
  them, without rotating the vertices into the principal frame (``Particle_class.py:288-292``);
* ``moment_of_inertia_size`` is one third of the trace (``Particle_class.py:151``).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Shape:
    vertices: np.ndarray          # (n, 3) float64, centred on the vertex mean
    faces: np.ndarray             # (f, 3) int32, indices into vertices
    volume: float
    density: float
    inertia: np.ndarray           # (3, 3) tensor about the vertex mean
    inertia_bf: np.ndarray        # (3, 3) diag(eigenvalues)
    inertia_bf_inv: np.ndarray    # (3, 3)
    inertia_size: float           # trace / 3
    normal: np.ndarray = field(default_factory=lambda: np.array([0.0, 0.0, 1.0]))

    @property
    def mass(self) -> float:
        return self.density * self.volume

    @property
    def num_vertices(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def radius(self) -> float:
        return float(np.sqrt((self.vertices ** 2).sum(1)).max())


def _outward_faces(points, simplices, centre):
    faces = np.array(simplices, dtype=np.int64)
    normals = np.zeros((len(faces), 3))
    for i, f in enumerate(faces):
        a, b, c = points[f[0]], points[f[1]], points[f[2]]
        n = np.cross(b - a, c - b)
        n = n / np.sqrt(n @ n)
        if np.dot(n, a - centre) < 0:
            n = -n
        normals[i] = n
    return faces, normals


def inertia_tensor(points, faces, normals, density):
    """Dobrovolskis' polyhedron inertia: per triangle (D, E, F) with outward unit normal n the
    signed tetrahedron volume is D.n/6 (apex at the origin) and the second moments follow the
    closed form for a tetrahedron with one vertex at the origin."""
    P = np.zeros((3, 3))
    for f, n in zip(faces, normals):
        D, E, F = points[f[0]], points[f[1]], points[f[2]]
        dv = np.dot(D, n) / 6.0
        for i in range(3):
            for j in range(3):
                P[i, j] += density * dv / 20.0 * (2 * D[i] * D[j] + 2 * E[i] * E[j] + 2 * F[i] * F[j]
                                                  + D[i] * E[j] + D[j] * E[i] + D[i] * F[j] + D[j] * F[i]
                                                  + E[i] * F[j] + E[j] * F[i])
    I = np.array([[P[1, 1] + P[2, 2], -P[0, 1], -P[0, 2]],
                  [-P[0, 1], P[0, 0] + P[2, 2], -P[1, 2]],
                  [-P[0, 2], -P[1, 2], P[0, 0] + P[1, 1]]])
    return I


def shape_from_points(points, density=1.0) -> Shape:
    from scipy.spatial import ConvexHull
    pts = np.asarray(points, dtype=np.float64)
    hull = ConvexHull(pts)
    verts = pts[hull.vertices]
    remap = {int(v): i for i, v in enumerate(hull.vertices)}
    simp = [[remap[int(a)] for a in s] for s in hull.simplices]
    centre = verts.mean(axis=0)
    verts = verts - centre
    faces, normals = _outward_faces(verts, simp, np.zeros(3))
    I = inertia_tensor(verts, faces, normals, density)
    eig = np.linalg.eig(I)[0]
    eig = np.real(eig)
    Ibf = np.diag(eig)
    return Shape(vertices=verts, faces=faces.astype(np.int32), volume=float(hull.volume), density=density,
                 inertia=I, inertia_bf=Ibf, inertia_bf_inv=np.linalg.inv(Ibf),
                 inertia_size=float(np.trace(I) / 3.0))


def random_hull(rng, n_min=12, n_max=32, r_min=0.8, r_max=1.2, density=1.0) -> Shape:
    """Hull of n ~ U{n_min..n_max} points uniform on a sphere of radius U[r_min, r_max]."""
    while True:
        n = int(rng.integers(n_min, n_max + 1))
        p = rng.normal(size=(n, 3))
        p /= np.sqrt((p ** 2).sum(1, keepdims=True))
        p *= rng.uniform(r_min, r_max)
        try:
            s = shape_from_points(p, density)
        except Exception:
            continue
        if s.num_vertices >= 4:
            return s


def cube(edge=1.0, density=1.0) -> Shape:
    """Unit-lattice cube like ``Particle_class.Cube_maker_3D`` (``Particle_class.py:305-370``)."""
    p = np.array([[x, y, z] for z in (0, edge) for y in (0, edge) for x in (0, edge)], dtype=np.float64)
    return shape_from_points(p, density)


def tetrahedron(edge=1.0, density=1.0) -> Shape:
    a = edge / np.sqrt(8.0)
    p = np.array([[a, a, a], [a, -a, -a], [-a, a, -a], [-a, -a, a]])
    return shape_from_points(p, density)


def slab(sx, sy, sz, density=1.0) -> Shape:
    """Box wall like ``Particle_class.Plane_maker_3D`` (``Particle_class.py:373-461``)."""
    p = np.array([[sx / 2 * i, sy / 2 * j, sz / 2 * k] for i in (1, -1) for j in (1, -1) for k in (1, -1)])
    return shape_from_points(p, density)


def quat_to_matrix(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def matrix_to_quat(R):
    """Unit quaternion (w, x, y, z), w >= 0, of a rotation matrix (Shepperd's method: the largest of
    the four squared components comes from the trace or a diagonal entry, the others from the
    off-diagonal sums and differences)."""
    R = np.asarray(R, dtype=np.float64)
    t = np.trace(R)
    k = int(np.argmax([t, R[0, 0], R[1, 1], R[2, 2]]))
    if k == 0:
        w = 0.5 * np.sqrt(1.0 + t)
        s = 0.25 / w
        q = [w, (R[2, 1] - R[1, 2]) * s, (R[0, 2] - R[2, 0]) * s, (R[1, 0] - R[0, 1]) * s]
    elif k == 1:
        x = 0.5 * np.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2])
        s = 0.25 / x
        q = [(R[2, 1] - R[1, 2]) * s, x, (R[0, 1] + R[1, 0]) * s, (R[0, 2] + R[2, 0]) * s]
    elif k == 2:
        y = 0.5 * np.sqrt(1.0 - R[0, 0] + R[1, 1] - R[2, 2])
        s = 0.25 / y
        q = [(R[0, 2] - R[2, 0]) * s, (R[0, 1] + R[1, 0]) * s, y, (R[1, 2] + R[2, 1]) * s]
    else:
        z = 0.5 * np.sqrt(1.0 - R[0, 0] - R[1, 1] + R[2, 2])
        s = 0.25 / z
        q = [(R[1, 0] - R[0, 1]) * s, (R[0, 2] + R[2, 0]) * s, (R[1, 2] + R[2, 1]) * s, z]
    q = np.asarray(q)
    q = q / np.sqrt(q @ q)
    return q if q[0] >= 0 else -q


def quat_mul(a, b):
    """Hamilton product a b of quaternions (w, x, y, z): R(a b) = R(a) R(b)."""
    aw, av = a[0], np.asarray(a[1:])
    bw, bv = b[0], np.asarray(b[1:])
    v = aw * bv + bw * av + np.cross(av, bv)
    return np.concatenate([[aw * bw - av @ bv], v])


def hull_inertia(vertices, mass):
    """Inertia tensor, about the origin of ``vertices`` (the body centre), of their convex hull
    carrying ``mass`` uniformly (the closed form of ``inertia_tensor``)."""
    from scipy.spatial import ConvexHull
    v = np.asarray(vertices, dtype=np.float64)
    h = ConvexHull(v)
    faces, normals = _outward_faces(v, h.simplices, v[h.vertices].mean(axis=0))
    return inertia_tensor(v, faces, normals, mass / h.volume)


def principal_frame(vertices, mass):
    """(r_p, moments, q0): the vertices expressed in the principal axes of the hull's inertia, the
    principal moments, and the orientation q0 with R(q0) r_p = vertices."""
    I = hull_inertia(vertices, mass)
    lam, P = np.linalg.eigh(I)
    if np.linalg.det(P) < 0:
        P[:, 2] = -P[:, 2]
    return np.ascontiguousarray(np.asarray(vertices, dtype=np.float64) @ P), lam, matrix_to_quat(P)


def random_quaternion(rng):
    q = rng.normal(size=4)
    return q / np.sqrt(q @ q)
