"""The particle object of ``CLASSES/Particle_class.py``: state vectors, convex-hull geometry and the
host-side movers that sync it with the simulator's accumulated rotation/translation.

Same attribute names, makers and movers as the reference (``Particle_class.py:9-628``), so scene
scripts written against it run unchanged; the makers draw from numpy's global RNG in the same
order as the reference's, so a seeded script builds the same shapes.  Hull construction, centring
and inertia are shared with ``mwdiem_gb300.shapes``.  ``to_body()`` hands the shape to the
device-resident simulator.
"""
from __future__ import annotations

import math

import numpy as np

from . import shapes


def _qmul(a, b):
    u, v = np.asarray(a[1:], float), np.asarray(b[1:], float)
    s = a[0] * v + b[0] * u + np.cross(u, v)
    return np.array([a[0] * b[0] - np.dot(u, v), s[0], s[1], s[2]])


def _qinv(q):
    return np.array([q[0], -q[1], -q[2], -q[3]], dtype=float)


def _qrot(q, v):
    """q (0,v) q^-1, vector part (LIBRARY_Quaternion.Quat_triple_prod with the inverse)."""
    return _qmul(q, _qmul(np.array([0.0, v[0], v[1], v[2]]), _qinv(q)))[1:]


class Particle(object):
    def __init__(self, particle_id):
        self.particle_id = particle_id
        z = lambda: np.array([0, 0, 0])  # noqa: E731
        self.velocity, self.velocity_12 = z(), z()
        self.force_normal, self.force_n_spring, self.force_n_damping, self.force_external = z(), z(), z(), z()
        self.torque, self.torque_bf, self.torque_external = z(), z(), z()
        self.angular_velocity_bf, self.angular_velocity_12_bf = z(), z()
        self.angular_velocity, self.angular_velocity_12 = z(), z()
        self.angular_acceleration_bf = z()
        self.quaternion = np.array([1, 0, 0, 0])
        self.quaternion_12 = np.array([1, 0, 0, 0])
        self.quaternion_all = np.array([1, 0, 0, 0])
        self.dx_all = z()

    # ------------------------------------------------------------------ geometry records
    class Vertex:
        def __init__(self, vertex_id, hull):
            self.vertex_id = vertex_id
            self.vertex_id_old = hull.vertices[vertex_id]
            self.vertex_coo = np.array(hull.points[self.vertex_id_old][:3], dtype=float)
            self.vertex_edges_id = []
            self.vertex_faces_id = []

    class Face:
        def __init__(self, face_id, hull, center_of_mass, vertex):
            self.face_id = face_id
            simplex = hull.simplices[face_id]
            self.face_num_vertices = len(simplex)
            self.face_vertices = np.array([hull.points[k] for k in simplex], dtype=float)
            old = {v.vertex_id_old: j for j, v in enumerate(vertex)}
            self.face_vertices_id = np.array([old[k] for k in simplex])
            a, b, c = self.face_vertices[0], self.face_vertices[1], self.face_vertices[2]
            n = np.cross(b - a, c - b)
            n = n / math.sqrt(n @ n)
            if np.dot(n, a - center_of_mass) < 0:
                n = -n
            self.face_normal = n

    def _from_points(self, points):
        from scipy.spatial import ConvexHull
        hull = ConvexHull(points)
        self.num_vertices = len(hull.vertices)
        self.num_faces = len(hull.simplices)
        self.num_edges = self.num_vertices + self.num_faces - 2
        self.volume = hull.volume
        self.vertices = [self.Vertex(i, hull) for i in range(self.num_vertices)]
        self.center_of_mass = sum(v.vertex_coo for v in self.vertices) / self.num_vertices
        self.faces = [self.Face(i, hull, self.center_of_mass, self.vertices) for i in range(self.num_faces)]

    def _finish(self, density, typee, acc_ext_def, torq_ext_def, diag=True):
        self.density = density
        self.moment_of_inertia, self.moment_of_inertia_size = self.Calc_inertia(density)
        if diag:
            self.eig = np.linalg.eig(self.moment_of_inertia)
            self.moment_of_inertia_bf = np.array([[self.eig[0][0], 0, 0], [0, self.eig[0][1], 0],
                                                  [0, 0, self.eig[0][2]]])
            self.moment_of_inertia_bf_inv = np.linalg.inv(self.moment_of_inertia_bf)
        self.mass = self.density * self.volume
        self.typee = typee
        self.force_external = self.mass * np.asarray(acc_ext_def)
        self.torque_external = torq_ext_def
        self.normvec = np.array([0, 0, 1])

    def Calc_inertia(self, density):
        """Dobrovolskis' polyhedron inertia over the faces (Particle_class.py:125-156)."""
        pts = np.array([v.vertex_coo for v in self.vertices])
        faces = np.array([f.face_vertices_id for f in self.faces])
        normals = np.array([f.face_normal for f in self.faces])
        I = shapes.inertia_tensor(pts, faces, normals, density)
        if not np.isfinite(np.linalg.cond(I)):
            print(I)
            print("Singular matrix, ohoh!")
        return I, 1 / 3 * (I[0, 0] + I[1, 1] + I[2, 2])

    # ------------------------------------------------------------------ makers
    def Spherical_convex_polygon_maker_3D(self, num_vertices_min, num_vertices_max, radius, variation, density, typee,
                                          acc_ext_def, torq_ext_def):
        n = np.random.randint(num_vertices_min, num_vertices_max)
        r = np.random.normal(radius, variation)
        fi = np.random.rand(n) * 180 * math.pi / 180
        teta = np.random.rand(n) * 360 * 0.9999999999999 * math.pi / 180
        pts = np.stack([r * np.sin(fi) * np.cos(teta), r * np.sin(fi) * np.sin(teta), r * np.cos(fi)], 1)
        self._from_points(pts)
        self.Translate(-self.center_of_mass)
        self._finish(density, typee, acc_ext_def, torq_ext_def)

    def Random_convex_polygon_maker_3D(self, num_vertices_min, num_vertices_max, min_radius, max_radius,
                                       density=1.0):
        n = np.random.randint(num_vertices_min, num_vertices_max)
        size = max_radius * 2
        np.random.randint(min_radius, max_radius)
        np.random.rand()
        np.random.rand(n)
        np.random.rand(n)
        pts = np.random.rand(n, 3) * size
        self._from_points(pts)
        self._finish(density, 0, np.zeros(3), np.zeros(3), diag=False)

    def Cube_maker_3D(self, side_length, density, typee, acc_ext_def, torq_ext_def):
        s = side_length
        pts = np.array([[x, y, z] for z in (0, s) for y in (0, s) for x in (0, s)], dtype=float)
        pts = pts[[0, 1, 2, 3, 4, 5, 6, 7]]
        self._from_points(pts)
        self.quaternion = [1, 0, 0, 0]
        self.Translate(-self.center_of_mass)
        self._finish(density, typee, acc_ext_def, torq_ext_def)

    def Plane_maker_3D(self, size_plane_x, size_plane_y, size_plane_z, density, max_particlesize, typee, acc_ext_def,
                       torq_ext_def):
        hx, hy, hz = size_plane_x / 2, size_plane_y / 2, size_plane_z / 2
        pts = np.array([[sx * hx, sy * hy, sz * hz] for sx in (1, -1) for sy in (1, -1) for sz in (1, -1)])
        self._from_points(pts)
        self._finish(density, typee, acc_ext_def, torq_ext_def)
        self.maxsize = math.sqrt(math.sqrt(size_plane_x ** 2 / 4 + size_plane_y ** 2 / 4) + size_plane_z ** 2 / 4)

    # ------------------------------------------------------------------ movers
    def Translate(self, transl):
        t = np.asarray(transl, dtype=float)
        for v in self.vertices:
            v.vertex_coo = v.vertex_coo + t
        self.center_of_mass = np.asarray(self.center_of_mass, dtype=float) + t
        for f in self.faces:
            f.face_vertices = f.face_vertices + t

    def Translate_wall(self, transl):
        t = np.asarray(transl, dtype=float)
        for v in self.vertices:
            v.vertex_coo = v.vertex_coo + t
        self.center_of_mass = np.asarray(self.center_of_mass, dtype=float) + t

    def Particles_to_cells_hash(self, cellsize_x, cellsize_y, cellsize_z, numcells_x, numcells_y):
        self.xc = int(self.center_of_mass[0] / cellsize_x)
        self.yc = int(self.center_of_mass[1] / cellsize_y)
        self.zc = int(self.center_of_mass[2] / cellsize_z)
        self.hashh = self.xc + self.yc * numcells_x + self.zc * numcells_x * numcells_y

    def Rotator_quaternion_initial(self, angle_deg, axis):
        """Rodrigues rotation about `axis` through the centre (Particle_class.py:523-536)."""
        ang = angle_deg * np.pi / 180
        axis = np.asarray(axis, dtype=float)

        def rot(v):
            return v * np.cos(ang) + np.cross(axis, v) * np.sin(ang) + np.dot(v, axis) * (1 - np.cos(ang)) * axis
        c = np.asarray(self.center_of_mass, dtype=float)
        for v in self.vertices:
            v.vertex_coo = rot(v.vertex_coo - c) + c
        for f in self.faces:
            f.face_vertices = np.array([rot(p - c) + c for p in f.face_vertices])
            f.face_normal = rot(f.face_normal)
        self.normvec = rot(self.normvec)

    def Rotator_quaternion(self, quaternion):
        c = np.asarray(self.center_of_mass, dtype=float)
        for v in self.vertices:
            v.vertex_coo = _qrot(quaternion, v.vertex_coo - c) + c

    def Rotator_quaternion_all(self):
        """Apply the accumulated rotation quaternion_all, then reset it (Particle_class.py:552-564)."""
        c = np.asarray(self.center_of_mass, dtype=float)
        q = np.asarray(self.quaternion_all, dtype=float)
        for v in self.vertices:
            v.vertex_coo = _qrot(q, v.vertex_coo - c) + c
        for f in self.faces:
            f.face_vertices = np.array([_qrot(q, p - c) + c for p in f.face_vertices])
            f.face_normal = _qrot(q, f.face_normal)
        self.quaternion_all = np.array([1, 0, 0, 0])

    def Translate_all(self):
        """Apply the accumulated translation dx_all, then reset it (Particle_class.py:567-590)."""
        self.Translate(self.dx_all)
        self.dx_all = np.array([0, 0, 0])

    # ------------------------------------------------------------------ bridge to the simulator
    def to_body(self):
        """Body-frame description for mwdiem_gb300.sim (vertices relative to the centre)."""
        from .scene import Body
        c = np.asarray(self.center_of_mass, dtype=float)
        verts = np.array([v.vertex_coo for v in self.vertices]) - c
        eig = np.real(np.diag(self.moment_of_inertia_bf)) if hasattr(self, "moment_of_inertia_bf") else \
            np.real(np.linalg.eig(self.moment_of_inertia)[0])
        return Body(vertices=verts, inertia_bf=np.asarray(eig, dtype=float),
                    inertia_size=float(self.moment_of_inertia_size), mass=float(self.mass))
