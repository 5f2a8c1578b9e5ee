"""Particle_class against the reference's own CLASSES/Particle_class.py: a seeded sequence of shape
makers builds the same vertices, faces, inertia and mass (numpy's global RNG drawn in the same
order).  Skipped without the reference checkout; the hull/inertia code it exercises is also covered
by the golden fixtures through the simulator tests."""
import sys

import numpy as np
import pytest

import oracle

ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not present")


def _reference_class():
    import build_ref
    for sub in ("CLASSES", "LIBRARIES"):
        p = str(build_ref.REFERENCE_ROOT / sub)
        if p not in sys.path:
            sys.path.insert(0, p)
    import Particle_class as RP
    return RP.Particle


@ref
def test_makers_match_reference():
    from mwdiem_gb300.Particle_class import Particle
    RefParticle = _reference_class()
    acc = np.array([0.0, 0.0, -9.81])
    for seed in range(5):
        out = []
        for cls in (Particle, RefParticle):
            np.random.seed(seed)
            ps = []
            for k in range(3):
                p = cls(k)
                p.Spherical_convex_polygon_maker_3D(12, 30, 1.0, 0.1, 2.5, 1, acc, np.zeros(3))
                ps.append(p)
            c = cls(9)
            c.Cube_maker_3D(1.0, 1.0, 1, acc, np.zeros(3))
            w = cls(10)
            w.Plane_maker_3D(40.0, 30.0, 24.0, 1.0, 2.4, 0, acc, np.zeros(3))
            w.Rotator_quaternion_initial(90, np.array([1.0, 0, 0]))
            ps += [c, w]
            out.append(ps)
        for a, b in zip(*out):
            va = np.array([v.vertex_coo for v in a.vertices])
            vb = np.array([v.vertex_coo for v in b.vertices])
            assert np.allclose(va, vb, rtol=0, atol=1e-12)
            assert np.allclose(a.moment_of_inertia, b.moment_of_inertia, rtol=1e-12, atol=1e-12)
            assert abs(a.moment_of_inertia_size - b.moment_of_inertia_size) <= 1e-12 * abs(b.moment_of_inertia_size)
            assert abs(a.mass - b.mass) <= 1e-12 * b.mass
            assert np.allclose(a.normvec, b.normvec, atol=1e-12)
            fa = np.array([f.face_vertices_id for f in a.faces])
            fb = np.array([f.face_vertices_id for f in b.faces])
            assert np.array_equal(fa, fb)


@ref
def test_sync_movers_match_reference():
    from mwdiem_gb300.Particle_class import Particle
    RefParticle = _reference_class()
    acc = np.zeros(3)
    res = []
    for cls in (Particle, RefParticle):
        np.random.seed(3)
        p = cls(0)
        p.Spherical_convex_polygon_maker_3D(12, 30, 1.0, 0.1, 2.5, 1, acc, np.zeros(3))
        p.quaternion_all = np.array([0.9, 0.1, -0.3, 0.2]) / np.linalg.norm([0.9, 0.1, -0.3, 0.2])
        p.dx_all = np.array([0.5, -0.25, 1.0])
        p.Rotator_quaternion_all()
        p.Translate_all()
        p.Particles_to_cells_hash(0.7, 0.8, 0.9, 11, 13)
        res.append((np.array([v.vertex_coo for v in p.vertices]), np.array(p.center_of_mass), p.hashh))
    assert np.allclose(res[0][0], res[1][0], atol=1e-12)
    assert np.allclose(res[0][1], res[1][1], atol=1e-12)
    assert res[0][2] == res[1][2]


def test_force_legacy_interface():
    from mwdiem_gb300.LIBRARY_Force import Force

    class P:
        def __init__(self, c, v):
            self.center_of_mass = np.array(c, float)
            self.velocity = np.array(v, float)
    A, B = P([0, 0, 0], [1, 0.5, 0]), P([1, 0, 0], [0, 0, 0])
    Fn, Fs, Fd, TA, TB = Force(A, B, 0.04, np.array([1.0, 0, 0]), [0.5, 0.1, 0], [0.5, -0.1, 0], 1e4, 10.0, 0.3)
    assert np.allclose(Fs, [-1e4 * 0.04 ** 1.5, 0, 0])
    assert np.allclose(Fd, [-10.0 * 0.2 * 1.0, 0, 0])
    assert Fn[0] < 0 and np.linalg.norm(TA) > 0 and np.linalg.norm(TB) > 0
