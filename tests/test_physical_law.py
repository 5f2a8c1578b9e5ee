"""The physical-mass contact law (an opt-in variant, not the reference's law) on the CPU side: the
oracle's restatement of it over a whole head-on impact, and the principal-axes body frames it
integrates in.  The device kernels are checked against this oracle in test_sim_gpu.py."""
import numpy as np

import stepper
from helpers import head_on_cubes
from mwdiem_gb300 import scene, shapes


def _rebound(law, steps=1500):
    sp = head_on_cubes(law)
    ref = stepper.RefStepper(sp)
    contact = 0
    for _ in range(steps):
        ref.step()
        contact += int(ref.last_collision is not None and (ref.last_collision == 1).any())
    W = sp.n_walls
    v = ref.st["v"][W:W + 2, 0]
    return -(v[0] - v[1]) / 1.0, contact, sp


def test_physical_law_rebounds_with_en():
    # linear spring-dashpot with the true effective mass m_n = 2: restitution en and contact time
    # tc = sqrt(m_n (pi^2 + ln^2 en) / Kn) (about 294 steps of 5e-5 s here)
    e, contact, sp = _rebound("physical")
    m_n = 2.0
    tc = np.sqrt(m_n * (np.pi ** 2 + np.log(sp.en) ** 2) / sp.Kn)
    print(f"physical: e {e:.4f} (en {sp.en:.4f}), contact steps {contact} (tc/dt {tc / sp.dt:.1f})")
    assert abs(e - sp.en) < 0.01
    assert abs(contact - tc / sp.dt) < 5


def test_reference_law_does_not():
    # the reference's law takes mu = 0.5 as the mass and turns the vertices by the whole orientation
    # every step: the same impact does not rebound with en
    e, _, sp = _rebound("reference")
    assert abs(e - sp.en) > 0.1


def test_principal_bodies_reproduce_the_scene():
    # explicit bodies and a shape pool: R(q0) r_p gives back each particle's vertices, and the inertia
    # of r_p is diagonal with the stated moments
    sp = scene.pour_scene(n=60, seed=5, box=16.0, spacing=2.45, pool=12)
    rng = np.random.default_rng(2)
    pool = [scene.fast_hull_body(rng, 12, 32, 0.8, 1.2) for _ in range(5)]
    sp2 = scene.SceneSpec(walls=sp.walls, bodies=scene.CompactBodies(
        pool=pool, pick=rng.integers(5, size=40), quats=np.array([shapes.random_quaternion(rng) for _ in range(40)])),
        centres=sp.centres[:40])
    for spec in (sp, sp2):
        pb, q0 = spec.principal_bodies()
        world = spec.body_list()
        for k, b in enumerate(pb.expand() if hasattr(pb, "expand") else pb):
            R = shapes.quat_to_matrix(q0[k])
            assert np.abs(b.vertices @ R.T - world[k].vertices).max() < 1e-12
            I = shapes.hull_inertia(b.vertices, b.mass)
            assert np.abs(I - np.diag(b.inertia_bf)).max() < 1e-9 * np.abs(I).max()
            assert np.isclose(b.inertia_size, np.trace(I) / 3)
    rng = np.random.default_rng(1)
    for _ in range(100):
        q = shapes.random_quaternion(rng)
        q = q if q[0] >= 0 else -q
        assert np.allclose(shapes.matrix_to_quat(shapes.quat_to_matrix(q)), q, atol=1e-12)
