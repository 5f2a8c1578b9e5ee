"""Parameter sets for which the reference kernels are rendered ahead of time.

TEST INFRASTRUCTURE ONLY.  The reference bakes its constants into the kernel source, so each
parameter set is a separate host build (oracle/build_ref.py).  Rendering needs the reference
checkout; the rendered sources travel with the repository snapshot (oracle/_ref, git-ignored) so a
machine without the checkout can still compile them.
"""
from __future__ import annotations

import build_ref

# narrow phase of the pour scene and of the tests (kn 1e5, damping ratio 0.3 -> en 0.372, mu 0.5)
CONTACT_SETS = [
    dict(Kn=1e5, en=0.372, et=0.372, mu=0.5, Kn_wall=1e5, en_wall=0.372, et_wall=0.372, mu_wall=0.5,
         num_vertices_max=32, num_particles_wall=4, timestep=5e-5),
]
VERLET_SETS: list = []


def register_contact(params: dict):
    if params not in CONTACT_SETS:
        CONTACT_SETS.append(dict(params))


def register_verlet(params: dict):
    if params not in VERLET_SETS:
        VERLET_SETS.append(dict(params))


def pour_sets(n=20000, box=40.0, spacing=2.6, r_max=1.2, zeta=0.3, kn=1e5, mu=0.5, dt=5e-5, V=32):
    """Contact and integrator parameter sets of the pour scene (the benchmark workload), computed
    from its sizes alone with the same code that builds the scene."""
    from mwdiem_gb300 import scene
    walls = scene.pour_walls(n, box, spacing, r_max)
    sp = scene.SceneSpec(walls=walls)
    en = scene.restitution_from_damping(zeta)
    W = len(walls)
    box6 = sp.box()
    c = dict(Kn=kn, en=en, et=en, mu=mu, Kn_wall=kn, en_wall=en, et_wall=en, mu_wall=mu, num_vertices_max=V,
             num_particles_wall=W, timestep=dt)
    v = dict(timestep_size=dt, num_particles=n + W, num_vertices_max=V, syssize_x_max=box6[0],
             syssize_x_min=box6[1], syssize_y_max=box6[2], syssize_y_min=box6[3], syssize_z_max=box6[4],
             syssize_z_min=box6[5], num_part_min=W, num_part_max=n + W)
    return c, v


def pairs_set(kn=1e5, zeta=0.3, mu=0.5, dt=5e-5, V=64):
    """Contact parameters of the independent-pair narrow-phase workload (hulls of up to 64 vertices,
    no walls), as mwdiem_gb300.pairbench.PairScene sets them."""
    from mwdiem_gb300 import scene
    en = scene.restitution_from_damping(zeta)
    return dict(Kn=kn, en=en, et=en, mu=mu, Kn_wall=kn, en_wall=en, et_wall=en, mu_wall=mu, num_vertices_max=V,
                num_particles_wall=0, timestep=dt)


def settling_sets():
    """Contact and integrator parameter sets of the 125-cube settling scene, as the reference path
    (oracle/stepper.py) derives them from the scene."""
    import stepper
    from mwdiem_gb300 import scene
    s = stepper.RefStepper(scene.settling_scene(), kind="port")
    return dict(s.params), s.verlet_params()


def batch_sample(specs, n_sample=8):
    """The scenes of a batch whose reference path the batched benchmark runs: the largest, then
    n_sample - 1 others drawn at random (seed 0)."""
    import numpy as np
    rng = np.random.default_rng(0)
    first = int(np.argmax([sp.n_particles for sp in specs]))
    rest = [i for i in range(len(specs)) if i != first]
    return [first] + [int(i) for i in rng.choice(rest, size=min(n_sample - 1, len(rest)), replace=False)]


def batch_sets(n_scenes=256, total=2_000_000):
    """Contact and integrator parameter sets of the sampled scenes of the batched benchmark."""
    import stepper
    from mwdiem_gb300 import scene
    specs = scene.batched_scenes(n_scenes=n_scenes, total=total, seed=0)
    out = []
    for i in batch_sample(specs):
        s = stepper.RefStepper(specs[i], kind="port")
        out.append((dict(s.params), s.verlet_params()))
    return out


def render_all():
    c, v = pour_sets()
    register_contact(c)
    register_verlet(v)
    register_contact(pairs_set())
    c, v = settling_sets()
    register_contact(c)
    register_verlet(v)
    for c, v in batch_sets():
        register_contact(c)
        register_verlet(v)
    out = []
    for p in CONTACT_SETS:
        out.append(build_ref.ensure_built("contact", p, "f32"))
    for p in VERLET_SETS:
        out.append(build_ref.ensure_built("verlet", p, "f32"))
    return out
