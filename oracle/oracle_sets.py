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


def render_all():
    out = []
    for p in CONTACT_SETS:
        out.append(build_ref.ensure_built("contact", p, "f32"))
    for p in VERLET_SETS:
        out.append(build_ref.ensure_built("verlet", p, "f32"))
    return out
