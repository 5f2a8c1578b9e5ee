"""Interface of ``LIBRARIES/LIBRARY_Force.py`` (a Hertzian normal force with a capped sliding
friction, ``LIBRARY_Force.py:3-47``).

The reference imports it (``MWDiem.py:17``) but never calls it: its contact force is the
spring-dashpot law inside the GPU contact kernel (``gpu_fine_contact_detection.Contact_detection_GPU``
here).  This function keeps the signature and the formula for scripts that call it directly; it
operates on one pair of host-side ``Particle`` objects and is not part of the simulated step.

    Fn_A = -sign * Ks depth^(3/2) n  -  Kd depth^(1/2) (v_rel . n) n    (n oriented from A to B)
    Ft_A = -min(mu |Fn_A|, Ks |v_t|) v_t / |v_t|
    returns (Fn_A, Fn_As, Fn_Ad, TorqueA, TorqueB) with TorqueX = (cp_X - c_X) x Ft_X, Ft_B = -Ft_A
"""
from __future__ import annotations

import numpy as np


def Force(particle_A, particle_B, penetration_depth, penetration_normal, contact_point_A, contact_point_B, Ks, Kd,
          mu):
    cA = np.asarray(particle_A.center_of_mass, dtype=float)
    cB = np.asarray(particle_B.center_of_mass, dtype=float)
    n = np.asarray(penetration_normal, dtype=float)
    if np.dot(cB - cA, n) < 0:
        n = -n
    spring = (Ks * penetration_depth ** 1.5) * n
    if np.dot(cB - cA, spring) > 0:
        spring = -spring
    v_rel = np.asarray(particle_A.velocity, dtype=float) - np.asarray(particle_B.velocity, dtype=float)
    v_n = np.dot(v_rel, n) * n
    damping = -(Kd * penetration_depth ** 0.5) * v_n
    Fn = spring + damping
    v_t = v_rel - v_n
    vt_len = np.linalg.norm(v_t)
    if vt_len != 0:
        Ft = -min(mu * np.linalg.norm(Fn), Ks * vt_len) * v_t / vt_len
    else:
        Ft = np.zeros(3)
    TA = np.cross(np.asarray(contact_point_A, dtype=float) - cA, Ft)
    TB = np.cross(np.asarray(contact_point_B, dtype=float) - cB, -Ft)
    return Fn, spring, damping, TA, TB
