"""Drop-in for ``LIBRARIES/gpu_fine_contact_detection.py`` (GJK/EPA narrow phase + contact force).

Same entry points, argument order, dtypes and return tuples as the reference:

* ``Contact_detection_GPU(...) -> (force, torque, displacement_tang, collision)``
  (``gpu_fine_contact_detection.py:76-119``);
* ``gpu_contact_detection_init(**constants)`` returns a callable with the constants fixed, and
  ``gpu_contact_detection(calc_function, ...) -> (force, torque, collision, displacement_tang)``
  (``gpu_fine_contact_detection.py:10-73``).

The reference renders a Jinja template and recompiles the kernel on every call; here the constants
are a POD argument of one precompiled sm_103a kernel (``mwd_contact_pairs`` in ``libmwdem.so``).
Arguments may be numpy arrays (copied to the GPU and back; ``force``, ``torque`` and
``displacement_tang`` are updated in place like pycuda's ``cuda.InOut``) or CUDA tensors (used in
place, no copies).  ``displacement_tang`` keeps the reference's stride-1 indexing by default
(``hist_mode=0``); ``hist_mode=1`` uses the array's own stride of 4.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _dev
from ._lib import ContactParams, check, lib


class ContactKernel:
    """What ``gpu_contact_detection_init`` returns: the contact law and sizes, fixed."""

    def __init__(self, Kn, en, et, Kn_wall, en_wall, et_wall, mu, mu_wall, num_vertices_max, num_particles_wall,
                 timestep, num_pairs=None, hist_mode=0, lanes=0):
        self.params = ContactParams(float(Kn), float(en), float(et), float(mu), float(Kn_wall), float(en_wall),
                                    float(et_wall), float(mu_wall), float(timestep), int(num_particles_wall),
                                    int(hist_mode), int(lanes), 0)
        self.V = int(num_vertices_max)

    def __call__(self, A_com, B_com, A_verts, B_verts, A_vel, B_vel, A_w, B_w, A_nv, B_nv, A_id, B_id, hist, force,
                 torque, qA, qB, IsA, IsB, *, diag=None, status=None, stream=None):
        _dev.require_cuda()
        f32, i32 = np.float32, np.int32
        n = int(A_com.shape[0])
        ins = [_dev.Arg(x, f32, nm) for x, nm in ((A_com, "A_com"), (B_com, "B_com"), (A_verts, "A_verts"),
                                                  (B_verts, "B_verts"), (A_vel, "A_vel"), (B_vel, "B_vel"),
                                                  (A_w, "A_angvel"), (B_w, "B_angvel"))]
        ints = [_dev.Arg(x, i32, nm) for x, nm in ((A_nv, "A_nv"), (B_nv, "B_nv"), (A_id, "A_id"), (B_id, "B_id"))]
        h = _dev.Arg(hist, f32, "displacement_tang", out=True)
        F = _dev.Arg(force, f32, "force", out=True)
        T = _dev.Arg(torque, f32, "torque", out=True)
        q = [_dev.Arg(x, f32, nm) for x, nm in ((qA, "quaternion_A"), (qB, "quaternion_B"))]
        Is = [_dev.Arg(x, f32, nm) for x, nm in ((IsA, "mom_inertia_size_A"), (IsB, "mom_inertia_size_B"))]
        dev = F.t.device
        coll = torch.empty(n, dtype=torch.int32, device=dev)
        V = self.V
        if n:
            if tuple(ins[2].t.shape[1:]) != (V, 3) or tuple(ins[3].t.shape[1:]) != (V, 3):
                raise ValueError(f"vertex arrays must be (P, {V}, 3)")
            n_particles = int(F.t.shape[0])
            s = _dev.stream_handle(stream)
            check(lib().mwd_contact_pairs(n, V, n_particles, *[a.ptr for a in ins], *[a.ptr for a in ints], h.ptr,
                                          F.ptr, T.ptr, q[0].ptr, q[1].ptr, Is[0].ptr, Is[1].ptr, coll.data_ptr(),
                                          self.params, diag.data_ptr() if diag is not None else None,
                                          status.data_ptr() if status is not None else None, s))
        host = F.host is not None
        collision = coll.cpu().numpy() if host else coll
        return F.result(), T.result(), collision, h.result()


def gpu_contact_detection_init(**args):
    """``gpu_fine_contact_detection.py:10-15``: here nothing is compiled per call."""
    return ContactKernel(**args)


def gpu_contact_detection(calc_function, particle_A_center_of_mass, particle_B_center_of_mass, particle_A_vertices,
                          particle_B_vertices, particle_A_velocity, particle_B_velocity, particle_A_angular_velocity,
                          particle_B_angular_velocity, particle_A_numvertices, particle_B_numvertices, particle_A_id,
                          particle_B_id, displacement_tang, force, torque, quaternion_A, quaternion_B,
                          mom_inertia_size_A, mom_inertia_size_B):
    """``gpu_fine_contact_detection.py:18-73``; returns (force, torque, collision, displacement_tang)."""
    return calc_function(particle_A_center_of_mass, particle_B_center_of_mass, particle_A_vertices,
                         particle_B_vertices, particle_A_velocity, particle_B_velocity, particle_A_angular_velocity,
                         particle_B_angular_velocity, particle_A_numvertices, particle_B_numvertices, particle_A_id,
                         particle_B_id, displacement_tang, force, torque, quaternion_A, quaternion_B,
                         mom_inertia_size_A, mom_inertia_size_B)


def Contact_detection_GPU(particle_A_center_of_mass, particle_B_center_of_mass, particle_A_vertices,
                          particle_B_vertices, particle_A_velocity, particle_B_velocity, particle_A_angular_velocity,
                          particle_B_angular_velocity, particle_A_numvertices, particle_B_numvertices, particle_A_id,
                          particle_B_id, displacement_tang, Kn, en, et, mu, Kn_wall, en_wall, et_wall, mu_wall,
                          num_particles_wall, force, torque, num_vertices_maxi, quaternion_A, quaternion_B,
                          timestep_size, mom_inertia_size_A, mom_inertia_size_B, *, hist_mode=0, lanes=0, diag=None,
                          status=None, stream=None):
    """``gpu_fine_contact_detection.py:76-119``; returns (force, torque, displacement_tang, collision)."""
    k = ContactKernel(Kn=Kn, en=en, et=et, Kn_wall=Kn_wall, en_wall=en_wall, et_wall=et_wall, mu=mu,
                      mu_wall=mu_wall, num_vertices_max=num_vertices_maxi, num_particles_wall=num_particles_wall,
                      timestep=timestep_size, hist_mode=hist_mode, lanes=lanes)
    F, T, coll, hist = k(particle_A_center_of_mass, particle_B_center_of_mass, particle_A_vertices,
                         particle_B_vertices, particle_A_velocity, particle_B_velocity, particle_A_angular_velocity,
                         particle_B_angular_velocity, particle_A_numvertices, particle_B_numvertices, particle_A_id,
                         particle_B_id, displacement_tang, force, torque, quaternion_A, quaternion_B,
                         mom_inertia_size_A, mom_inertia_size_B, diag=diag, status=status, stream=stream)
    return F, T, hist, coll
