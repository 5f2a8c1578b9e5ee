"""Drop-in for ``LIBRARIES/gpu_Verlet.py`` (quaternion leapfrog integrator, FP64).

* ``Verlet_GPU(27 arguments) -> 11-tuple`` in the reference's order (``gpu_Verlet.py:53-92``);
* ``gpu_Verlet_init(**constants)`` / ``gpu_Verlett(calc_function, ...)`` (``gpu_Verlet.py:10-50``).

One precompiled sm_103a kernel (``mwd_verlet_ref``) replaces the per-call template render and
compile.  numpy arguments are copied to the GPU and back with in-place semantics (pycuda's
``cuda.InOut``); float64 CUDA tensors are updated in place.
"""
from __future__ import annotations

import numpy as np

from . import _dev
from ._lib import VerletParams, check, lib

_INOUT = ("velocity_arr", "velocity_12_arr", "angular_velocity_12_bf_arr", "quaternion_12_arr", "quaternion_arr",
          "quaternion_all_arr", "angular_velocity_bf_arr", "angular_velocity_arr")


class VerletKernel:
    """What ``gpu_Verlet_init`` returns: timestep, box and row range fixed (``gpu_Verlet.py:63-73``)."""

    def __init__(self, timestep_size, num_particles, num_vertices_max, syssize_x_max, syssize_x_min, syssize_y_max,
                 syssize_y_min, syssize_z_max, syssize_z_min, num_part_min, num_part_max):
        p = VerletParams()
        p.dt = float(timestep_size)
        for i, v in enumerate((syssize_x_max, syssize_x_min, syssize_y_max, syssize_y_min, syssize_z_max,
                               syssize_z_min)):
            p.box[i] = float(v)
        p.n_min, p.n_max, p.V = int(num_part_min), int(num_part_max), int(num_vertices_max)
        self.params = p
        self.num_particles = int(num_particles)

    def __call__(self, velocity_arr, velocity_12_arr, angular_velocity_12_bf_arr, quaternion_12_arr, quaternion_arr,
                 quaternion_all_arr, angular_velocity_bf_arr, angular_velocity_arr, force_arr, torque_arr,
                 vertices_arr, center_of_mass_arr, mass_arr, moment_of_inertia_inv_arr, moment_of_inertia_arr,
                 dx_all_arr, *, n_reset=None, stream=None):
        _dev.require_cuda()
        f64 = np.float64
        io = [_dev.Arg(x, f64, nm, out=True) for x, nm in zip(
            (velocity_arr, velocity_12_arr, angular_velocity_12_bf_arr, quaternion_12_arr, quaternion_arr,
             quaternion_all_arr, angular_velocity_bf_arr, angular_velocity_arr), _INOUT)]
        F = _dev.Arg(force_arr, f64, "force_arr")
        T = _dev.Arg(torque_arr, f64, "torque_arr")
        verts = _dev.Arg(vertices_arr, f64, "vertices_arr", out=True)
        com = _dev.Arg(center_of_mass_arr, f64, "center_of_mass_arr", out=True)
        mass = _dev.Arg(mass_arr, f64, "mass_arr")
        Iinv = _dev.Arg(moment_of_inertia_inv_arr, f64, "moment_of_inertia_inv_arr")
        I = _dev.Arg(moment_of_inertia_arr, f64, "moment_of_inertia_arr")
        dx = _dev.Arg(dx_all_arr, f64, "dx_all_arr", out=True)
        N = int(com.t.shape[0])
        if N and int(verts.t.shape[1]) != self.params.V:
            raise ValueError(f"vertices_arr must be (N, {self.params.V}, 3)")
        s = _dev.stream_handle(stream)
        v, v12, w12bf, q12, q, qall, wbf, w = (a.ptr for a in io)
        check(lib().mwd_verlet_ref(N, v, v12, w12bf, q12, q, qall, wbf, w, F.ptr, T.ptr, verts.ptr, com.ptr, mass.ptr,
                                   Iinv.ptr, I.ptr, dx.ptr, self.params,
                                   n_reset.data_ptr() if n_reset is not None else None, s))
        r = [a.result() for a in io]
        vel, vel12, om12bf, quat12, quat, quatall, ombf, om = r
        return (vel12, quat, ombf, om12bf, om, quat12, vel, com.result(), verts.result(), quatall, dx.result())


def gpu_Verlet_init(**args):
    return VerletKernel(**args)


def gpu_Verlett(calc_function, velocity_arr, velocity_12_arr, angular_velocity_12_bf_arr, quaternion_12_arr,
                quaternion_arr, quaternion_all_arr, angular_velocity_bf_arr, angular_velocity_arr, force_arr,
                torque_arr, vertices_arr, center_of_mass_arr, mass_arr, moment_of_inertia_inv_arr,
                moment_of_inertia_arr, dx_all_arr):
    """``gpu_Verlet.py:18-50``."""
    return calc_function(velocity_arr, velocity_12_arr, angular_velocity_12_bf_arr, quaternion_12_arr,
                         quaternion_arr, quaternion_all_arr, angular_velocity_bf_arr, angular_velocity_arr, force_arr,
                         torque_arr, vertices_arr, center_of_mass_arr, mass_arr, moment_of_inertia_inv_arr,
                         moment_of_inertia_arr, dx_all_arr)


def Verlet_GPU(velocity_arr, velocity_12_arr, angular_velocity_12_bf_arr, quaternion_12_arr, quaternion_arr,
               quaternion_all_arr, angular_velocity_bf_arr, angular_velocity_arr, force_arr, torque_arr, vertices_arr,
               center_of_mass_arr, timestep_size, mass_arr, num_particles, moment_of_inertia_inv_arr,
               moment_of_inertia_arr, dx_all_arr, num_vertices_max, syssize_x_max, syssize_x_min, syssize_y_max,
               syssize_y_min, syssize_z_max, syssize_z_min, num_part_min, num_part_max, *, n_reset=None,
               stream=None):
    """``gpu_Verlet.py:53-92``; returns (velocity_12, quaternion, angular_velocity_bf, angular_velocity_12_bf,
    angular_velocity, quaternion_12, velocity, center_of_mass, vertices, quaternion_all, dx_all)."""
    k = VerletKernel(timestep_size, num_particles, num_vertices_max, syssize_x_max, syssize_x_min, syssize_y_max,
                     syssize_y_min, syssize_z_max, syssize_z_min, num_part_min, num_part_max)
    return k(velocity_arr, velocity_12_arr, angular_velocity_12_bf_arr, quaternion_12_arr, quaternion_arr,
             quaternion_all_arr, angular_velocity_bf_arr, angular_velocity_arr, force_arr, torque_arr, vertices_arr,
             center_of_mass_arr, mass_arr, moment_of_inertia_inv_arr, moment_of_inertia_arr, dx_all_arr,
             n_reset=n_reset, stream=stream)
