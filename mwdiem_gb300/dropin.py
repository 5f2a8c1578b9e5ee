"""The reference's per-step loop over the drop-in modules, state in host memory.

What a user of the reference who only swaps its imports for this package runs each step
(MWDiem.py:671-1001), with every array in host memory as the reference keeps it:

  cell keys (MWDiem.py:813-816) and wall candidates (:808-811)     -> LIBRARY_Coarse_contact_detection
  Linked_cell_hash (:817)                                           -> LIBRARY_Coarse_contact_detection
  per-pair gather into float32 arrays padded to V vertices (:847-903), history zero (:966)
  Contact_detection_GPU (:917-932)                                  -> gpu_fine_contact_detection
  wall rows' force/torque zeroed (:977-978), external force added in FP64 (:980-981)
  Verlet_GPU (:986-1001)                                            -> gpu_Verlet

Each module call copies its numpy arguments to the GPU and back (the reference's pycuda In/InOut
semantics).  The reference gathers the pairs with a Python loop and pandas lookups; here the gather is
vectorised numpy, which is faster, so the time of this loop is a lower bound on the drop-in path's.
The device-resident simulator (sim.Simulator) is the fast path; this loop is what the drop-in costs.
"""
from __future__ import annotations

import numpy as np

from . import LIBRARY_Coarse_contact_detection as CCD
from . import gpu_fine_contact_detection as G
from . import gpu_Verlet
from .scene import SceneSpec, reference_arrays


class ReferenceLoop:
    def __init__(self, spec: SceneSpec, V=None):
        if getattr(spec, "law", "reference") != "reference":
            raise ValueError("the drop-in modules carry the reference's contact law only")
        st, aux = reference_arrays(spec, V=V)
        self.st, self.aux = st, aux
        self.spec = spec
        self.W, self.N, self.V = aux["W"], aux["N"], aux["V"]
        box = aux["box"]
        self.verlet = gpu_Verlet.gpu_Verlet_init(timestep_size=spec.dt, num_particles=self.N, num_vertices_max=self.V,
                                                 syssize_x_max=box[0], syssize_x_min=box[1], syssize_y_max=box[2],
                                                 syssize_y_min=box[3], syssize_z_max=box[4], syssize_z_min=box[5],
                                                 num_part_min=self.W, num_part_max=self.N)
        self.last_pairs = None
        self.last_collision = None

    def candidate_pairs(self):
        st, a = self.st, self.aux
        W, N = self.W, self.N
        walls = CCD.wall_pairs(st["com"], a["wall_n"], a["wall_c"], W, W, N, a["wall_range"]).cpu().numpy()
        keys = CCD.cell_keys(st["com"], a["cs"][0], a["cs"][1], a["cs"][2], a["nx"], a["ny"])
        cells = CCD.linked_cell_pairs(keys, W, N, a["nx"], a["ny"]).cpu().numpy()
        return np.concatenate([walls, cells], 0).astype(np.int32)

    def gather(self, pairs):
        st, a, V = self.st, self.aux, self.V
        A, B = pairs[:, 0], pairs[:, 1]
        f32 = np.float32
        nv = a["nv"]
        mask_a = np.arange(V)[None, :] < nv[A][:, None]
        mask_b = np.arange(V)[None, :] < nv[B][:, None]
        return dict(A_com=st["com"][A].astype(f32), B_com=st["com"][B].astype(f32),
                    A_verts=(st["verts"][A] * mask_a[..., None]).astype(f32),
                    B_verts=(st["verts"][B] * mask_b[..., None]).astype(f32),
                    A_vel=st["v"][A].astype(f32), B_vel=st["v"][B].astype(f32),
                    A_w=st["w"][A].astype(f32), B_w=st["w"][B].astype(f32), A_nv=nv[A], B_nv=nv[B],
                    A_id=A.astype(np.int32), B_id=B.astype(np.int32), hist=np.zeros((len(pairs), 4), f32),
                    qA=st["q"][A].astype(f32), qB=st["q"][B].astype(f32), IsA=a["Is"][A].astype(f32),
                    IsB=a["Is"][B].astype(f32))

    def step(self):
        st, sp = self.st, self.spec
        W, N = self.W, self.N
        pairs = self.candidate_pairs()
        self.last_pairs = pairs
        force = np.zeros((N, 3), np.float32)
        torque = np.zeros((N, 3), np.float32)
        if len(pairs):
            g = self.gather(pairs)
            force, torque, _, coll = G.Contact_detection_GPU(
                g["A_com"], g["B_com"], g["A_verts"], g["B_verts"], g["A_vel"], g["B_vel"], g["A_w"], g["B_w"],
                g["A_nv"], g["B_nv"], g["A_id"], g["B_id"], g["hist"], sp.Kn, sp.en, sp.et, sp.mu, sp.Kn_wall,
                sp.en_wall, sp.et_wall, sp.mu_wall, W, force, torque, self.V, g["qA"], g["qB"], sp.dt, g["IsA"],
                g["IsB"])
            self.last_collision = coll
        force[:W] = 0.0
        torque[:W] = 0.0
        st["F"][:] = force + self.aux["ext"]
        st["T"][:] = torque
        r = gpu_Verlet.gpu_Verlett(self.verlet, st["v"], st["v12"], st["w12bf"], st["q12"], st["q"], st["qall"],
                                   st["wbf"], st["w"], st["F"], st["T"], st["verts"], st["com"], st["mass"],
                                   st["Iinv"], st["I"], st["dxall"])
        (st["v12"], st["q"], st["wbf"], st["w12bf"], st["w"], st["q12"], st["v"], st["com"], st["verts"],
         st["qall"], st["dxall"]) = r
        return len(pairs)
