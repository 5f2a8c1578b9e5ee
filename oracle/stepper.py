"""The reference's whole per-step CPU path, restated over the reference's own arrays.

TEST INFRASTRUCTURE ONLY: the step-level checker for the device-resident simulator and the timed
CPU baseline of bench.py.  One step follows MWDiem.py:671-1001:

  wall candidates (MWDiem.py:808-811) + cell keys (:813-816) + Linked_cell_hash (:817)
  -> per-pair gather into float32 arrays padded to V vertices (:847-903), history all zero (:966)
  -> contact_detection (FP32, :917-932)
  -> wall rows' force/torque zeroed (:977-978), external force added in FP64 (:980-981)
  -> Verlet (FP64, :986-1001).

The two kernels are either the oracle's C restatement ("port") or the reference kernels compiled
for the host from their own source ("reference", oracle/_ref); both agree bit for bit.
"""
from __future__ import annotations

import numpy as np

import oracle
from mwdiem_gb300 import scene
from mwdiem_gb300.shapes import quat_to_matrix


class RefStepper:
    def __init__(self, spec, V=None, kind="port", nthreads=1, inlet=None):
        """spec: mwdiem_gb300.scene.SceneSpec (walls first, then particles).

        inlet: optional (period, per_spawn, first_row, spawn) -- particles entering during the run
        (MWDiem.py:685-714): rows from first_row on wait outside the broad phase and the integrator
        (the reference's num_particles_temp bound) and, every `period` steps from step 0, the next
        `per_spawn` of them enter at rest at their row of `spawn` ((N, 3) centres), unrotated."""
        W = spec.n_walls
        self.law = getattr(spec, "law", "reference")
        q0 = np.tile([1.0, 0.0, 0.0, 0.0], (W + spec.n_particles, 1))
        parts = None
        if self.law == "physical":
            # principal-axes body frames and starting orientations (SceneSpec.principal_bodies)
            pb, q0[W:] = spec.principal_bodies()
            parts = pb.expand() if hasattr(pb, "expand") else pb
            rot = [quat_to_matrix(q) for q in q0[W:]]
            parts = [type(b)(vertices=b.vertices @ R.T, inertia_bf=b.inertia_bf, inertia_size=b.inertia_size,
                             mass=b.mass) for b, R in zip(parts, rot)]
        st, aux = scene.reference_arrays(spec, V=V, bodies=parts, q0=q0)
        N = aux["N"]
        self.V = aux["V"]
        V = self.V
        centres = st["com"].copy()
        self.st = st
        self.ext = aux["ext"]
        self.nv = aux["nv"]
        self.Is = aux["Is"]
        self.W = W
        self.N = N
        self.wall_n = aux["wall_n"]
        self.wall_range = aux["wall_range"]
        self.nx, self.ny = aux["nx"], aux["ny"]
        self.cs = aux["cs"]
        self.box = aux["box"]
        self.dt = spec.dt
        self.params = dict(Kn=spec.Kn, en=spec.en, et=spec.et, mu=spec.mu, Kn_wall=spec.Kn_wall,
                           en_wall=spec.en_wall, et_wall=spec.et_wall, mu_wall=spec.mu_wall, num_vertices_max=V,
                           num_particles_wall=W, timestep=spec.dt)
        self.kind = kind
        self.nthreads = nthreads
        if self.law != "reference" and kind == "reference":
            raise ValueError("the reference's own kernel has only its own contact law")
        if kind == "reference":
            self.ref_c = oracle.RefContact(self.params, "f32")
            vp = dict(timestep_size=spec.dt, num_particles=N, num_vertices_max=V, syssize_x_max=self.box[0],
                      syssize_x_min=self.box[1], syssize_y_max=self.box[2], syssize_y_min=self.box[3],
                      syssize_z_max=self.box[4], syssize_z_min=self.box[5], num_part_min=W, num_part_max=N)
            self.ref_v = oracle.RefVerlet(vp)
        self.last_pairs = None
        self.last_collision = None
        self.n_steps = 0
        self.active_end = N          # rows [W, active_end) take part in the step
        self.inlet = None
        if inlet is not None:
            period, per_spawn, first, spawn = inlet
            self.inlet = (int(period), int(per_spawn), np.asarray(spawn, dtype=np.float64))
            self.active_end = int(first)
            self.body = [st["verts"][i] - centres[i] for i in range(N)]  # body-frame vertices (unrotated)

    def _inlet_step(self):
        """Rows entering at the start of this step (MWDiem.py:685-714)."""
        period, per_spawn, spawn = self.inlet
        if self.n_steps % period != 0:
            return
        st = self.st
        lo, hi = self.active_end, min(self.N, self.active_end + per_spawn)
        for r in range(lo, hi):
            c = spawn[r]
            for k in ("v", "v12", "w12bf", "wbf", "w", "F", "T", "dxall"):
                st[k][r] = 0.0
            for k in ("q", "q12", "qall"):
                st[k][r] = (1.0, 0.0, 0.0, 0.0)
            st["com"][r] = c
            k = self.nv[r]
            st["verts"][r] = 0.0
            st["verts"][r, :k] = c + self.body[r][:k]
        self.active_end = hi

    def verlet_params(self):
        return dict(timestep_size=self.dt, num_particles=self.N, num_vertices_max=self.V, syssize_x_max=self.box[0],
                    syssize_x_min=self.box[1], syssize_y_max=self.box[2], syssize_y_min=self.box[3],
                    syssize_z_max=self.box[4], syssize_z_min=self.box[5], num_part_min=self.W, num_part_max=self.N)

    def candidate_pairs(self):
        st, W, N = self.st, self.W, self.active_end
        wall = oracle.wall_pairs(W, W, N, st["com"], self.wall_n, st["com"][:W], self.wall_range)
        keys = oracle.cell_keys(st["com"], self.cs[0], self.cs[1], self.cs[2], self.nx, self.ny)
        cells = oracle.linked_cell_hash(W, N, keys, self.nx, self.ny)
        return np.concatenate([wall, cells], 0).astype(np.int32)

    def gather(self, pairs):
        st, V = self.st, self.V
        a, b = pairs[:, 0], pairs[:, 1]
        P = len(pairs)
        f32 = np.float32
        mask_a = np.arange(V)[None, :] < self.nv[a][:, None]
        mask_b = np.arange(V)[None, :] < self.nv[b][:, None]
        return dict(A_com=st["com"][a].astype(f32), B_com=st["com"][b].astype(f32),
                    A_verts=(st["verts"][a] * mask_a[..., None]).astype(f32),
                    B_verts=(st["verts"][b] * mask_b[..., None]).astype(f32),
                    A_vel=st["v"][a].astype(f32), B_vel=st["v"][b].astype(f32),
                    A_angvel=st["w"][a].astype(f32), B_angvel=st["w"][b].astype(f32),
                    A_nv=self.nv[a], B_nv=self.nv[b], A_id=a.astype(np.int32), B_id=b.astype(np.int32),
                    hist=np.zeros((P, 4), f32), qA=st["q"][a].astype(f32), qB=st["q"][b].astype(f32),
                    IsA=self.Is[a].astype(f32), IsB=self.Is[b].astype(f32))

    def inv_mass(self, pairs):
        """Per-pair inverse masses (float32, 0 for a wall side) for the physical contact law."""
        im = (1.0 / self.st["mass"]).astype(np.float32)
        im[: self.W] = 0.0
        return im[pairs[:, 0]], im[pairs[:, 1]]

    def step(self):
        if self.inlet is not None:
            self._inlet_step()
        st, W, N, act = self.st, self.W, self.N, self.active_end
        self.n_steps += 1
        pairs = self.candidate_pairs()
        self.last_pairs = pairs
        if len(pairs):
            inp = self.gather(pairs)
            if self.kind == "reference":
                r = self.ref_c.run(inp, N, nthreads=self.nthreads, snapshot=True)
            else:
                r = oracle.contact(inp, self.params, N, "f32",
                                   inv_mass=self.inv_mass(pairs) if self.law == "physical" else None)
            force, torque = r["force"], r["torque"]
            self.last_collision = r["collision"]
        else:
            force = np.zeros((N, 3), np.float32)
            torque = np.zeros((N, 3), np.float32)
        force[:W] = 0.0
        torque[:W] = 0.0
        st["F"][:] = force + self.ext
        st["T"][:] = torque
        if self.kind == "reference":
            if act != N:
                raise ValueError("the reference's own integrator build covers every row; use kind='port' with an inlet")
            self.ref_v.run(st, nthreads=self.nthreads)
        else:
            oracle.verlet_f64(st, self.dt, self.box, W, act, physical=self.law == "physical")
        return len(pairs)


def inv_mass_from_sim(sim, pairs):
    """Per-pair inverse masses (0 for a wall row) as the device step reads them."""
    im = sim.t["inv_inertia"][:, 3].cpu().numpy().copy()
    im[(sim.t["info"].cpu().numpy() & 1) != 0] = 0.0
    return im[pairs[:, 0]], im[pairs[:, 1]]


def gather_from_sim(sim, pairs, V):
    """Per-pair float32 arrays (the reference's gather, MWDiem.py:847-903) built from a device
    simulator's own state: its world-frame vertices, centres, velocities and quaternions."""
    t = {k: v.cpu().numpy() for k, v in sim.t.items()}
    wv = sim.world_vertices_padded(V)
    nv = np.diff(sim.vert_off_host).astype(np.int32)
    a, b = pairs[:, 0], pairs[:, 1]
    f32 = np.float32
    return dict(A_com=t["pos"][a, :3].astype(f32), B_com=t["pos"][b, :3].astype(f32), A_verts=wv[a], B_verts=wv[b],
                A_vel=t["vel"][a, :3], B_vel=t["vel"][b, :3], A_angvel=t["w"][a, :3], B_angvel=t["w"][b, :3],
                A_nv=nv[a], B_nv=nv[b], A_id=a.astype(np.int32), B_id=b.astype(np.int32),
                hist=np.zeros((len(pairs), 4), f32), qA=t["q"][a], qB=t["q"][b], IsA=t["inertia"][a, 3],
                IsB=t["inertia"][b, 3])
