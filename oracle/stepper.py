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
from mwdiem_gb300.shapes import quat_to_matrix


class RefStepper:
    def __init__(self, spec, V=None, kind="port", nthreads=1):
        """spec: mwdiem_gb300.scene.SceneSpec (walls first, then particles)."""
        W = spec.n_walls
        self.law = getattr(spec, "law", "reference")
        q0 = np.tile([1.0, 0.0, 0.0, 0.0], (W + spec.n_particles, 1))
        if self.law == "physical":
            # principal-axes body frames and starting orientations (SceneSpec.principal_bodies)
            pb, q0[W:] = spec.principal_bodies()
            parts = pb.expand() if hasattr(pb, "expand") else pb
            rot = [quat_to_matrix(q) for q in q0[W:]]
            parts = [type(b)(vertices=b.vertices @ R.T, inertia_bf=b.inertia_bf, inertia_size=b.inertia_size,
                             mass=b.mass) for b, R in zip(parts, rot)]
        else:
            parts = spec.body_list()
        bodies = [b for b, _, _ in spec.walls] + parts
        centres = np.concatenate([np.array([c for _, c, _ in spec.walls]).reshape(-1, 3), spec.centres], 0)
        N = len(bodies)
        nv = np.array([b.vertices.shape[0] for b in bodies], dtype=np.int32)
        self.V = int(V or nv.max())
        V = self.V
        verts = np.zeros((N, V, 3))
        for i, b in enumerate(bodies):
            verts[i, :nv[i]] = centres[i] + b.vertices
        mass = np.array([b.mass for b in bodies])
        I = np.zeros((N, 3, 3))
        Iinv = np.zeros((N, 3, 3))
        for i, b in enumerate(bodies):
            I[i] = np.diag(b.inertia_bf)
            Iinv[i] = np.diag(1.0 / np.asarray(b.inertia_bf))
        z = lambda: np.zeros((N, 3))  # noqa: E731
        q = lambda: np.tile([1.0, 0.0, 0.0, 0.0], (N, 1))  # noqa: E731
        st = dict(v=z(), v12=z(), w12bf=z(), wbf=z(), w=z(), F=z(), T=z(), com=centres.copy(), dxall=z(),
                  q12=q0.copy(), q=q0.copy(), qall=q(), verts=verts, mass=mass, Iinv=Iinv, I=I)
        if spec.velocities is not None:
            st["v"][W:] = spec.velocities
            st["v12"][W:] = spec.velocities
        self.st = st
        self.ext = np.zeros((N, 3))
        self.ext[W:] = mass[W:, None] * np.asarray(spec.gravity)[None, :]
        self.nv = nv
        self.Is = np.array([b.inertia_size for b in bodies])
        self.W = W
        self.N = N
        self.wall_n = np.array([n for _, _, n in spec.walls]).reshape(-1, 3)
        self.wall_range = 6.0 * spec.max_particlesize
        ncell, cs = spec.grid()
        self.nx, self.ny = int(ncell[0]), int(ncell[1])
        self.cs = cs
        self.box = spec.box()
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

    def verlet_params(self):
        return dict(timestep_size=self.dt, num_particles=self.N, num_vertices_max=self.V, syssize_x_max=self.box[0],
                    syssize_x_min=self.box[1], syssize_y_max=self.box[2], syssize_y_min=self.box[3],
                    syssize_z_max=self.box[4], syssize_z_min=self.box[5], num_part_min=self.W, num_part_max=self.N)

    def candidate_pairs(self):
        st, W, N = self.st, self.W, self.N
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
        st, W, N = self.st, self.W, self.N
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
            self.ref_v.run(st, nthreads=self.nthreads)
        else:
            oracle.verlet_f64(st, self.dt, self.box, W, N, physical=self.law == "physical")
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
