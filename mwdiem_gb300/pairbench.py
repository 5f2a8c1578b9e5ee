"""Narrow-phase workload of independent pairs (the GJK/EPA pairs/s measurement).

``PairScene(n_pairs)`` builds, on the device, 2 n_pairs rows: pair i is rows (2i, 2i+1), each a
random convex hull of U{n_min..n_max} points on a sphere of radius U[r_min, r_max] (drawn from a
pool of distinct hulls), with a random orientation, the two centres U[dist]·(rA + rB)/2 apart along
a random direction, random velocities and spins.  The pair list is fixed, so ``narrow()`` runs just
the narrow phase + force of the device step (``mwd_narrow_force``) over it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import scene
from ._lib import EPA_COUNT_INTS, ContactParams, Scene, State, Work, check, lib


class PairScene:
    def __init__(self, n_pairs, seed=0, n_min=8, n_max=64, r_min=0.8, r_max=1.2, dist=(0.5, 2.2), pool=1024,
                 kn=1e5, zeta=0.3, mu=0.5, dt=5e-5, lanes=8, two_pass=True, device="cuda"):
        self.n_pairs = int(n_pairs)
        self.lanes = int(lanes)
        dev = torch.device(device)
        rng = np.random.default_rng(seed)
        bodies = [scene.fast_hull_body(rng, n_min, n_max, r_min, r_max) for _ in range(pool)]
        V = max(b.vertices.shape[0] for b in bodies)
        pv = np.zeros((pool, V, 3), np.float32)
        cnt = np.zeros(pool, np.int64)
        rad = np.zeros(pool, np.float64)
        inert = np.zeros((pool, 4), np.float32)
        inv = np.zeros((pool, 4), np.float32)
        for k, b in enumerate(bodies):
            n = b.vertices.shape[0]
            pv[k, :n] = b.vertices
            cnt[k] = n
            rad[k] = np.sqrt((b.vertices ** 2).sum(1)).max()
            inert[k] = [*b.inertia_bf, b.inertia_size]
            inv[k] = [*(1.0 / np.asarray(b.inertia_bf)), 1.0 / b.mass]
        g = torch.Generator(device=dev).manual_seed(seed)
        rows = 2 * self.n_pairs
        shape = torch.randint(0, pool, (rows,), generator=g, device=dev)
        pv_t = torch.from_numpy(pv).to(dev)
        cnt_t = torch.from_numpy(cnt).to(dev)
        rad_t = torch.from_numpy(rad).to(dev)
        q = torch.randn((rows, 4), generator=g, device=dev)
        q = q / q.norm(dim=1, keepdim=True)
        R = _quat_to_matrix(q)                                     # (rows,3,3)
        ca = (torch.rand((self.n_pairs, 3), generator=g, device=dev, dtype=torch.float64) - 0.5) * 200.0
        d = torch.randn((self.n_pairs, 3), generator=g, device=dev, dtype=torch.float64)
        d = d / d.norm(dim=1, keepdim=True)
        ra, rb = rad_t[shape[0::2]], rad_t[shape[1::2]]
        u = torch.rand(self.n_pairs, generator=g, device=dev, dtype=torch.float64) * (dist[1] - dist[0]) + dist[0]
        cb = ca + d * (u * (ra + rb) / 2)[:, None]
        pos = torch.zeros((rows, 4), dtype=torch.float64, device=dev)
        pos[0::2, :3] = ca
        pos[1::2, :3] = cb
        counts = cnt_t[shape]
        off = torch.zeros(rows + 1, dtype=torch.int64, device=dev)
        off[1:] = torch.cumsum(counts, 0)
        total = int(off[-1].item())
        # body-frame vertices with the orientation baked in, compacted to CSR
        body = torch.zeros((total, 4), dtype=torch.float32, device=dev)
        world = torch.zeros((total, 4), dtype=torch.float32, device=dev)
        chunk = 1 << 20
        for r0 in range(0, rows, chunk):
            r1 = min(rows, r0 + chunk)
            v = torch.einsum("rij,rkj->rki", R[r0:r1], pv_t[shape[r0:r1]])       # (n,V,3)
            mask = torch.arange(V, device=dev)[None, :] < counts[r0:r1, None]
            flat = v[mask]
            o0, o1 = int(off[r0].item()), int(off[r1].item())
            body[o0:o1, :3] = flat
            owner = torch.repeat_interleave(torch.arange(r0, r1, device=dev), counts[r0:r1])
            world[o0:o1, :3] = (pos[owner, :3] + flat.double()).float()

        pos[:, 3] = rad_t[shape]  # bounding radius (rotation keeps the vertex norms)
        f32 = dict(dtype=torch.float32, device=dev)
        vel = torch.cat([torch.randn((rows, 3), generator=g, **f32) * 0.5, torch.zeros((rows, 1), **f32)], 1)
        w = torch.cat([torch.randn((rows, 3), generator=g, **f32) * 2.0, torch.zeros((rows, 1), **f32)], 1)
        q = torch.cat([torch.ones((rows, 1), **f32), torch.zeros((rows, 3), **f32)], 1)
        en = scene.restitution_from_damping(zeta)
        self._assemble(pos, vel, w, q, torch.from_numpy(inert).to(dev)[shape].contiguous(),
                       torch.from_numpy(inv).to(dev)[shape].contiguous(), off, body, world, int(V),
                       dict(Kn=kn, en=en, et=en, mu=mu, Kn_wall=kn, en_wall=en, et_wall=en, mu_wall=mu,
                            num_vertices_max=int(V), num_particles_wall=0, timestep=dt), two_pass)

    @classmethod
    def from_arrays(cls, inp, params, lanes=8, two_pass=True, device="cuda"):
        """The pairs of per-pair arrays in the reference's layout (MWDiem.py:847-903; world-frame
        vertices padded to V, as the oracle takes them), as the device step holds them: pair i is rows
        (2i, 2i+1) with exactly those vertices, centres, velocities, spins and quaternions.  The narrow
        phase then sees the oracle's inputs bit for bit.  `params`: the contact law (the reference's
        constants; no walls)."""
        self = cls.__new__(cls)
        dev = torch.device(device)
        P = int(np.asarray(inp["A_com"]).shape[0])
        self.n_pairs = P
        self.lanes = int(lanes)
        rows = 2 * P

        def inter(a, b, width):
            out = np.zeros((rows, width), np.float64)
            out[0::2, :np.asarray(a).shape[1]] = a
            out[1::2, :np.asarray(b).shape[1]] = b
            return out

        com = inter(inp["A_com"], inp["B_com"], 4)
        V = int(np.asarray(inp["A_verts"]).shape[1])
        counts = np.empty(rows, np.int64)
        counts[0::2], counts[1::2] = inp["A_nv"], inp["B_nv"]
        verts = np.empty((rows, V, 3), np.float32)
        verts[0::2], verts[1::2] = inp["A_verts"], inp["B_verts"]
        mask = np.arange(V)[None, :] < counts[:, None]
        world = np.zeros((int(counts.sum()), 4), np.float32)
        world[:, :3] = verts[mask]
        rel = verts.astype(np.float64) - com[:, None, :3]
        com[:, 3] = np.sqrt((rel ** 2).sum(2) * mask).max(1)
        off = np.zeros(rows + 1, np.int64)
        off[1:] = np.cumsum(counts)
        inert = np.zeros((rows, 4), np.float32)
        inert[0::2, 3], inert[1::2, 3] = inp["IsA"], inp["IsB"]
        f32 = dict(dtype=torch.float32, device=dev)
        world_t = torch.from_numpy(world).to(dev)
        self._assemble(torch.from_numpy(com).to(dev), torch.from_numpy(inter(inp["A_vel"], inp["B_vel"], 4)).to(**f32),
                       torch.from_numpy(inter(inp["A_angvel"], inp["B_angvel"], 4)).to(**f32),
                       torch.from_numpy(inter(inp["qA"], inp["qB"], 4)).to(**f32), torch.from_numpy(inert).to(dev),
                       torch.ones((rows, 4), **f32), torch.from_numpy(off).to(dev), world_t.clone(), world_t, V,
                       dict(params, num_particles_wall=0), two_pass)
        return self

    def _assemble(self, pos, vel, w, q, inertia, inv_inertia, off, body, world, V, params, two_pass):
        """State, scene and work arrays of the rows (pair i = rows 2i, 2i+1) for mwd_narrow_force."""
        dev = pos.device
        rows = int(pos.shape[0])
        total = int(world.shape[0])
        f32 = dict(dtype=torch.float32, device=dev)
        t = {"pos": pos, "dx_all": torch.zeros((rows, 4), dtype=torch.float64, device=dev),
             "wall_normal": torch.zeros((rows, 4), dtype=torch.float64, device=dev),
             "vel": vel, "w": w, "q": q, "inertia": inertia, "inv_inertia": inv_inertia,
             "info": torch.zeros(rows, dtype=torch.int32, device=dev),
             "vert_off": off.to(torch.int32), "body_verts": body, "world_verts": world}
        for k in ("vel_half", "w_half_bf", "w_bf", "q_half", "q_all", "q_acc", "force", "torque", "ext_force",
                  "ext_torque"):
            t[k] = torch.zeros((rows, 4), **f32)
        self.t = t
        st = State()
        for k in ("pos", "dx_all", "vel", "vel_half", "w_half_bf", "w_bf", "w", "q", "q_half", "q_all", "q_acc",
                  "force", "torque", "ext_force", "ext_torque", "inertia", "inv_inertia", "info", "wall_normal",
                  "vert_off", "body_verts", "world_verts"):
            setattr(st, k, t[k].data_ptr())
        st.n, st.n_verts, st.max_verts = rows, total, int(V)
        self.state = st
        p = params
        sc = (Scene * 1)()
        sc[0].dt = p["timestep"]
        sc[0].law = ContactParams(p["Kn"], p["en"], p["et"], p["mu"], p["Kn_wall"], p["en_wall"], p["et_wall"],
                                  p["mu_wall"], p["timestep"], 0, 0, self.lanes, 0)
        check(lib().mwd_derive_material(C.byref(sc[0].law), sc[0].mat))
        self.params = dict(p, num_vertices_max=int(V), num_particles_wall=0)
        self.scenes_host = sc
        raw = bytes(C.string_at(C.addressof(sc), C.sizeof(sc)))
        self.scenes_dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)
        i32 = dict(dtype=torch.int32, device=dev)
        idx = torch.arange(self.n_pairs, dtype=torch.int32, device=dev)
        w = {"pairs": torch.stack([2 * idx, 2 * idx + 1], 1).contiguous(),
             "n_pairs": torch.tensor([self.n_pairs], dtype=torch.int64, device=dev),
             "status": torch.zeros(1, **i32), "collision": torch.zeros(self.n_pairs, **i32),
             "counters": torch.zeros(3, dtype=torch.int64, device=dev)}
        wk = Work()
        wk.pairs, wk.n_pairs, wk.status = w["pairs"].data_ptr(), w["n_pairs"].data_ptr(), w["status"].data_ptr()
        wk.collision = w["collision"].data_ptr()
        wk.pair_cap = self.n_pairs
        if two_pass:
            w["epa_count"] = torch.zeros(EPA_COUNT_INTS, **i32)
            w["epa_rec"] = torch.zeros(self.n_pairs * 80, dtype=torch.uint8, device=dev)
            wk.epa_count, wk.epa_rec, wk.epa_cap = w["epa_count"].data_ptr(), w["epa_rec"].data_ptr(), self.n_pairs
        self.w = w
        self.work = wk
        self.V = int(V)
        self.vert_off_host = None

    def narrow(self, count_work=False):
        self.work.work_counters = self.w["counters"].data_ptr() if count_work else None
        if count_work:
            self.w["counters"].zero_()
        check(lib().mwd_narrow_force(C.byref(self.state), self.scenes_dev.data_ptr(), C.byref(self.work), self.lanes,
                                     int(torch.cuda.current_stream().cuda_stream)))
        self.work.work_counters = None

    def gather(self, idx):
        """Per-pair float32 arrays (reference layout) for the pairs `idx` (host), for the oracle.  Only
        the rows of those pairs are copied from the device."""
        idx = np.asarray(idx)
        dev = self.t["pos"].device
        a = torch.from_numpy(2 * idx).to(dev)
        b = a + 1
        off = self.t["vert_off"].long()
        V = self.V

        def verts(rows):
            cnt = off[rows + 1] - off[rows]
            ar = torch.arange(V, device=dev)
            mask = ar[None, :] < cnt[:, None]
            src = torch.where(mask, off[rows][:, None] + ar[None, :], torch.zeros_like(mask, dtype=torch.long))
            out = torch.where(mask[..., None], self.t["world_verts"][src][..., :3], 0.0)
            return out.cpu().numpy()

        def rows_of(k, rows, cols=slice(0, 3)):
            return self.t[k][rows][:, cols].cpu().numpy()

        nv = (off[1:] - off[:-1]).int()
        ai, bi = a.cpu().numpy(), b.cpu().numpy()
        return dict(A_com=rows_of("pos", a).astype(np.float32), B_com=rows_of("pos", b).astype(np.float32),
                    A_verts=verts(a), B_verts=verts(b), A_vel=rows_of("vel", a), B_vel=rows_of("vel", b),
                    A_angvel=rows_of("w", a), B_angvel=rows_of("w", b), A_nv=nv[a].cpu().numpy(),
                    B_nv=nv[b].cpu().numpy(), A_id=ai.astype(np.int32), B_id=bi.astype(np.int32),
                    hist=np.zeros((len(idx), 4), np.float32), qA=rows_of("q", a, slice(0, 4)),
                    qB=rows_of("q", b, slice(0, 4)), IsA=self.t["inertia"][a, 3].cpu().numpy(),
                    IsB=self.t["inertia"][b, 3].cpu().numpy())


def _quat_to_matrix(q):
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return torch.stack([torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], 1),
                        torch.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], 1),
                        torch.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1)], 1)
