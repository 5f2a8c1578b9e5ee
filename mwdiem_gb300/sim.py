"""Device-resident DEM step: state in HBM, one C-ABI call per step (or a CUDA-graph replay).

The state is a structure of arrays over "rows" (walls first, then particles, per scene; several
scenes are simply concatenated -- that is the batched mode).  A step is broad phase -> narrow phase
+ force -> integrator (``mwd_step`` in ``libmwdem.so``), the per-step body of ``MWDiem.py:671-1001``
without its host round-trips: no per-pair gather (``MWDiem.py:847-903``), no pandas history table,
no per-step kernel compilation.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _dev
from ._lib import (HULL_CAP, ST_PAIR_OVERFLOW, ContactParams, Material, MwdError, Scene, State, Work, check, lib,
                   status_names)
from .scene import SceneSpec

_STATE_F64 = ("pos", "dx_all", "wall_normal")
_STATE_F32 = ("vel", "vel_half", "w_half_bf", "w_bf", "w", "q", "q_half", "q_all", "q_acc", "force", "torque",
              "ext_force", "ext_torque", "inertia", "inv_inertia")


def _trunc(x):
    return int(np.trunc(x))


@dataclass
class Layout:
    row_begin: list
    wall_end: list
    row_end: list


class Simulator:
    def __init__(self, scenes, lanes=8, pair_cap=None, device="cuda", collect_collisions=False, two_pass=True,
                 cull_pairs=True):
        _dev.require_cuda()
        if isinstance(scenes, SceneSpec):
            scenes = [scenes]
        self.specs = list(scenes)
        self.lanes = int(lanes)
        self.device = torch.device(device)
        self._build_state()
        self._build_scenes()
        self.two_pass = bool(two_pass)
        self.cull_pairs = bool(cull_pairs)
        self._build_work(pair_cap, collect_collisions)
        self.graph = None
        self.graph_steps = 0
        self.steps_done = 0

    # ------------------------------------------------------------------ set-up
    def _build_state(self):
        rows_pos, rows_nrm, rows_vel, rows_inertia, rows_inv, rows_ext, info = [], [], [], [], [], [], []
        verts, counts = [], []
        rb, we, re = [], [], []
        row = 0
        for s_id, sp in enumerate(self.specs):
            rb.append(row)
            for b, c, nrm in sp.walls:
                rows_pos.append(c)
                rows_nrm.append(nrm)
                rows_vel.append(np.zeros(3))
                I = np.asarray(b.inertia_bf, dtype=np.float64)
                rows_inertia.append([I[0], I[1], I[2], b.inertia_size])
                rows_inv.append([1 / I[0], 1 / I[1], 1 / I[2], 1 / b.mass])
                rows_ext.append(np.zeros(3))
                info.append((s_id << 1) | 1)
                verts.append(b.vertices)
                counts.append(b.vertices.shape[0])
                row += 1
            we.append(row)
            g = np.asarray(sp.gravity, dtype=np.float64)
            vel = sp.velocities if sp.velocities is not None else np.zeros((sp.n_particles, 3))
            for k, b in enumerate(sp.bodies):
                rows_pos.append(sp.centres[k])
                rows_nrm.append(np.zeros(3))
                rows_vel.append(vel[k])
                I = np.asarray(b.inertia_bf, dtype=np.float64)
                rows_inertia.append([I[0], I[1], I[2], b.inertia_size])
                rows_inv.append([1 / I[0], 1 / I[1], 1 / I[2], 1 / b.mass])
                rows_ext.append(b.mass * g)
                info.append(s_id << 1)
                verts.append(b.vertices)
                counts.append(b.vertices.shape[0])
                row += 1
            re.append(row)
        n = row
        self.layout = Layout(rb, we, re)
        self.n = n
        counts = np.asarray(counts, dtype=np.int64)
        if counts.max() > HULL_CAP:
            raise ValueError(f"a shape has {counts.max()} vertices; the narrow phase stages at most {HULL_CAP}")
        off = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(counts, out=off[1:])
        self.vert_off_host = off
        self.max_verts = int(counts.max())
        bv = np.zeros((int(off[-1]), 4), dtype=np.float32)
        bv[:, :3] = np.concatenate(verts, 0)
        pos = np.zeros((n, 4))
        pos[:, :3] = np.asarray(rows_pos)
        # bounding radius of each row (used by the narrow phase's sphere pre-test)
        pos[:, 3] = [float(np.sqrt((v.astype(np.float32).astype(np.float64) ** 2).sum(1)).max()) for v in verts]
        f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(self.device)  # noqa: E731
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(self.device)  # noqa: E731
        z4 = np.zeros((n, 4))
        qid = np.tile([1.0, 0.0, 0.0, 0.0], (n, 1))
        vel4 = np.zeros((n, 4))
        vel4[:, :3] = np.asarray(rows_vel)
        nrm4 = np.zeros((n, 4))
        nrm4[:, :3] = np.asarray(rows_nrm)
        ext4 = np.zeros((n, 4))
        ext4[:, :3] = np.asarray(rows_ext)
        t = {}
        t["pos"] = f64(pos)
        t["dx_all"] = f64(z4)
        t["wall_normal"] = f64(nrm4)
        t["vel"] = f32(vel4)
        t["vel_half"] = f32(vel4)
        for k in ("w_half_bf", "w_bf", "w", "force", "torque", "ext_torque"):
            t[k] = f32(z4)
        for k in ("q", "q_half", "q_all", "q_acc"):
            t[k] = f32(qid)
        t["ext_force"] = f32(ext4)
        t["inertia"] = f32(np.asarray(rows_inertia))
        t["inv_inertia"] = f32(np.asarray(rows_inv))
        t["info"] = torch.from_numpy(np.asarray(info, dtype=np.int32)).to(self.device)
        t["vert_off"] = torch.from_numpy(off.astype(np.int32)).to(self.device)
        t["body_verts"] = f32(bv)
        wv = bv.copy()
        owner = np.repeat(np.arange(n), counts)
        wv[:, :3] = (pos[owner, :3] + bv[:, :3].astype(np.float64)).astype(np.float32)
        t["world_verts"] = f32(wv)
        self.t = t
        st = State()
        for k in _STATE_F64 + _STATE_F32 + ("info", "vert_off", "body_verts", "world_verts"):
            setattr(st, k, t[k].data_ptr())
        st.n = n
        st.n_verts = int(off[-1])
        st.max_verts = self.max_verts
        self.state = st

    def _build_scenes(self):
        S = len(self.specs)
        arr = (Scene * S)()
        base = 0
        for i, sp in enumerate(self.specs):
            sc = arr[i]
            ncell, cs = sp.grid()
            box = sp.box()
            for a in range(3):
                sc.cs[a] = float(cs[a])
            for a in range(6):
                sc.box[a] = float(box[a])
            sc.dt = float(sp.dt)
            sc.wall_range = 6.0 * float(sp.max_particlesize)
            nx, ny = int(ncell[0]), int(ncell[1])
            sc.nx, sc.ny = nx, ny
            lo = [_trunc(box[1] / cs[0]), _trunc(box[3] / cs[1]), _trunc(box[5] / cs[2])]
            hi = [_trunc(box[0] / cs[0]), _trunc(box[2] / cs[1]), _trunc(box[4] / cs[2])]
            kmin = lo[0] + lo[1] * nx + lo[2] * nx * ny
            kmax = hi[0] + hi[1] * nx + hi[2] * nx * ny
            sc.key_min = kmin
            sc.n_keys = kmax - kmin + 1
            sc.cell_base = base
            base += sc.n_keys
            sc.row_begin, sc.wall_end, sc.row_end = self.layout.row_begin[i], self.layout.wall_end[i], \
                self.layout.row_end[i]
            sc.law = ContactParams(float(sp.Kn), float(sp.en), float(sp.et), float(sp.mu), float(sp.Kn_wall),
                                   float(sp.en_wall), float(sp.et_wall), float(sp.mu_wall), float(sp.dt),
                                   int(sp.n_walls), 0, self.lanes, 0)
            check(lib().mwd_derive_material(C.byref(sc.law), sc.mat))
        self.scenes_host = arr
        self.total_cells = base
        raw = bytes(C.string_at(C.addressof(arr), C.sizeof(arr)))
        self.scenes_dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.device)

    def _build_work(self, pair_cap, collect_collisions):
        n = self.n
        n_part = sum(sp.n_particles for sp in self.specs)
        cap = int(pair_cap) if pair_cap else max(4096, 16 * n_part)
        i32 = dict(dtype=torch.int32, device=self.device)
        w = {}
        w["cell_count"] = torch.zeros(max(self.total_cells, 1), **i32)
        w["cell_start"] = torch.zeros(self.total_cells + 1, **i32)
        w["cell_of"] = torch.zeros(n, **i32)
        w["sorted"] = torch.zeros(n, **i32)
        w["pair_count"] = torch.zeros(n + 1, **i32)
        w["pairs"] = torch.zeros((cap, 2), **i32)
        w["scan_tmp"] = torch.zeros(int(lib().mwd_scan_tmp_ints(max(self.total_cells, n) + 1)), **i32)
        w["n_pairs"] = torch.zeros(1, dtype=torch.int64, device=self.device)
        w["status"] = torch.zeros(1, **i32)
        w["collision"] = torch.zeros(cap, **i32) if collect_collisions else None
        crowded_cap = n // 33 + 1
        w["crowded"] = torch.zeros(crowded_cap + 1, **i32)
        self.w = w
        wk = Work()
        for k in ("cell_count", "cell_start", "cell_of", "sorted", "pair_count", "pairs", "scan_tmp", "n_pairs",
                  "status"):
            setattr(wk, k, w[k].data_ptr())
        wk.collision = w["collision"].data_ptr() if w["collision"] is not None else None
        wk.n_crowded = w["crowded"].data_ptr()
        wk.crowded = w["crowded"].data_ptr() + 4
        wk.crowded_cap = crowded_cap
        w["work_counters"] = torch.zeros(3, dtype=torch.int64, device=self.device)
        wk.work_counters = None
        if self.two_pass:
            w["epa_count"] = torch.zeros(1, **i32)
            w["epa_rec"] = torch.zeros(cap * 80, dtype=torch.uint8, device=self.device)
            wk.epa_count = w["epa_count"].data_ptr()
            wk.epa_rec = w["epa_rec"].data_ptr()
            wk.epa_cap = cap
        wk.cull_pairs = 1 if self.cull_pairs else 0
        w["sorted_pos"] = torch.zeros((n, 4), dtype=torch.float32, device=self.device)
        w["sorted_cell"] = torch.zeros(n, **i32)
        wk.sorted_pos = w["sorted_pos"].data_ptr()
        wk.sorted_cell = w["sorted_cell"].data_ptr()
        wk.total_cells = self.total_cells
        wk.pair_cap = cap
        self.work = wk
        self.pair_cap = cap

    # ------------------------------------------------------------------ stepping
    def step(self, n_steps=1, stream=None):
        s = _dev.stream_handle(stream)
        check(lib().mwd_step(C.byref(self.state), self.scenes_dev.data_ptr(), C.addressof(self.scenes_host),
                             len(self.specs), C.byref(self.work), self.lanes, int(n_steps), s))
        self.steps_done += n_steps

    def broadphase(self, stream=None):
        check(lib().mwd_broadphase(C.byref(self.state), self.scenes_dev.data_ptr(), C.addressof(self.scenes_host),
                                   len(self.specs), C.byref(self.work), _dev.stream_handle(stream)))

    def narrow_force(self, stream=None):
        check(lib().mwd_narrow_force(C.byref(self.state), self.scenes_dev.data_ptr(), C.byref(self.work),
                                     self.lanes, _dev.stream_handle(stream)))

    def count_narrow_work(self, stream=None):
        """Run one narrow phase with work counting on: returns (vertex dot products, EPA faces,
        support queries) of the current pair list.  Forces are accumulated as by narrow_force."""
        self.w["work_counters"].zero_()
        self.work.work_counters = self.w["work_counters"].data_ptr()
        try:
            self.narrow_force(stream)
        finally:
            self.work.work_counters = None
        c = self.w["work_counters"].cpu().numpy()
        return int(c[0]), int(c[1]), int(c[2])

    def integrate(self, stream=None):
        check(lib().mwd_integrate(C.byref(self.state), self.scenes_dev.data_ptr(), self.w["status"].data_ptr(),
                                  _dev.stream_handle(stream)))

    def capture(self, steps_per_replay=1):
        """Capture `steps_per_replay` steps in one CUDA graph (warm-up step first, outside capture)."""
        self.step(1)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            check(lib().mwd_step(C.byref(self.state), self.scenes_dev.data_ptr(), C.addressof(self.scenes_host),
                                 len(self.specs), C.byref(self.work), self.lanes, int(steps_per_replay),
                                 _dev.stream_handle()))
        self.graph = g
        self.graph_steps = int(steps_per_replay)
        return g

    def replay(self, n=1):
        for _ in range(n):
            self.graph.replay()
        self.steps_done += n * self.graph_steps

    # ------------------------------------------------------------------ host-resident state
    MUTABLE = ("pos", "dx_all", "vel", "vel_half", "w_half_bf", "w_bf", "w", "q", "q_half", "q_all", "q_acc")

    def host_state(self):
        """Pinned host copies of the state the step updates (what a caller holding its state in host
        memory, as the reference does, passes in and gets back)."""
        return {k: self.t[k].cpu().pin_memory() for k in self.MUTABLE}

    def host_state_bytes(self):
        return sum(self.t[k].numel() * self.t[k].element_size() for k in self.MUTABLE)

    def step_host(self, host, n_steps=1, stream=None):
        """Copy `host` (pinned) to the device, run n_steps, copy the state back into `host`.
        Uses the captured graph when there is one (and n_steps is a multiple of its length)."""
        for k in self.MUTABLE:
            self.t[k].copy_(host[k], non_blocking=True)
        if self.graph is not None and n_steps % self.graph_steps == 0:
            self.replay(n_steps // self.graph_steps)
        else:
            self.step(n_steps, stream)
        for k in self.MUTABLE:
            host[k].copy_(self.t[k], non_blocking=True)
        return host

    # ------------------------------------------------------------------ inspection
    def status(self) -> int:
        return int(self.w["status"].item()) & 0xffffffff

    def check_status(self, allow=0):
        st = self.status() & ~allow
        if st & ST_PAIR_OVERFLOW:
            raise MwdError(3, f"pair buffer overflow (capacity {self.pair_cap}); status {status_names(st)}")
        return st

    def n_pairs(self) -> int:
        return int(self.w["n_pairs"].item())

    def pairs(self):
        return self.w["pairs"][: self.n_pairs()]

    def particle_rows(self, scene=0):
        return slice(self.layout.wall_end[scene], self.layout.row_end[scene])

    def positions(self, scene=None):
        p = self.t["pos"][:, :3]
        if scene is not None:
            p = p[self.particle_rows(scene)]
        return p

    def world_vertices_padded(self, V):
        """(n, V, 3) float32 world vertices padded with zeros, like the reference's per-pair gather."""
        off = self.vert_off_host
        wv = self.t["world_verts"].cpu().numpy()
        out = np.zeros((self.n, V, 3), dtype=np.float32)
        for r in range(self.n):
            k = off[r + 1] - off[r]
            out[r, :k] = wv[off[r]:off[r + 1], :3]
        return out

    def reference_state(self):
        """State as the reference's FP64 arrays (MWDiem.py:603-631) plus per-row vertex counts."""
        t = {k: v.cpu().numpy() for k, v in self.t.items()}
        d = dict(com=t["pos"][:, :3].copy(), dxall=t["dx_all"][:, :3].copy(), v=t["vel"][:, :3].astype(np.float64),
                 v12=t["vel_half"][:, :3].astype(np.float64), w12bf=t["w_half_bf"][:, :3].astype(np.float64),
                 wbf=t["w_bf"][:, :3].astype(np.float64), w=t["w"][:, :3].astype(np.float64),
                 q=t["q"].astype(np.float64), q12=t["q_half"].astype(np.float64), qall=t["q_all"].astype(np.float64))
        return d
