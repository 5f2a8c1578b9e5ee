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
from ._lib import (CELL_TABLE_AUTO, CELL_TABLE_COMPRESSED, CELL_TABLE_DENSE, EPA_COUNT_INTS, HULL_CAP, INFO_INACTIVE,
                   LAW_PHYSICAL, LAW_REFERENCE, ST_PAIR_OVERFLOW, ContactParams, Inlet, Material, MwdError, Scene,
                   State, Work, check, lib, status_names)
from .scene import CompactBodies, SceneSpec

CONTACT_LAWS = {"reference": LAW_REFERENCE, "physical": LAW_PHYSICAL}

_STATE_F64 = ("pos", "dx_all", "wall_normal")
_STATE_F32 = ("vel", "vel_half", "w_half_bf", "w_bf", "w", "q", "q_half", "q_all", "q_acc", "force", "torque",
              "ext_force", "ext_torque", "inertia", "inv_inertia")


def _trunc(x):
    return int(np.trunc(x))


@dataclass
class InletSpec:
    """Particles entering during the run (MWDiem.py:685-714): the first `initial` particle rows of the
    scene are there from the start; the others wait and enter `per_spawn` at a time every `period`
    steps, at rest, at a point drawn uniformly (seeded) from the box `lo`..`hi`."""
    period: int = 5
    per_spawn: int = 1
    initial: int = 0
    lo: tuple = (0.0, 0.0, 0.0)
    hi: tuple = (0.0, 0.0, 0.0)
    seed: int = 0


@dataclass
class Layout:
    row_begin: list
    wall_end: list
    row_end: list


class Simulator:
    def __init__(self, scenes, lanes=8, pair_cap=None, device="cuda", collect_collisions=False, two_pass=True,
                 cull_pairs=True, deterministic=False, persistent_history=False, inlet=None, cell_table="auto"):
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
        self.deterministic = bool(deterministic)
        self.persistent_history = bool(persistent_history)
        # the broad phase's cell table: "dense" (a count and a start per cell), "compressed" (a bit per
        # cell, counts and starts per occupied cell, where it fits: on a sparse domain a small fraction
        # of the dense table's memory), or "auto" (dense, the faster of the two on every workload
        # measured, up to 2^27 cells; compressed beyond, where it fits): the same pairs either way
        tables = {"auto": CELL_TABLE_AUTO, "dense": CELL_TABLE_DENSE, "compressed": CELL_TABLE_COMPRESSED}
        if cell_table not in tables:
            raise ValueError(f"cell_table must be one of {sorted(tables)}")
        self.cell_table = tables[cell_table]
        compressed = lib().mwd_cell_table(self.n, self.total_cells, self.cell_table) == 2
        self.cell_table_in_use = "compressed" if compressed else "dense"
        if (self.deterministic or self.persistent_history) and not self.two_pass:
            raise ValueError("deterministic accumulation and persistent history need the two-pass narrow phase")
        self._build_work(pair_cap, collect_collisions)
        self.inlet = None
        if inlet is not None:
            self._build_inlet(inlet)
        self.graph = None
        self.graph_steps = 0
        self.host_graph = None
        self.host_graph_buffer = None
        self.steps_done = 0

    # ------------------------------------------------------------------ set-up
    def _build_state(self):
        """Row arrays of every scene (walls, then particles), concatenated; vertex tables in CSR.
        Explicit bodies are assembled on the host; CompactBodies are rotated on the device."""
        dev = self.device
        parts = []          # per scene: dict of row arrays
        explicit = []       # (global row, vertices (k,3))
        compact = []        # (global rows (m,), pool id, pick (m,), quats (m,4))
        pools = {}
        rb, we, re = [], [], []
        row = 0
        for s_id, sp in enumerate(self.specs):
            rb.append(row)
            W = len(sp.walls)
            n_p = sp.n_particles
            g = np.asarray(sp.gravity, dtype=np.float64)
            wall_I = np.array([np.asarray(b.inertia_bf, float) for b, _, _ in sp.walls]).reshape(W, 3)
            wall_size = np.array([b.inertia_size for b, _, _ in sp.walls])
            wall_mass = np.array([b.mass for b, _, _ in sp.walls])
            wall_cnt = np.array([b.vertices.shape[0] for b, _, _ in sp.walls], dtype=np.int64)
            wall_rad = np.array([np.sqrt((b.vertices.astype(np.float32).astype(np.float64) ** 2).sum(1)).max()
                                 for b, _, _ in sp.walls])
            for k, (b, _, _) in enumerate(sp.walls):
                explicit.append((row + k, b.vertices))
            cb = sp.bodies
            q0 = np.tile([1.0, 0.0, 0.0, 0.0], (n_p, 1))
            if sp.law == "physical":  # principal-axes body frames (SceneSpec.principal_bodies)
                cb, q0 = sp.principal_bodies()
            if isinstance(cb, CompactBodies):
                key = id(cb.pool)
                if key not in pools:
                    pools[key] = cb.pool
                pick = np.asarray(cb.pick, dtype=np.int64)
                pm = np.array([b.mass for b in cb.pool])
                pI = np.array([np.asarray(b.inertia_bf, float) for b in cb.pool])
                ps = np.array([b.inertia_size for b in cb.pool])
                pc = np.array([b.vertices.shape[0] for b in cb.pool], dtype=np.int64)
                pr = np.array([np.sqrt((b.vertices.astype(np.float32).astype(np.float64) ** 2).sum(1)).max()
                               for b in cb.pool])
                p_mass, p_I, p_size, p_cnt, p_rad = pm[pick], pI[pick], ps[pick], pc[pick], pr[pick]
                compact.append((np.arange(row + W, row + W + n_p), key, pick, np.asarray(cb.quats, float)))
            else:
                bl = list(cb)
                p_mass = np.array([b.mass for b in bl])
                p_I = np.array([np.asarray(b.inertia_bf, float) for b in bl]).reshape(n_p, 3)
                p_size = np.array([b.inertia_size for b in bl])
                p_cnt = np.array([b.vertices.shape[0] for b in bl], dtype=np.int64)
                p_rad = np.array([np.sqrt((b.vertices.astype(np.float32).astype(np.float64) ** 2).sum(1)).max()
                                  for b in bl])
                for k, b in enumerate(bl):
                    explicit.append((row + W + k, b.vertices))
            vel = sp.velocities if sp.velocities is not None else np.zeros((n_p, 3))
            parts.append(dict(
                pos=np.concatenate([np.array([c for _, c, _ in sp.walls]).reshape(W, 3), np.asarray(sp.centres)]),
                nrm=np.concatenate([np.array([nn for _, _, nn in sp.walls]).reshape(W, 3), np.zeros((n_p, 3))]),
                vel=np.concatenate([np.zeros((W, 3)), np.asarray(vel, float)]),
                I=np.concatenate([wall_I, p_I]), size=np.concatenate([wall_size, p_size]),
                mass=np.concatenate([wall_mass, p_mass]),
                ext=np.concatenate([np.zeros((W, 3)), p_mass[:, None] * g[None, :]]),
                info=np.concatenate([np.full(W, (s_id << 1) | 1), np.full(n_p, s_id << 1)]).astype(np.int32),
                cnt=np.concatenate([wall_cnt, p_cnt]), rad=np.concatenate([wall_rad, p_rad]),
                q0=np.concatenate([np.tile([1.0, 0.0, 0.0, 0.0], (W, 1)), q0])))
            row += W
            we.append(row)
            row += n_p
            re.append(row)
        n = row
        self.layout = Layout(rb, we, re)
        self.n = n
        cat = {k: np.concatenate([pt[k] for pt in parts]) for k in parts[0]}
        counts = cat["cnt"].astype(np.int64)
        if counts.max() > HULL_CAP:
            raise ValueError(f"a shape has {counts.max()} vertices; the narrow phase stages at most {HULL_CAP}")
        off = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(counts, out=off[1:])
        self.vert_off_host = off
        self.max_verts = int(counts.max())
        total = int(off[-1])
        f32 = dict(dtype=torch.float32, device=dev)
        off_d = torch.from_numpy(off).to(dev)
        counts_d = torch.from_numpy(counts).to(dev)
        body = torch.zeros((total, 4), **f32)
        if explicit:
            rows_e = np.array([r for r, _ in explicit], dtype=np.int64)
            vals = np.concatenate([v for _, v in explicit], 0).astype(np.float32)
            idx = _ranges(off_d[torch.from_numpy(rows_e).to(dev)], counts_d[torch.from_numpy(rows_e).to(dev)])
            body[idx, :3] = torch.from_numpy(vals).to(dev)
        for rows_c, key, pick, quats in compact:
            pool = pools[key]
            Vp = max(b.vertices.shape[0] for b in pool)
            pv = np.zeros((len(pool), Vp, 3), np.float32)
            for i, b in enumerate(pool):
                pv[i, :b.vertices.shape[0]] = b.vertices
            pv_d = torch.from_numpy(pv).to(dev)
            rows_t = torch.from_numpy(rows_c).to(dev)
            pick_t = torch.from_numpy(pick).to(dev)
            q_t = torch.from_numpy(quats.astype(np.float32)).to(dev)
            chunk = 1 << 18
            for a0 in range(0, len(rows_c), chunk):
                a1 = min(len(rows_c), a0 + chunk)
                R = _quat_to_matrix(q_t[a0:a1])
                v = torch.einsum("rij,rkj->rki", R, pv_d[pick_t[a0:a1]])
                c = counts_d[rows_t[a0:a1]]
                mask = torch.arange(Vp, device=dev)[None, :] < c[:, None]
                idx = _ranges(off_d[rows_t[a0:a1]], c)
                body[idx, :3] = v[mask]
        pos = np.zeros((n, 4))
        pos[:, :3] = cat["pos"]
        pos[:, 3] = cat["rad"]  # bounding radius (used by the narrow phase's sphere test)
        I = cat["I"]
        inertia = np.concatenate([I, cat["size"][:, None]], 1)
        inv = np.concatenate([1.0 / I, 1.0 / cat["mass"][:, None]], 1)
        # FP64 row constants and initial values (the differentiable step computes in FP64)
        self.row_data = dict(inertia=inertia, inv_inertia=inv, ext=cat["ext"], pos=cat["pos"], vel=cat["vel"],
                             info=cat["info"])
        z4 = torch.zeros((n, 4), **f32)
        t = {}
        t["pos"] = torch.from_numpy(pos).to(dev)
        t["dx_all"] = torch.zeros((n, 4), dtype=torch.float64, device=dev)
        nrm4 = np.zeros((n, 4))
        nrm4[:, :3] = cat["nrm"]
        t["wall_normal"] = torch.from_numpy(nrm4).to(dev)
        vel4 = np.zeros((n, 4), np.float32)
        vel4[:, :3] = cat["vel"]
        t["vel"] = torch.from_numpy(vel4).to(dev)
        t["vel_half"] = t["vel"].clone()
        for k in ("w_half_bf", "w_bf", "w", "force", "torque", "ext_torque"):
            t[k] = z4.clone()
        qid = torch.zeros((n, 4), **f32)
        qid[:, 0] = 1.0
        t["q_all"] = qid
        q0 = torch.from_numpy(cat["q0"].astype(np.float32)).to(dev)  # identity unless a principal frame
        for k in ("q", "q_half", "q_acc"):
            t[k] = q0.clone()
        ext4 = np.zeros((n, 4), np.float32)
        ext4[:, :3] = cat["ext"]
        t["ext_force"] = torch.from_numpy(ext4).to(dev)
        t["inertia"] = torch.from_numpy(inertia.astype(np.float32)).to(dev)
        t["inv_inertia"] = torch.from_numpy(inv.astype(np.float32)).to(dev)
        t["info"] = torch.from_numpy(cat["info"]).to(dev)
        t["vert_off"] = off_d.to(torch.int32)
        t["body_verts"] = body
        owner = torch.repeat_interleave(torch.arange(n, device=dev), counts_d)
        # world vertices: written below by the device's own transform (as every step writes them)
        world = body.clone()
        t["world_verts"] = world
        # the integrator's vertex pass: one thread per vertex, through each row's transform
        t["vert_owner"] = owner.to(torch.int32)
        t["xform"] = torch.zeros((n, 16), **f32)
        # the state a step updates, in one contiguous buffer: a host round trip of it is then one copy
        # each way (step_host)
        nbytes = sum(t[k].numel() * t[k].element_size() for k in self.MUTABLE)
        buf = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        off = 0
        for k in self.MUTABLE:
            v = t[k]
            b = v.numel() * v.element_size()
            view = buf[off:off + b].view(v.dtype).view(v.shape)
            view.copy_(v)
            t[k] = view
            off += b
        self.mutable = buf
        self.t = t
        st = State()
        for k in _STATE_F64 + _STATE_F32 + ("info", "vert_off", "body_verts", "world_verts", "vert_owner", "xform"):
            setattr(st, k, t[k].data_ptr())
        st.n = n
        st.n_verts = total
        st.max_verts = self.max_verts
        self.state = st
        # world = pos + R(q_acc) r0 with the integrator's arithmetic, so that the first step sees the
        # vertices every later step sees (q_acc is the principal-frame orientation q0 under the
        # physical law, identity otherwise)
        check(lib().mwd_refresh_vertices(C.byref(st), _dev.stream_handle()))

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
            for k in range(3):
                sc.inv_cs[k] = float(np.float32(1.0 / cs[k]))
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
            if sp.law not in CONTACT_LAWS:
                raise ValueError(f"unknown contact law {sp.law!r}; expected one of {sorted(CONTACT_LAWS)}")
            sc.law.law = CONTACT_LAWS[sp.law]
            check(lib().mwd_derive_material(C.byref(sc.law), sc.mat))
        self.scenes_host = arr
        if base > (1 << 31) - 64:
            raise ValueError(f"{base} cells: the cell tables index cells with 32-bit integers (at most 2^31 - 64)")
        self.total_cells = base
        raw = bytes(C.string_at(C.addressof(arr), C.sizeof(arr)))
        self.scenes_dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.device)

    def _build_work(self, pair_cap, collect_collisions):
        n = self.n
        n_part = sum(sp.n_particles for sp in self.specs)
        # default capacity: the bounding-sphere filter keeps a few candidates per particle; the
        # reference's full list (8-cell stencil, walls) holds up to ~30 per particle in dense packing
        cap = int(pair_cap) if pair_cap else max(4096, (16 if self.cull_pairs else 40) * n_part)
        i32 = dict(dtype=torch.int32, device=self.device)
        w = {}
        # the cell table's arrays: a count and a start per cell, or the compressed table's smaller ones
        cnt_ints, start_ints = C.c_int64(), C.c_int64()
        lib().mwd_cell_table_ints(n, self.total_cells, self.cell_table, C.byref(cnt_ints), C.byref(start_ints))
        w["cell_count"] = torch.zeros(max(int(cnt_ints.value), 1), **i32)
        w["cell_start"] = torch.zeros(int(start_ints.value), **i32)
        w["cell_of"] = torch.zeros(n, **i32)
        w["sorted"] = torch.zeros(n, **i32)
        w["pair_count"] = torch.zeros(n + 1, **i32)
        w["pairs"] = torch.zeros((cap, 2), **i32)
        w["scan_tmp"] = torch.zeros(int(lib().mwd_scan_tmp_ints(max(self.total_cells, n) + 1)), **i32)
        w["n_pairs"] = torch.zeros(1, dtype=torch.int64, device=self.device)
        w["status"] = torch.zeros(1, **i32)
        w["collision"] = torch.zeros(cap, **i32) if collect_collisions else None
        self.w = w
        wk = Work()
        for k in ("cell_count", "cell_start", "cell_of", "sorted", "pair_count", "pairs", "scan_tmp", "n_pairs",
                  "status"):
            setattr(wk, k, w[k].data_ptr())
        wk.collision = w["collision"].data_ptr() if w["collision"] is not None else None
        w["work_counters"] = torch.zeros(3, dtype=torch.int64, device=self.device)
        wk.work_counters = None
        if self.two_pass:
            w["epa_count"] = torch.zeros(EPA_COUNT_INTS, **i32)
            w["epa_rec"] = torch.zeros(cap * 80, dtype=torch.uint8, device=self.device)
            wk.epa_count = w["epa_count"].data_ptr()
            wk.epa_rec = w["epa_rec"].data_ptr()
            wk.epa_cap = cap
        wk.cull_pairs = 1 if self.cull_pairs else 0
        wk.cell_table = self.cell_table
        w["sorted_pos"] = torch.zeros((n, 4), dtype=torch.float32, device=self.device)
        w["sorted_cell"] = torch.zeros(n, **i32)
        wk.sorted_pos = w["sorted_pos"].data_ptr()
        wk.sorted_cell = w["sorted_cell"].data_ptr()
        if self.persistent_history:
            hcap = 1 << max(10, int(2 * cap - 1).bit_length())  # power of two >= 2 x the contact capacity
            w["hist_keys"] = torch.zeros(2 * hcap, dtype=torch.int64, device=self.device)
            w["hist_vals"] = torch.zeros((2 * hcap, 4), dtype=torch.float32, device=self.device)
            w["hist_parity"] = torch.zeros(1, **i32)
            wk.hist_cap = hcap
            wk.hist_keys = w["hist_keys"].data_ptr()
            wk.hist_vals = w["hist_vals"].data_ptr()
            wk.hist_parity = w["hist_parity"].data_ptr()
        if self.deterministic:
            nb = int(lib().mwd_det_scratch_bytes(n, cap))
            w["det_scratch"] = torch.zeros(nb, dtype=torch.uint8, device=self.device)
            wk.deterministic = 1
            wk.det_scratch = w["det_scratch"].data_ptr()
        wk.total_cells = self.total_cells
        wk.pair_cap = cap
        self.work = wk
        self.pair_cap = cap

    def _build_inlet(self, spec: InletSpec):
        if len(self.specs) != 1:
            raise ValueError("the inlet is for a single scene")
        if spec.period < 1 or spec.per_spawn < 0:
            raise ValueError("inlet period must be >= 1 and per_spawn >= 0")
        w0, r1 = self.layout.wall_end[0], self.layout.row_end[0]
        first = w0 + int(spec.initial)
        if first > r1:
            raise ValueError("more initial particles than the scene has")
        rng = np.random.default_rng(spec.seed)
        sp = np.zeros((self.n, 4))
        lo, hi = np.asarray(spec.lo, float), np.asarray(spec.hi, float)
        sp[first:r1, :3] = lo + rng.random((r1 - first, 3)) * (hi - lo)
        dev = self.device
        info = self.t["info"]
        info[first:r1] = info[first:r1] | INFO_INACTIVE
        self.inlet_t = {"spawn_pos": torch.from_numpy(sp).to(dev),
                        "next_row": torch.tensor([first], dtype=torch.int32, device=dev),
                        "step": torch.zeros(1, dtype=torch.int32, device=dev)}
        st = Inlet()
        st.period, st.per_spawn, st.row_end = int(spec.period), int(spec.per_spawn), int(r1)
        st.next_row = self.inlet_t["next_row"].data_ptr()
        st.step = self.inlet_t["step"].data_ptr()
        st.spawn_pos = self.inlet_t["spawn_pos"].data_ptr()
        self.inlet = st
        self.work.inlet = C.addressof(st)

    def active_rows(self):
        """Boolean (n,) mask of the rows in the domain (walls included)."""
        return (self.t["info"] & INFO_INACTIVE) == 0

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

    def integrate_rows(self, stream=None):
        """The integrator's row pass alone (the state is final after it; world vertices follow from
        world_vertices())."""
        check(lib().mwd_integrate_rows(C.byref(self.state), self.scenes_dev.data_ptr(), self.w["status"].data_ptr(),
                                       _dev.stream_handle(stream)))

    def world_vertices(self, stream=None):
        check(lib().mwd_world_vertices(C.byref(self.state), _dev.stream_handle(stream)))

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
        """Pinned host copy of the state the step updates (what a caller holding its state in host
        memory, as the reference does, passes in and gets back): a dict of per-array views of one
        pinned buffer (key "_buffer"), laid out as the device buffer."""
        hb = self.mutable.cpu().pin_memory()
        host = {"_buffer": hb}
        off = 0
        for k in self.MUTABLE:
            v = self.t[k]
            b = v.numel() * v.element_size()
            host[k] = hb[off:off + b].view(v.dtype).view(v.shape)
            off += b
        return host

    def host_state_bytes(self):
        return int(self.mutable.numel())

    def step_host(self, host, n_steps=1, stream=None):
        """Copy `host` (pinned, from host_state) to the device, run n_steps, copy the state back into
        `host`: one copy each way.  One step on the `host` given to capture_host replays that graph;
        otherwise the step graph is used when there is one (and n_steps is a multiple of its length)."""
        if n_steps == 1 and self.host_graph is not None and host["_buffer"] is self.host_graph_buffer:
            self.host_graph.replay()
            self.steps_done += 1
            return host
        self.mutable.copy_(host["_buffer"], non_blocking=True)
        if self.graph is not None and n_steps % self.graph_steps == 0:
            self.replay(n_steps // self.graph_steps)
        else:
            self.step(n_steps, stream)
        host["_buffer"].copy_(self.mutable, non_blocking=True)
        return host

    def host_mapped(self, host):
        """Device address of the pinned buffer of `host` (from host_state), or None when the GPU cannot
        address it directly."""
        dp = C.c_void_p()
        rc = lib().mwd_host_mapped(C.c_void_p(host["_buffer"].data_ptr()), C.byref(dp))
        return dp.value if rc == 0 else None

    def capture_host(self, host, mirror=True):
        """Capture one step between the pinned buffers of `host` (from host_state) in one CUDA graph,
        replayed by step_host(host, 1).  The centres, the first array of the state, are copied in
        first and the broad phase (which reads no other array of the state) starts on them while the
        rest of the state is copied in on a second stream; the narrow phase waits for that copy.  The
        state returns to `host` during the integrator's row pass, which writes each updated row both to
        the device and to the host buffer (mwd_integrate_rows_mirror; `mirror`, and the buffer mapped
        for the device), or else by a copy after that pass, beside its vertex pass.  The same kernels as
        step(): the same results.  Not with an inlet (its rows enter inside mwd_step)."""
        if self.inlet is not None:
            raise ValueError("capture_host: the inlet runs inside mwd_step; use step_host without capture")
        hb = host["_buffer"]
        if hb.device.type != "cpu" or not hb.is_pinned() or hb.dtype != self.mutable.dtype or \
                hb.numel() != self.mutable.numel():
            raise ValueError("capture_host: `host` must come from this simulator's host_state()")
        mapped = self.host_mapped(host) if mirror else None
        self.step_host(host, 1)  # warm-up outside capture
        torch.cuda.synchronize()
        npos = self.t["pos"].numel() * self.t["pos"].element_size()
        side = torch.cuda.Stream(device=self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            main = torch.cuda.current_stream()
            self.mutable[:npos].copy_(hb[:npos], non_blocking=True)
            side.wait_stream(main)  # after the centres: one copy engine would otherwise take them second
            with torch.cuda.stream(side):
                self.mutable[npos:].copy_(hb[npos:], non_blocking=True)
            self.broadphase()
            main.wait_stream(side)
            self.narrow_force()
            if mapped is not None:
                check(lib().mwd_integrate_rows_mirror(C.byref(self.state), self.scenes_dev.data_ptr(),
                                                      self.w["status"].data_ptr(), C.c_void_p(mapped),
                                                      self.mutable.data_ptr(), self.mutable.numel(),
                                                      _dev.stream_handle()))
                self.world_vertices()
            else:
                self.integrate_rows()
                side.wait_stream(main)
                with torch.cuda.stream(side):
                    hb.copy_(self.mutable, non_blocking=True)
                self.world_vertices()
                main.wait_stream(side)
        self.host_graph = g
        self.host_graph_buffer = hb
        self.host_graph_mirrored = mapped is not None
        return g

    # ------------------------------------------------------------------ inspection
    def status(self) -> int:
        return int(self.w["status"].item()) & 0xffffffff

    def check_status(self, allow=0):
        st = self.status() & ~allow
        if st & ST_PAIR_OVERFLOW:
            raise MwdError(3, f"pair buffer overflow (capacity {self.pair_cap}); status {status_names(st)}")
        return st

    def nonfinite_rows(self) -> int:
        """Rows whose centre or velocity is not finite (they drop out of the cell table)."""
        p = self.t["pos"][:, :3]
        v = self.t["vel"][:, :3]
        return int((~torch.isfinite(p).all(1) | ~torch.isfinite(v).all(1)).sum().item())

    def history_table(self):
        """Persistent history the next narrow phase reads: {(lower row, higher row): (3,) float32
        tangential displacement in that orientation}."""
        if not self.persistent_history:
            return {}
        cap = self.work.hist_cap
        par = int(self.w["hist_parity"].item()) & 1
        keys = self.w["hist_keys"][par * cap:(par + 1) * cap].cpu().numpy().view(np.uint64)
        vals = self.w["hist_vals"][par * cap:(par + 1) * cap, :3].cpu().numpy()
        used = np.nonzero(keys)[0]
        return {(int(keys[i] >> np.uint64(32)), int(keys[i] & np.uint64(0xffffffff))): vals[i] for i in used}

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
        cnt = off[1:] - off[:-1]
        out = np.zeros((self.n, V, 3), dtype=np.float32)
        mask = np.arange(V)[None, :] < cnt[:, None]
        src = off[:-1][:, None] + np.arange(V)[None, :]
        out[mask] = wv[src[mask], :3]
        return out

    # ------------------------------------------------------------------ snapshots
    SNAPSHOT = MUTABLE + ("world_verts", "force", "torque", "info")

    def save(self, path):
        """Write the simulated state to an .npz file: every array a step updates, the world vertices,
        the force/torque accumulators, the row flags (an inlet activates rows), the inlet and
        persistent-history tables when present, and the step count.  Call between steps."""
        torch.cuda.synchronize()
        out = {k: self.t[k].cpu().numpy() for k in self.SNAPSHOT}
        out["steps_done"] = np.array(self.steps_done)
        if self.inlet is not None:
            for k in ("next_row", "step"):
                out["inlet_" + k] = self.inlet_t[k].cpu().numpy()
        if self.persistent_history:
            for k in ("hist_keys", "hist_vals", "hist_parity"):
                out[k] = self.w[k].cpu().numpy()
        np.savez(path, **out)

    def load(self, path):
        """Restore a snapshot written by save() into this simulator, built from the same scenes with
        the same options; a captured graph stays valid (the arrays are refilled in place)."""
        z = np.load(path)
        keys = list(self.SNAPSHOT)
        if self.inlet is not None:
            keys += ["inlet_next_row", "inlet_step"]
        if self.persistent_history:
            keys += ["hist_keys", "hist_vals", "hist_parity"]
        for k in keys:
            if k not in z.files:
                raise ValueError(f"snapshot {path} has no {k!r}: written by a simulator with other options")
            dst = (self.inlet_t[k[6:]] if k.startswith("inlet_") else
                   self.w[k] if k.startswith("hist_") else self.t[k])
            src = torch.from_numpy(z[k])
            if tuple(src.shape) != tuple(dst.shape) or src.dtype != dst.dtype:
                raise ValueError(f"snapshot array {k!r} is {tuple(src.shape)} {src.dtype}, this simulator's is "
                                 f"{tuple(dst.shape)} {dst.dtype}")
            dst.copy_(src)
        self.steps_done = int(z["steps_done"])
        self.w["status"].zero_()

    def reference_state(self):
        """State as the reference's FP64 arrays (MWDiem.py:603-631) plus per-row vertex counts."""
        t = {k: v.cpu().numpy() for k, v in self.t.items()}
        d = dict(com=t["pos"][:, :3].copy(), dxall=t["dx_all"][:, :3].copy(), v=t["vel"][:, :3].astype(np.float64),
                 v12=t["vel_half"][:, :3].astype(np.float64), w12bf=t["w_half_bf"][:, :3].astype(np.float64),
                 wbf=t["w_bf"][:, :3].astype(np.float64), w=t["w"][:, :3].astype(np.float64),
                 q=t["q"].astype(np.float64), q12=t["q_half"].astype(np.float64), qall=t["q_all"].astype(np.float64))
        return d


def _ranges(starts, counts):
    """Concatenation of arange(starts[i], starts[i] + counts[i]) (device tensors)."""
    total = int(counts.sum().item())
    if total == 0:
        return torch.zeros(0, dtype=torch.int64, device=starts.device)
    rep_start = torch.repeat_interleave(starts, counts)
    first = torch.cumsum(counts, 0) - counts
    within = torch.arange(total, device=starts.device) - torch.repeat_interleave(first, counts)
    return rep_start + within


def _quat_to_matrix(q):
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return torch.stack([torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], 1),
                        torch.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], 1),
                        torch.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1)], 1)
