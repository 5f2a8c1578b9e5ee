"""Differentiable rollout of one scene: an FP64 restatement of the device step with a hand-written
adjoint, behind ``torch.autograd.Function``.

Forward, per step (``libmwdem``; one CUDA graph replay per step after the first):

  FP32 broad phase + narrow phase on FP32 copies of the state (the contact topology: pairs in
  contact and the support vertices of each pair's final EPA face)  ->  ``mwd_diff_collect`` logs it
  ->  ``mwd_diff_force``: FP64 spring-dashpot + Coulomb force of the logged contacts (depth, normal
  and contact points re-evaluated from the face's support vertices)  ->  ``mwd_diff_integrate``: FP64
  leapfrog, centre of mass, a checkpoint every K steps, FP32 copies for the next detection.

Backward, per segment of K steps from the last: restore the checkpoint, recompute the K states
and forces from the logged topology (no detection), then apply ``mwd_diff_adjoint`` (transposed
integrator, then transposed contact force) from the last step of the segment to the first.

The topology is piecewise constant in the inputs, so the gradient is that of the step with the
forward's topology held fixed -- the derivative almost everywhere.  Differentiable inputs: the
FP64 state of every row (centres, velocities, angular velocities, quaternions; see ``DIFF_SLICES``)
and the law ``(2, 4)``: Kn, en, et, mu of particle pairs and of wall pairs.  Restitution enters the
law; ``law_from`` builds it from a damping ratio differentiably (MWDiem.py:87-96).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _dev
from ._lib import DIFF_ROW, DIFF_SLICES, ContactRec, Diff, MwdError, check, lib, status_names
from .sim import Simulator

ST_DIFF_FATAL = 128 | 256 | 512   # degenerate face, log overflow, fly-away reset


def law_from(kn, zeta, mu, kn_wall=None, zeta_wall=None, mu_wall=None):
    """(2,4) float64 law [[Kn, en, et, mu], [Kn_wall, en_wall, et_wall, mu_wall]] from damping ratios,
    en = et = exp(-pi zeta / sqrt(1 - zeta^2)); differentiable in every argument that is a tensor."""
    def t(v):
        return v if torch.is_tensor(v) else torch.tensor(float(v), dtype=torch.float64)
    kn, zeta, mu = t(kn), t(zeta), t(mu)
    kw = kn if kn_wall is None else t(kn_wall)
    zw = zeta if zeta_wall is None else t(zeta_wall)
    mw = mu if mu_wall is None else t(mu_wall)
    e = torch.exp(-math.pi * zeta / torch.sqrt(1.0 - zeta * zeta))
    ew = torch.exp(-math.pi * zw / torch.sqrt(1.0 - zw * zw))
    return torch.stack([torch.stack([kn, e, e, mu]), torch.stack([kw, ew, ew, mw])])


class DiffEngine:
    """Buffers and launches of the differentiable rollout of one scene.

    n_steps_max: the longest rollout; ckpt_every: K; rec_per_step: topology-log records reserved
    per step (default 8 per row, checked on the device: overflow raises); contact_point: the torque
    arm's contact point, "reference" = (cpA - cpB)/2 as gpu_fine_contact_detection.cu:677 computes
    it (about the origin, so the arm is about minus the centre's position) or "midpoint" =
    (cpA + cpB)/2."""

    def __init__(self, spec, n_steps_max, ckpt_every=100, lanes=8, rec_per_step=None, device="cuda",
                 use_graph=True, contact_point="reference"):
        _dev.require_cuda()
        self.sim = Simulator(spec, lanes=lanes, device=device, collect_collisions=True)
        sim = self.sim
        dev = sim.device
        self.device = dev
        self.n = sim.n
        self.n_walls = spec.n_walls
        self.n_particles = sim.n - spec.n_walls
        self.n_steps_max = int(n_steps_max)
        self.K = int(ckpt_every)
        rd = sim.row_data
        f64 = dict(dtype=torch.float64, device=dev)
        pad = lambda a: torch.from_numpy(np.concatenate([a, np.zeros((a.shape[0], 4 - a.shape[1]))], 1)).to(**f64) \
            if a.shape[1] < 4 else torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(**f64)  # noqa: E731
        self.inertia = pad(rd["inertia"])
        self.inv_inertia = pad(rd["inv_inertia"])
        self.ext = pad(rd["ext"])
        self.law = torch.zeros((2, 4), **f64)
        self.F = torch.zeros((self.n, 4), **f64)
        self.T = torch.zeros((self.n, 4), **f64)
        per = int(rec_per_step) if rec_per_step else max(1024, 8 * self.n)
        self.rec_cap = per * self.n_steps_max
        self.rec = torch.zeros((self.rec_cap, 8), dtype=torch.int32, device=dev)
        self.step_off = torch.zeros(self.n_steps_max + 1, dtype=torch.int64, device=dev)
        self.step_count = torch.zeros(self.n_steps_max, dtype=torch.int32, device=dev)
        self.t_dev = torch.zeros(1, dtype=torch.int32, device=dev)
        self.sync = torch.zeros(1, dtype=torch.int32, device=dev)
        self.com = torch.zeros((self.n_steps_max, 4), **f64)
        self.n_ckpt = self.n_steps_max // self.K + 1
        self.ckpt = torch.zeros((self.n_ckpt, self.n, DIFF_ROW), **f64)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.x = torch.zeros((self.n, DIFF_ROW), **f64)
        self.face_ids = torch.zeros((sim.pair_cap, 6), dtype=torch.int32, device=dev)
        sim.work.face_ids = self.face_ids.data_ptr()
        d = Diff()
        d.n, d.n_particles, d.n_steps, d.ckpt_every = self.n, self.n_particles, self.n_steps_max, self.K
        if contact_point not in ("reference", "midpoint"):
            raise ValueError("contact_point: 'reference' ((cpA - cpB)/2) or 'midpoint' ((cpA + cpB)/2)")
        d.contact_point = 1 if contact_point == "midpoint" else 0
        d.dt = float(spec.dt)
        for i, b in enumerate(spec.box()):
            d.box[i] = float(b)
        d.inertia, d.inv_inertia, d.ext = self.inertia.data_ptr(), self.inv_inertia.data_ptr(), self.ext.data_ptr()
        d.body_verts = sim.t["body_verts"].data_ptr()
        d.vert_off = sim.t["vert_off"].data_ptr()
        d.info = sim.t["info"].data_ptr()
        d.law, d.F, d.T = self.law.data_ptr(), self.F.data_ptr(), self.T.data_ptr()
        d.rec, d.rec_cap = self.rec.data_ptr(), self.rec_cap
        d.step_off, d.step_count = self.step_off.data_ptr(), self.step_count.data_ptr()
        d.t_dev, d.sync = self.t_dev.data_ptr(), self.sync.data_ptr()
        d.com, d.ckpt, d.status = self.com.data_ptr(), self.ckpt.data_ptr(), self.status.data_ptr()
        self.d = d
        self.spec = spec
        self.use_graph = bool(use_graph)
        self.graph = None
        self.generation = 0
        self.steps = 0
        self._bwd = None

    # ------------------------------------------------------------------ state
    def initial_state(self):
        """(n, 32) float64 state of the scene as built: centres, velocities (v and v_half), zero spins,
        identity quaternions (the orientation is baked into the body-frame vertices)."""
        rd = self.sim.row_data
        x = np.zeros((self.n, DIFF_ROW))
        x[:, DIFF_SLICES["c"]] = rd["pos"]
        x[:, DIFF_SLICES["v"]] = rd["vel"]
        x[:, DIFF_SLICES["v_half"]] = rd["vel"]
        for k in ("q", "q_half", "q_acc"):
            x[:, DIFF_SLICES[k].start] = 1.0
        return torch.from_numpy(x).to(self.device)

    def default_law(self):
        s = self.spec
        return torch.tensor([[s.Kn, s.en, s.et, s.mu], [s.Kn_wall, s.en_wall, s.et_wall, s.mu_wall]],
                            dtype=torch.float64, device=self.device)

    # ------------------------------------------------------------------ forward
    def _step_launches(self):
        """One forward step on the current stream (the capture stream while a graph is captured)."""
        sim = self.sim
        stream = _dev.stream_handle()
        sim.broadphase()
        sim.narrow_force()
        check(lib().mwd_diff_collect(C.byref(self.d), C.byref(sim.work), stream))
        check(lib().mwd_diff_force(C.byref(self.d), self.x.data_ptr(), -1, stream))
        check(lib().mwd_diff_integrate(C.byref(self.d), self.x.data_ptr(), self.x.data_ptr(), None,
                                       C.byref(sim.state), -1, stream))

    def forward(self, x0, law, n_steps):
        """Run n_steps from x0 with law; returns (com (n_steps,3), final state (n,32)) and keeps
        the checkpoints and the topology log for ``backward``."""
        if n_steps < 1 or n_steps > self.n_steps_max:
            raise ValueError(f"n_steps {n_steps} outside 1..{self.n_steps_max}")
        if x0.shape != (self.n, DIFF_ROW):
            raise ValueError(f"state shape {tuple(x0.shape)}, expected ({self.n}, {DIFF_ROW})")
        stream = _dev.stream_handle()
        self.law.copy_(law.detach().reshape(2, 4))
        self.x.copy_(x0.detach())
        self.ckpt[0].copy_(self.x)
        for buf in (self.step_count, self.step_off, self.t_dev, self.sync, self.com, self.status, self.F, self.T):
            buf.zero_()
        self.sim.w["status"].zero_()
        check(lib().mwd_diff_mirror(C.byref(self.d), self.x.data_ptr(), C.byref(self.sim.state), stream))
        self._step_launches()
        if n_steps > 1:
            if self.use_graph:
                if self.graph is None:
                    torch.cuda.synchronize()
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g):
                        self._step_launches()
                    self.graph = g
                for _ in range(n_steps - 1):
                    self.graph.replay()
            else:
                for _ in range(n_steps - 1):
                    self._step_launches()
        self.steps = int(n_steps)
        self.generation += 1
        self.check_status()
        return self.com[:n_steps, :3].clone(), self.x.clone()

    def check_status(self):
        st = int(self.status.item()) & 0xffffffff
        if st & 256:
            raise MwdError(3, f"topology log overflow (capacity {self.rec_cap} records); status {status_names(st)}")
        if st & 128:
            raise MwdError(3, f"a logged contact face has zero area; status {status_names(st)}")
        return st

    def status_word(self):
        return (int(self.status.item()) | int(self.sim.w["status"].item())) & 0xffffffff

    def topology(self, t):
        """Records of step t: int32 (m, 8) = A, B, fa0..2, fb0..2."""
        off = int(self.step_off[t].item())
        cnt = min(int(self.step_count[t].item()), self.rec_cap - off)
        return self.rec[off:off + max(cnt, 0)].clone()

    # ------------------------------------------------------------------ backward
    def _bwd_buffers(self):
        if self._bwd is None:
            f64 = dict(dtype=torch.float64, device=self.device)
            K = self.K
            self._bwd = dict(seg=torch.zeros((K + 1, self.n, DIFF_ROW), **f64),
                             FT=torch.zeros((K, self.n, 8), **f64),
                             lam=torch.zeros((self.n, DIFF_ROW), **f64),
                             lam2=torch.zeros((self.n, DIFF_ROW), **f64),
                             gFT=torch.zeros((self.n, 8), **f64),
                             glaw=torch.zeros(8, **f64),
                             com_grad=torch.zeros((self.n_steps_max, 4), **f64),
                             t_base=torch.zeros(1, dtype=torch.int32, device=self.device),
                             graphs={})
        return self._bwd

    def _segment_launches(self, m, with_com):
        """Backward over steps t_base .. t_base + m - 1: recompute the m states and forces from
        seg[0] and the topology log, then the transposed steps from the last to the first.  The
        gradient enters and leaves in lam."""
        b = self._bwd
        stream = _dev.stream_handle()
        seg, FT = b["seg"], b["FT"]
        d = C.byref(self.d)
        L = lib()
        cg = b["com_grad"].data_ptr() if with_com else None
        for j in range(m):
            check(L.mwd_diff_force(d, seg[j].data_ptr(), j, stream))
            check(L.mwd_diff_integrate(d, seg[j].data_ptr(), seg[j + 1].data_ptr(), FT[j].data_ptr(), None, j,
                                       stream))
        lam, lam2 = b["lam"], b["lam2"]
        for j in range(m - 1, -1, -1):
            check(L.mwd_diff_adjoint(d, seg[j].data_ptr(), FT[j].data_ptr(), j, lam.data_ptr(), lam2.data_ptr(), cg,
                                     b["gFT"].data_ptr(), b["glaw"].data_ptr(), stream))
            lam, lam2 = lam2, lam
        if lam is not b["lam"]:
            b["lam"].copy_(lam)

    def backward(self, g_com=None, g_final=None):
        """Gradients of <g_com, com> + <g_final, final state> with respect to x0 and the law."""
        b = self._bwd_buffers()
        n_steps, K = self.steps, self.K
        if g_final is not None:
            b["lam"].copy_(g_final.detach())
        else:
            b["lam"].zero_()
        b["glaw"].zero_()
        with_com = g_com is not None
        if with_com:
            b["com_grad"].zero_()
            b["com_grad"][:n_steps, :3].copy_(g_com.detach())
        self.d.t_base = b["t_base"].data_ptr()
        try:
            n_seg = (n_steps + K - 1) // K
            for s in range(n_seg - 1, -1, -1):
                t0 = s * K
                m = min(K, n_steps - t0)
                b["t_base"].fill_(t0)
                b["seg"][0].copy_(self.ckpt[s])
                if self.use_graph and m == K and n_seg > 2:
                    g = b["graphs"].get(with_com)
                    if g is None:
                        torch.cuda.synchronize()
                        g = torch.cuda.CUDAGraph()
                        with torch.cuda.graph(g):   # recorded, not run
                            self._segment_launches(m, with_com)
                        b["graphs"][with_com] = g
                    g.replay()
                else:
                    self._segment_launches(m, with_com)
        finally:
            self.d.t_base = None
        return b["lam"].clone(), b["glaw"].view(2, 4).clone()


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, law, engine, n_steps):
        com, xT = engine.forward(x0, law, n_steps)
        ctx.engine = engine
        ctx.generation = engine.generation
        return com, xT

    @staticmethod
    def backward(ctx, g_com, g_xT):
        eng = ctx.engine
        if eng.generation != ctx.generation:
            raise RuntimeError("the engine ran another forward since this one; its checkpoints are gone")
        g_com_full = None
        if g_com is not None:
            g_com_full = g_com
        gx0, glaw = eng.backward(g_com_full, g_xT)
        return gx0, glaw.to(torch.float64), None, None


def rollout(engine: DiffEngine, x0, law, n_steps):
    """(com (n_steps, 3), final state (n, 32)), differentiable with respect to x0 and law (2, 4)."""
    law = law.to(device=engine.device, dtype=torch.float64)
    com, xT = _Rollout.apply(x0, law, engine, int(n_steps))
    return com, xT
