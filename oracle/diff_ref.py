"""Float64 pure-torch restatement of the differentiable step, differentiated by torch autograd.

TEST INFRASTRUCTURE ONLY: the checker of the hand-written CUDA adjoint (mwd_diff_adjoint) and of
the FP64 forward kernels (mwd_diff_force / mwd_diff_integrate).  Given the contact topology of each
step (the engine's log: rows A, B and the support vertices of the final EPA face), it evaluates

  face vertices  a_k = c_A + R(qacc_A) r0_A[fa_k], b_k likewise, V_k = a_k - b_k
  normal, depth  n0 = unit((V1 - V0) x (V2 - V1)), depth = n0 . V0    (gpu_fine_contact_detection.cu:270-325)
  contact points barycentric weights of depth n0 in the face          (.cu:548-600)
  force          the spring-dashpot + Coulomb law with zero tangential history (.cu:647-871,
                 MWDiem.py:966), torque arm from cp = (cpA + s cpB) / 2 (s = -1 as .cu:677)
  integrator     the leapfrog of gpu_Verlet.cu:164-323, q_acc <- unit(q q_acc)

as vectorised torch operations, so ``torch.autograd`` gives the reference gradient.
"""
from __future__ import annotations

import torch

ROW = 32
PI = 3.141592653589793


def qmul(a, b):
    aw, av = a[..., :1], a[..., 1:]
    bw, bv = b[..., :1], b[..., 1:]
    w = aw * bw - (av * bv).sum(-1, keepdim=True)
    v = bv * aw + av * bw + torch.cross(av, bv, dim=-1)
    return torch.cat([w, v], -1)


def conj(q):
    return torch.cat([q[..., :1], -q[..., 1:]], -1)


def pure(v):
    return torch.cat([torch.zeros_like(v[..., :1]), v], -1)


def qtrip(q1, v, q2):
    return qmul(q1, qmul(pure(v), q2))[..., 1:]


def rotv(q, r):
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    rx, ry, rz = r[..., 0], r[..., 1], r[..., 2]
    X = (1 - 2 * (y * y + z * z)) * rx + 2 * (x * y - w * z) * ry + 2 * (x * z + w * y) * rz
    Y = 2 * (x * y + w * z) * rx + (1 - 2 * (x * x + z * z)) * ry + 2 * (y * z - w * x) * rz
    Z = 2 * (x * z - w * y) * rx + 2 * (y * z + w * x) * ry + (1 - 2 * (x * x + y * y)) * rz
    return torch.stack([X, Y, Z], -1)


def rot_inc(w, s):
    """(cos th, sin(th) w/|w|), th = |w| s; Taylor series in th^2 below 1e-6 (as the kernels)."""
    w2 = (w * w).sum(-1)
    t2 = w2 * s * s
    small = t2 < 1e-6
    c_ser = 1 - t2 * 0.5 + t2 * t2 / 24
    k_ser = s * (1 - t2 / 6 + t2 * t2 / 120)
    wn = torch.sqrt(torch.where(small, torch.ones_like(w2), w2))
    th = wn * s
    c_dir = torch.cos(th)
    k_dir = torch.sin(th) / wn
    c = torch.where(small, c_ser, c_dir)
    k = torch.where(small, k_ser, k_dir)
    return torch.cat([c[..., None], w * k[..., None]], -1)


def pair_forces(x, rec, body, vert_off, inertia, info, law, cps=-1.0):
    """Per-row contact force and torque (n,3) of the logged contacts rec (m,8) int."""
    n = x.shape[0]
    F = torch.zeros((n, 3), dtype=x.dtype, device=x.device)
    T = torch.zeros((n, 3), dtype=x.dtype, device=x.device)
    if rec.shape[0] == 0:
        return F, T
    p = pair_terms(x, rec, body, vert_off, inertia, info, law, cps)
    A, B = rec[:, 0].long(), rec[:, 1].long()
    notA = (~(info[A] & 1).bool()).to(x.dtype)[:, None]
    notB = (~(info[B] & 1).bool()).to(x.dtype)[:, None]
    F = F.index_add(0, A, p["F"] * notA).index_add(0, B, -p["F"] * notB)
    T = T.index_add(0, A, p["TA"] * notA).index_add(0, B, p["TB"] * notB)
    return F, T


def pair_terms(x, rec, body, vert_off, inertia, info, law, cps=-1.0):
    """Per-contact depth, face normal n0, contact points, force on A (Fn) and torques."""
    rec = rec.long()
    A, B = rec[:, 0], rec[:, 1]
    fa, fb = rec[:, 2:5], rec[:, 5:8]
    cA, cB = x[A, 0:3], x[B, 0:3]
    vA, vB = x[A, 3:6], x[B, 3:6]
    wA, wB = x[A, 15:18], x[B, 15:18]
    qA, qB = x[A, 26:30], x[B, 26:30]
    rA = body[vert_off[A][:, None].long() + fa, :3].to(x.dtype)
    rB = body[vert_off[B][:, None].long() + fb, :3].to(x.dtype)
    a = cA[:, None, :] + rotv(qA[:, None, :].expand(-1, 3, -1), rA)
    b = cB[:, None, :] + rotv(qB[:, None, :].expand(-1, 3, -1), rB)
    V = a - b
    e1 = V[:, 1] - V[:, 0]
    e2 = V[:, 2] - V[:, 1]
    m = torch.cross(e1, e2, dim=-1)
    n0 = m / torch.sqrt((m * m).sum(-1, keepdim=True))
    depth = (n0 * V[:, 0]).sum(-1)
    Pr = n0 * depth[:, None]
    u1 = V[:, 2] - V[:, 0]
    w2 = Pr - V[:, 0]
    d00 = (e1 * e1).sum(-1)
    d01 = (e1 * u1).sum(-1)
    d11 = (u1 * u1).sum(-1)
    d20 = (w2 * e1).sum(-1)
    d21 = (w2 * u1).sum(-1)
    den = d00 * d11 - d01 * d01
    b1 = (d11 * d20 - d01 * d21) / den
    b2 = (d00 * d21 - d01 * d20) / den
    b0 = 1 - b2 - b1
    cpA = a[:, 0] * b0[:, None] + a[:, 1] * b1[:, None] + a[:, 2] * b2[:, None]
    cpB = b[:, 0] * b0[:, None] + b[:, 1] * b1[:, None] + b[:, 2] * b2[:, None]
    cp = (cpA + cpB * cps) * 0.5
    dA = cp - cA
    dB = cp - cB
    wall = ((info[A] & 1) | (info[B] & 1)).bool()
    L = torch.where(wall[:, None], law[1][None, :], law[0][None, :])
    Kn, en, et, mu = L[:, 0], L[:, 1], L[:, 2], L[:, 3]
    IsA, IsB = inertia[A, 3], inertia[B, 3]
    Cc = 1 / mu + (dA * dA).sum(-1) / IsA + (dB * dB).sum(-1) / IsB
    Len, Let = torch.log(en), torch.log(et)
    Xen = Len * Len + PI * PI
    S = torch.sqrt(mu * Kn / Xen)
    Gn = -2 * Len * S
    Gt = -2 * Let / Cc
    sgn = torch.where(((cB - cA) * n0).sum(-1) < 0, -1.0, 1.0).to(x.dtype)
    nn = n0 * sgn[:, None]
    ra, rb = cpA - cA, cpB - cB
    u = vA + torch.cross(wA, ra, dim=-1) - vB - torch.cross(wB, rb, dim=-1)
    uns = (u * nn).sum(-1)
    un = nn * uns[:, None]
    ut = u - un
    Fn = nn * (-Kn * depth)[:, None] - un * Gn[:, None]
    Fnn = torch.sqrt((Fn * Fn).sum(-1))
    Ftl = ut * (-Gt)[:, None]
    Ftn = torch.sqrt((Ftl * Ftl).sum(-1))
    slip = Ftn > mu * Fnn
    utn = torch.sqrt(torch.where(slip, (ut * ut).sum(-1), torch.ones_like(Ftn)))
    Fts = (ut / utn[:, None]) * (-mu * Fnn)[:, None]
    Ft = torch.where(slip[:, None], Fts, Ftl)
    Ff = Ft + Fn
    TA = torch.cross(dA, Ff, dim=-1)
    TB = -torch.cross(dB, Ff, dim=-1)
    return dict(depth=depth, n0=n0, cpA=cpA, cpB=cpB, F=Fn, TA=TA, TB=TB, slip=slip)


def integrate(x, F, T, inertia, inv_inertia, info, dt, box):
    """One leapfrog step of every non-wall row; walls keep their state."""
    c, vh, whbf, wbf, w = x[:, 0:3], x[:, 6:9], x[:, 9:12], x[:, 12:15], x[:, 15:18]
    q, qh, qa = x[:, 18:22], x[:, 22:26], x[:, 26:30]
    I, Ii, invm = inertia[:, :3], inv_inertia[:, :3], inv_inertia[:, 3:4]
    k = invm * dt
    v32 = vh + F * k
    tbf = qtrip(conj(q), T, q)
    p1 = I * wbf
    p2 = tbf - torch.cross(wbf, p1, dim=-1)
    al = Ii * p2
    w32bf = whbf + al * dt
    q32 = qmul(rot_inc(w, dt * 0.5), qh)
    dx = v32 * dt
    w34bf = w32bf + al * (dt * 0.25)
    w34 = qtrip(q32, w34bf, conj(q32))
    qn = qmul(rot_inc(w34, dt * 0.25), q32)
    wbf2 = w32bf + al * (dt * 0.5)
    w2 = qtrip(qn, wbf2, conj(qn))
    v2 = v32 + F * k
    qraw = qmul(qn, qa)
    qa2 = qraw / torch.sqrt((qraw * qraw).sum(-1, keepdim=True))
    c2 = c + dx
    out = (c2[:, 0] > box[0]) | (c2[:, 0] < box[1]) | (c2[:, 1] > box[2]) | (c2[:, 1] < box[3]) | \
          (c2[:, 2] > box[4]) | (c2[:, 2] < box[5])
    keep = out[:, None]
    z3 = torch.zeros_like(c2)
    c2 = torch.where(keep, c, c2)
    v2, v32, w32bf, wbf2, w2 = [torch.where(keep, z3, t) for t in (v2, v32, w32bf, wbf2, w2)]
    new = torch.cat([c2, v2, v32, w32bf, wbf2, w2, qn, q32, qa2, x[:, 30:32]], 1)
    wall = (info & 1).bool()[:, None]
    return torch.where(wall, x, new)


def rollout(x0, law, logs, consts, n_steps, cps=-1.0):
    """(com (n_steps,3), final state) of n_steps steps with the logged topology logs[t]."""
    body, vert_off, inertia, inv_inertia, ext, info, dt, box = (consts[k] for k in (
        "body", "vert_off", "inertia", "inv_inertia", "ext", "info", "dt", "box"))
    part = ~(info & 1).bool()
    x = x0
    com = []
    for t in range(n_steps):
        F, T = pair_forces(x, logs[t], body, vert_off, inertia, info, law, cps)
        x = integrate(x, F + ext[:, :3], T, inertia, inv_inertia, info, dt, box)
        com.append(x[part, 0:3].mean(0))
    return torch.stack(com), x


def engine_consts(engine):
    """Constant arrays of a DiffEngine, for rollout()."""
    sim = engine.sim
    return dict(body=sim.t["body_verts"].double(), vert_off=sim.t["vert_off"], inertia=engine.inertia,
                inv_inertia=engine.inv_inertia, ext=engine.ext, info=sim.t["info"], dt=float(engine.spec.dt),
                box=[float(b) for b in engine.spec.box()])


def check_finite(*ts):
    return all(bool(torch.isfinite(t).all()) for t in ts)

