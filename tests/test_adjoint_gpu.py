"""The differentiable step (mwdiem_gb300.diff) on the GPU.

Forward: the FP64 CUDA rollout equals the float64 torch restatement (oracle/diff_ref.py, pinned to
the oracle by test_diff_ref.py) run over the same logged contact topology.  Adjoint: the CUDA
gradient equals torch autograd of that restatement, for every checkpoint interval, and equals FP64
central finite differences of the full forward (detection included) at 16 particles x 50 steps,
with respect to kn, damping ratio, mu and the initial velocities, within 1e-4 relative."""
import numpy as np
import pytest
import torch

import diff_ref

pytestmark = pytest.mark.gpu

STEPS = 50


def make_engine(n=16, steps=STEPS, K=10, seed=3, contact_point="reference", spin=3.0, spacing=2.0):
    from mwdiem_gb300 import scene
    from mwdiem_gb300.diff import DiffEngine
    spec = scene.packed_scene(n=n, seed=seed, spacing=spacing)
    eng = DiffEngine(spec, steps, ckpt_every=K, contact_point=contact_point)
    x0 = eng.initial_state()
    g = torch.Generator(device="cuda").manual_seed(seed)
    W = eng.n_walls
    w = torch.randn((n, 3), generator=g, device="cuda", dtype=torch.float64) * spin
    x0[W:, 9:12] = w      # w_half_bf
    x0[W:, 12:15] = w     # w_bf
    x0[W:, 15:18] = w     # w (the initial orientation is the identity: body frame = world frame)
    return eng, x0


def logs_of(eng, steps):
    return [eng.topology(t) for t in range(steps)]


def topo_key(eng, steps):
    return [tuple(sorted(map(tuple, eng.topology(t).cpu().numpy().tolist()))) for t in range(steps)]


def test_forward_matches_torch_restatement():
    eng, x0 = make_engine()
    law = eng.default_law()
    com, xT = eng.forward(x0, law, STEPS)
    logs = logs_of(eng, STEPS)
    assert sum(len(l) for l in logs) > 8 * STEPS, "the scene should be in contact throughout"
    assert eng.status_word() & 0x380 == 0
    com_r, xT_r = diff_ref.rollout(x0, law, logs, diff_ref.engine_consts(eng), STEPS)
    assert torch.isfinite(com).all() and torch.isfinite(xT).all()
    assert (com - com_r).abs().max() <= 1e-11 * (1 + com_r.abs().max())
    err = (xT - xT_r).abs().max(0).values / (1 + xT_r.abs().max(0).values)
    assert err.max() <= 1e-9, err


@pytest.mark.parametrize("contact_point", ["reference", "midpoint"])
def test_adjoint_matches_torch_autograd(contact_point):
    from mwdiem_gb300.diff import rollout
    eng, x0 = make_engine(K=7, contact_point=contact_point)
    law0 = eng.default_law()
    rng = np.random.default_rng(1)
    wc = torch.from_numpy(rng.normal(size=(STEPS, 3))).cuda()
    wx = torch.from_numpy(rng.normal(size=(eng.n, 32))).cuda() * 1e-2
    X = x0.clone().requires_grad_(True)
    L = law0.clone().requires_grad_(True)
    com, xT = rollout(eng, X, L, STEPS)
    ((com * wc).sum() + (xT * wx).sum()).backward()
    logs = logs_of(eng, STEPS)
    Xr = x0.clone().requires_grad_(True)
    Lr = law0.clone().requires_grad_(True)
    cps = 1.0 if contact_point == "midpoint" else -1.0
    com_r, xT_r = diff_ref.rollout(Xr, Lr, logs, diff_ref.engine_consts(eng), STEPS, cps=cps)
    ((com_r * wc).sum() + (xT_r * wx).sum()).backward()
    gx, gxr = X.grad, Xr.grad
    W = eng.n_walls
    # per state column; a column whose true gradient is zero (the radial part of the unit q_acc at
    # the identity) is compared against the largest gradient of the state instead
    col = gxr[W:, :30].abs().max(0).values
    scale = torch.maximum(col, 1e-9 * col.max())
    err = (gx[W:, :30] - gxr[W:, :30]).abs().max(0).values / scale
    assert err.max() <= 1e-8, err
    gl_err = ((L.grad - Lr.grad).abs() / (Lr.grad.abs() + 1e-30)).max()
    assert gl_err <= 1e-8, (L.grad, Lr.grad)


def test_checkpoint_interval_leaves_gradient_unchanged():
    from mwdiem_gb300.diff import rollout
    grads = []
    for K in (1, 7, STEPS):
        eng, x0 = make_engine(K=K)
        X = x0.clone().requires_grad_(True)
        L = eng.default_law().requires_grad_(True)
        com, xT = rollout(eng, X, L, STEPS)
        (com ** 2).sum().backward()
        grads.append((X.grad.clone(), L.grad.clone()))
    for gx, gl in grads[1:]:
        assert (gx - grads[0][0]).abs().max() <= 1e-10 * grads[0][0].abs().max()
        assert ((gl - grads[0][1]).abs() <= 1e-10 * grads[0][1].abs().max()).all()


def test_gradient_matches_fp64_finite_differences():
    """Loss = MSE of the per-step centre of mass against a target trajectory made by the same
    simulator with other parameters (kn 2e5, damping ratio 0.2, mu 0.4); gradients with respect to
    kn, damping ratio, mu and the initial velocities against FP64 central differences of the whole
    forward (detection re-run), checking the topology stays the one the adjoint differentiates."""
    from mwdiem_gb300.diff import law_from, rollout
    eng, x0 = make_engine(K=10, spacing=2.2)
    W = eng.n_walls
    dev = x0.device
    tgt_law = law_from(2e5, 0.2, 0.4).to(dev)
    com_t, _ = eng.forward(x0, tgt_law, STEPS)
    target = com_t.clone()
    base = dict(kn=1e5, zeta=0.3, mu=0.5)
    v0 = x0[W:, 3:6].clone()

    def loss(kn, zeta, mu, v, keep_topology=False):
        x = x0.clone()
        x = torch.cat([x[:W], torch.cat([x[W:, :3], v, v, x[W:, 9:]], 1)], 0)
        com, _ = rollout(eng, x, law_from(kn, zeta, mu).to(dev), STEPS)
        out = ((com - target) ** 2).mean()
        return out, (topo_key(eng, STEPS) if keep_topology else None)

    p = {k: torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=True) for k, v in base.items()}
    vv = v0.clone().requires_grad_(True)
    L0, topo0 = loss(p["kn"], p["zeta"], p["mu"], vv, keep_topology=True)
    L0.backward()
    grads = {k: float(t.grad) for k, t in p.items()}
    rng = np.random.default_rng(7)
    d = torch.from_numpy(rng.normal(size=tuple(v0.shape))).to(dev)
    grads["v0"] = float((vv.grad * d).sum())
    for name in ("kn", "zeta", "mu", "v0"):
        h = 1e-6 * (base[name] if name != "v0" else 1.0)
        vals = []
        for sgn in (1, -1):
            args = {k: v for k, v in base.items()}
            v = v0
            if name == "v0":
                v = v0 + sgn * h * d
            else:
                args[name] = base[name] + sgn * h
            with torch.no_grad():
                Lv, topo = loss(args["kn"], args["zeta"], args["mu"], v, keep_topology=True)
            assert topo == topo0, f"{name}: the perturbation changed the contact topology"
            vals.append(float(Lv))
        fd = (vals[0] - vals[1]) / (2 * h)
        an = grads[name]
        assert abs(fd - an) <= 1e-4 * abs(fd), (name, fd, an)


def test_fp64_forces_agree_with_fp32_narrow_phase():
    """The smooth FP64 force of each logged contact (depth and normal re-evaluated from the final
    face's support vertices) agrees with the FP32 narrow phase's own force to FP32 accuracy."""
    import ctypes as C

    from mwdiem_gb300._lib import check, lib
    eng, x0 = make_engine(spacing=2.2)
    law = eng.default_law()
    eng.forward(x0, law, 1)
    # the FP32 narrow phase of the first step, re-run on the same mirrors
    sim = eng.sim
    check(lib().mwd_diff_mirror(C.byref(eng.d), x0.data_ptr(), C.byref(sim.state), None))
    sim.t["force"].zero_()
    sim.t["torque"].zero_()
    sim.broadphase()
    sim.narrow_force()
    f32 = sim.t["force"][:, :3].double()
    eng.F.zero_()
    eng.T.zero_()
    check(lib().mwd_diff_force(C.byref(eng.d), x0.data_ptr(), 0, None))
    f64 = eng.F[:, :3].clone()
    eng.F.zero_()
    eng.T.zero_()
    W = eng.n_walls
    rel = (f32[W:] - f64[W:]).norm(dim=1) / (f64[W:].norm(dim=1) + 1.0)
    assert float(rel.median()) < 1e-4 and float(rel.max()) < 1e-2, rel
