"""The float64 torch restatement of the differentiable step (oracle/diff_ref.py), pinned to the
oracle on the CPU: each contact's depth, face normal, contact points, force and torques
re-evaluated from the final EPA face the oracle's FP64 contact path found must equal what that
path computed (gpu_fine_contact_detection.cu:270-871 restated), and one leapfrog step must equal
the oracle's FP64 integrator (gpu_Verlet.cu:164-352 restated).  Its autograd gradient is what the
CUDA adjoint is checked against on the GPU."""
import numpy as np
import torch

import diff_ref
import oracle
from helpers import CONTACT_PARAMS, make_pairs, make_verlet_state


def _pair_rows(inp, r, n_wall):
    """Two rows per resolved pair (A then B): FP64 state with identity q_acc and body-frame
    vertices = world vertices - centre, and the logged record of the oracle's final face."""
    ok = np.nonzero((r["collision"] == 1) & (r["status"] == 0))[0]
    P = len(ok)
    x = np.zeros((2 * P, diff_ref.ROW))
    x[:, 26] = 1.0
    counts, verts, info, inert = [], [], np.zeros(2 * P, np.int32), np.zeros((2 * P, 4))
    rec = np.zeros((P, 8), np.int64)
    for k, p in enumerate(ok):
        for side, (c, v, w, nv, idn, Is) in enumerate((("A_com", "A_vel", "A_angvel", "A_nv", "A_id", "IsA"),
                                                       ("B_com", "B_vel", "B_angvel", "B_nv", "B_id", "IsB"))):
            row = 2 * k + side
            cen = np.asarray(inp[c][p], np.float64)
            x[row, 0:3] = cen
            x[row, 3:6] = np.asarray(inp[v][p], np.float64)
            x[row, 15:18] = np.asarray(inp[w][p], np.float64)
            vv = np.asarray(inp["A_verts" if side == 0 else "B_verts"][p][: inp[nv][p]], np.float64) - cen
            verts.append(np.concatenate([vv, np.zeros((len(vv), 1))], 1))
            counts.append(len(vv))
            info[row] = 1 if inp[idn][p] < n_wall else 0
            inert[row, 3] = float(inp[Is][p])
        rec[k] = [2 * k, 2 * k + 1, *r["counters"][p, 3:9]]
    off = np.zeros(2 * P + 1, np.int64)
    np.cumsum(counts, out=off[1:])
    return ok, x, np.concatenate(verts, 0), off, info, inert, rec


def test_pair_terms_match_oracle_fp64():
    prm = dict(CONTACT_PARAMS)
    inp, n_particles = make_pairs(160, seed=21, V=32, dist=(0.6, 1.6))
    r = oracle.contact(inp, prm, n_particles, "f64")
    ok, x, body, off, info, inert, rec = _pair_rows(inp, r, prm["num_particles_wall"])
    assert len(ok) >= 40
    law = torch.tensor([[prm["Kn"], prm["en"], prm["et"], prm["mu"]],
                        [prm["Kn_wall"], prm["en_wall"], prm["et_wall"], prm["mu_wall"]]], dtype=torch.float64)
    t = diff_ref.pair_terms(torch.from_numpy(x), torch.from_numpy(rec), torch.from_numpy(body),
                            torch.from_numpy(off), torch.from_numpy(inert), torch.from_numpy(info), law)
    dg = r["diag"][ok]
    for name, cols in (("depth", [0]), ("n0", [1, 2, 3]), ("cpA", [4, 5, 6]), ("cpB", [7, 8, 9]), ("F", [10, 11, 12]),
                       ("TA", [13, 14, 15]), ("TB", [16, 17, 18])):
        got = t[name].detach().numpy().reshape(len(ok), -1)
        want = dg[:, cols]
        scale = np.abs(want).max()
        err = np.abs(got - want).max() / scale
        assert err < 1e-9, (name, err)


def test_integrator_matches_oracle_fp64():
    N, V, W = 12, 24, 3
    st, box = make_verlet_state(N, V, seed=5, W=W)
    # no fly-away row here: the reset is compared in the next test
    st["com"][W + 1] = [0.0, 0.0, 0.0]
    st["v12"][W + 1] = [1.0, 0.0, 0.0]
    rng = np.random.default_rng(2)
    q = rng.normal(size=(N, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    st["q"][:] = q
    st["q12"][:] = q[::-1]
    st["wbf"][:] = rng.normal(size=(N, 3))
    ref = {k: np.ascontiguousarray(v.copy()) for k, v in st.items()}
    oracle.verlet_f64(ref, 1e-3, box, W, N)
    x = np.zeros((N, diff_ref.ROW))
    x[:, 0:3], x[:, 3:6], x[:, 6:9] = st["com"], st["v"], st["v12"]
    x[:, 9:12], x[:, 12:15], x[:, 15:18] = st["w12bf"], st["wbf"], st["w"]
    x[:, 18:22], x[:, 22:26] = st["q"], st["q12"]
    x[:, 26] = 1.0
    I = np.stack([np.diag(m) for m in st["I"]])
    Ii = np.stack([np.diag(m) for m in st["Iinv"]])
    inertia = np.concatenate([I, np.ones((N, 1))], 1)
    inv = np.concatenate([Ii, 1.0 / st["mass"][:, None]], 1)
    info = np.zeros(N, np.int32)
    info[:W] = 1
    out = diff_ref.integrate(torch.from_numpy(x), torch.from_numpy(st["F"]), torch.from_numpy(st["T"]),
                             torch.from_numpy(inertia), torch.from_numpy(inv), torch.from_numpy(info), 1e-3,
                             list(box)).numpy()
    p = slice(W, N)
    for name, cols, key in (("c", slice(0, 3), "com"), ("v", slice(3, 6), "v"), ("vh", slice(6, 9), "v12"),
                            ("whbf", slice(9, 12), "w12bf"), ("wbf", slice(12, 15), "wbf"), ("w", slice(15, 18), "w"),
                            ("q", slice(18, 22), "q"), ("qh", slice(22, 26), "q12")):
        err = np.abs(out[p, cols] - ref[key][p]).max() / max(1.0, np.abs(ref[key][p]).max())
        assert err < 1e-13, (name, err)
    # walls keep their state
    assert np.array_equal(out[:W], x[:W])


def test_integrator_fly_away_reset_matches_oracle():
    N, V, W = 8, 24, 3
    st, box = make_verlet_state(N, V, seed=6, W=W)
    ref = {k: np.ascontiguousarray(v.copy()) for k, v in st.items()}
    oracle.verlet_f64(ref, 1e-3, box, W, N)
    x = np.zeros((N, diff_ref.ROW))
    x[:, 0:3], x[:, 3:6], x[:, 6:9] = st["com"], st["v"], st["v12"]
    x[:, 9:12], x[:, 12:15], x[:, 15:18] = st["w12bf"], st["wbf"], st["w"]
    x[:, 18:22], x[:, 22:26] = st["q"], st["q12"]
    x[:, 26] = 1.0
    I = np.stack([np.diag(m) for m in st["I"]])
    Ii = np.stack([np.diag(m) for m in st["Iinv"]])
    out = diff_ref.integrate(torch.from_numpy(x), torch.from_numpy(st["F"]), torch.from_numpy(st["T"]),
                             torch.from_numpy(np.concatenate([I, np.ones((N, 1))], 1)),
                             torch.from_numpy(np.concatenate([Ii, 1.0 / st["mass"][:, None]], 1)),
                             torch.from_numpy(np.r_[np.ones(W), np.zeros(N - W)].astype(np.int32)), 1e-3,
                             list(box)).numpy()
    r = W + 1
    assert np.array_equal(out[r, 0:3], st["com"][r])
    assert np.array_equal(ref["com"][r], st["com"][r])
    assert not out[r, 3:18].any() and not ref["v"][r].any() and not ref["w"][r].any()


def test_torch_reference_gradient_is_finite_difference_of_itself():
    """Autograd of the torch restatement through a few steps of frozen topology equals FP64
    central differences (guards the restatement's differentiable form: the series branch of the
    rotation increment, the slip branch, the normalisations)."""
    prm = dict(CONTACT_PARAMS)
    inp, n_particles = make_pairs(40, seed=4, V=32, dist=(0.6, 1.4))
    r = oracle.contact(inp, prm, n_particles, "f64")
    ok, x, body, off, info, inert, rec = _pair_rows(inp, r, prm["num_particles_wall"])
    n = x.shape[0]
    x[:, 18] = 1.0
    x[:, 22] = 1.0
    Iv = np.abs(inert[:, 3:4]) * np.array([[0.9, 1.0, 1.1]])
    inertia = np.concatenate([Iv, inert[:, 3:4]], 1)
    inv = np.concatenate([1.0 / Iv, np.full((n, 1), 0.25)], 1)
    consts = dict(body=torch.from_numpy(body), vert_off=torch.from_numpy(off), inertia=torch.from_numpy(inertia),
                  inv_inertia=torch.from_numpy(inv), ext=torch.zeros((n, 4), dtype=torch.float64),
                  info=torch.from_numpy(info), dt=5e-5, box=[1e9, -1e9, 1e9, -1e9, 1e9, -1e9])
    logs = [torch.from_numpy(rec)] * 4
    law0 = torch.tensor([[1e5, 0.4, 0.4, 0.5], [1e5, 0.4, 0.4, 0.5]], dtype=torch.float64)
    rng = np.random.default_rng(0)
    wc = torch.from_numpy(rng.normal(size=(4, 3)))
    wx = torch.from_numpy(rng.normal(size=(n, diff_ref.ROW)))

    def loss(x0, law):
        com, xT = diff_ref.rollout(x0, law, logs, consts, 4)
        return (com * wc).sum() + (xT * wx).sum() * 1e-3

    X = torch.from_numpy(x).requires_grad_(True)
    Lw = law0.clone().requires_grad_(True)
    loss(X, Lw).backward()
    d = torch.from_numpy(rng.normal(size=(n, diff_ref.ROW)))
    d[:, 18:30] = 0.0  # keep the quaternions unit
    eps = 1e-6
    fd = (loss(X.detach() + eps * d, law0) - loss(X.detach() - eps * d, law0)) / (2 * eps)
    an = (X.grad * d).sum()
    assert abs(float(fd - an)) < 1e-6 * max(1.0, abs(float(an)))
    for i, j in ((0, 0), (0, 1), (0, 3)):
        h = 1e-6 * float(law0[i, j])
        lp, lm = law0.clone(), law0.clone()
        lp[i, j] += h
        lm[i, j] -= h
        fdl = (loss(X.detach(), lp) - loss(X.detach(), lm)) / (2 * h)
        assert abs(float(fdl - Lw.grad[i, j])) < 1e-5 * max(1e-8, abs(float(Lw.grad[i, j]))), (i, j)
