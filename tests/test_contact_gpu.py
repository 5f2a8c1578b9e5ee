"""Narrow phase + contact force on the GPU (``mwd_contact_pairs`` through the drop-in
``Contact_detection_GPU``) against the oracle.

Bar: contact flags, depth, normal, contact points, per-particle force/torque and the history are
bit-identical to the FP32 oracle (which is itself bit-identical to the reference kernel compiled for
the CPU, see test_oracle.py), when every particle appears in one pair (one atomic term per particle).
With shared particles the float atomics reorder the sums: tolerance 1e-5 relative to the largest
force.  Against the FP64 oracle: identical flags outside a 1e-9 band, depth/normal within 1e-4.
"""
import numpy as np
import pytest
import torch

import oracle
from helpers import CONTACT_PARAMS, cube_pair_kat, make_pairs, select

pytestmark = pytest.mark.gpu


def run_gpu(inp, N, params, lanes=8, hist_mode=0):
    from mwdiem_gb300 import gpu_fine_contact_detection as G
    P = inp["A_com"].shape[0]
    diag = torch.zeros((max(P, 1), 10), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    F, T, hist, coll = G.Contact_detection_GPU(
        inp["A_com"], inp["B_com"], inp["A_verts"], inp["B_verts"], inp["A_vel"], inp["B_vel"], inp["A_angvel"],
        inp["B_angvel"], inp["A_nv"], inp["B_nv"], inp["A_id"], inp["B_id"], inp["hist"].copy(), params["Kn"],
        params["en"], params["et"], params["mu"], params["Kn_wall"], params["en_wall"], params["et_wall"],
        params["mu_wall"], params["num_particles_wall"], np.zeros((N, 3), np.float32), np.zeros((N, 3), np.float32),
        params["num_vertices_max"], inp["qA"], inp["qB"], params["timestep"], inp["IsA"], inp["IsB"],
        hist_mode=hist_mode, lanes=lanes, diag=diag, status=status)
    torch.cuda.synchronize()
    return dict(force=F, torque=T, hist=hist, collision=coll, diag=diag.cpu().numpy()[:P],
                status=int(status.item()))


def bits_equal(a, b):
    """Bit-identical, except that NaNs compare by position only (payload bits differ between the CPU
    and the GPU, which produce different NaN encodings)."""
    a = np.array(a)
    b = np.array(b, dtype=a.dtype)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        na, nb = np.isnan(a), np.isnan(b)
        if not np.array_equal(na, nb):
            return False
        a[na] = 0
        b[nb] = 0
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("lanes", [4, 8, 16, 32])
def test_bitexact_vs_oracle_f32(lanes):
    inp, N = make_pairs(1500, seed=11)
    o = oracle.contact(inp, CONTACT_PARAMS, N, "f32")
    g = run_gpu(inp, N, CONTACT_PARAMS, lanes=lanes)
    assert np.array_equal(g["collision"], o["collision"])
    assert (o["collision"] == 1).sum() > 300 and (o["collision"] == 0).sum() > 300
    assert bits_equal(g["diag"], o["diag"][:, :10])
    assert bits_equal(g["force"], o["force"])
    assert bits_equal(g["torque"], o["torque"])
    assert bits_equal(g["hist"], o["hist"])
    expect = 0
    for s in np.unique(o["status"]):
        expect |= int(s)
    assert g["status"] == expect


def test_bitexact_hull64_hist_stride4():
    p = dict(CONTACT_PARAMS, num_vertices_max=64)
    inp, N = make_pairs(800, seed=12, V=64, n_min=8, n_max=64)
    inp["hist"] = (np.random.default_rng(5).normal(size=inp["hist"].shape) * 1e-4).astype(np.float32)
    o = oracle.contact(inp, p, N, "f32", hist_stride4=True)
    g = run_gpu(inp, N, p, lanes=16, hist_mode=1)
    assert np.array_equal(g["collision"], o["collision"])
    assert bits_equal(g["diag"], o["diag"][:, :10])
    assert bits_equal(g["force"], o["force"])
    assert bits_equal(g["torque"], o["torque"])
    assert bits_equal(g["hist"], o["hist"])


def test_stride1_history_nonzero_input():
    # the reference reads displacement_tang[P..P+2] and writes [P..P+3] (overlapping rows)
    inp, N = make_pairs(400, seed=13)
    inp["hist"] = (np.random.default_rng(7).normal(size=inp["hist"].shape) * 1e-4).astype(np.float32)
    o = oracle.contact(inp, CONTACT_PARAMS, N, "f32")
    g = run_gpu(inp, N, CONTACT_PARAMS)
    assert bits_equal(g["hist"], o["hist"])
    assert bits_equal(g["force"], o["force"])
    assert bits_equal(g["torque"], o["torque"])


def test_walls_and_shared_particles():
    p = dict(CONTACT_PARAMS, num_particles_wall=40, Kn_wall=3e4, en_wall=0.5, et_wall=0.6, mu_wall=0.3)
    inp, N = make_pairs(1200, seed=14, unique_ids=False, n_particles=200)
    o = oracle.contact(inp, p, N, "f32")
    g = run_gpu(inp, N, p)
    assert np.array_equal(g["collision"], o["collision"])
    assert bits_equal(g["diag"], o["diag"][:, :10])
    scale = np.abs(o["force"]).max()
    assert np.abs(g["force"] - o["force"]).max() <= 1e-5 * scale
    assert np.abs(g["torque"] - o["torque"]).max() <= 1e-5 * np.abs(o["torque"]).max()


def test_against_fp64_oracle():
    inp, N = make_pairs(1500, seed=15)
    o32 = oracle.contact(inp, CONTACT_PARAMS, N, "f32")
    o64 = oracle.contact(inp, CONTACT_PARAMS, N, "f64")
    g = run_gpu(inp, N, CONTACT_PARAMS)
    # flags: identical except pairs whose FP64 separation/depth lies within 1e-9
    band = (o64["collision"] == 1) & (np.abs(o64["diag"][:, 0]) < 1e-9)
    differ = (g["collision"] != o64["collision"]) & ~band
    assert differ.sum() == 0
    both = (g["collision"] == 1) & (o64["collision"] == 1) & (o32["status"] == 0) & (o64["status"] == 0)
    d64 = o64["diag"][both, 0]
    assert np.all(np.abs(g["diag"][both, 0] - d64) <= 1e-4 * np.abs(d64) + 1e-6)
    n32, n64 = g["diag"][both, 1:4], o64["diag"][both, 1:4]
    assert np.all(np.abs(n32 - n64).max(axis=1) <= 1e-4)


def test_cube_known_answer():
    inp = cube_pair_kat(0.1)
    p = dict(CONTACT_PARAMS, num_vertices_max=8, num_particles_wall=0, Kn=1e4)
    g = run_gpu(inp, 2, p)
    assert g["collision"][0] == 1
    assert abs(g["diag"][0, 0] - 0.1) < 1e-6
    # |F| = Kn * depth for a pair at rest (MWDiem's contact law, no damping term without motion)
    assert abs(np.linalg.norm(g["force"][0]) - 1e4 * 0.1) < 1e-2
    assert np.allclose(g["force"][0], -g["force"][1])
    o = oracle.contact(inp, p, 2, "f32")
    assert bits_equal(g["force"], o["force"])


def test_separated_and_degenerate():
    inp, N = make_pairs(300, seed=16, dist=(2.5, 4.0))
    g = run_gpu(inp, N, CONTACT_PARAMS)
    assert np.all(g["collision"] == 0)
    assert np.all(g["force"] == 0) and np.all(g["hist"] == 0)
    # identical position and shape: origin inside the Minkowski difference, CorrectFlat path
    inp2, N2 = make_pairs(64, seed=17)
    inp2["B_com"] = inp2["A_com"].copy()
    inp2["B_verts"] = inp2["A_verts"].copy()
    inp2["B_nv"] = inp2["A_nv"].copy()
    o = oracle.contact(inp2, CONTACT_PARAMS, N2, "f32")
    g2 = run_gpu(inp2, N2, CONTACT_PARAMS)
    assert np.array_equal(g2["collision"], o["collision"])
    assert bits_equal(g2["diag"], o["diag"][:, :10])
    assert bits_equal(g2["force"], o["force"])


def test_support_ties_first_index():
    # duplicated vertices make equal support values; the first index must win on both sides
    inp, N = make_pairs(200, seed=18, V=32, n_max=16)
    for k in ("A_verts", "B_verts"):
        nv = inp["A_nv"] if k == "A_verts" else inp["B_nv"]
        for p in range(inp[k].shape[0]):
            n = int(nv[p])
            inp[k][p, n:2 * n] = inp[k][p, :n]
        nv *= 2
    o = oracle.contact(inp, CONTACT_PARAMS, N, "f32")
    g = run_gpu(inp, N, CONTACT_PARAMS, lanes=8)
    assert np.array_equal(g["collision"], o["collision"])
    assert bits_equal(g["diag"], o["diag"][:, :10])


def test_empty_and_single():
    inp, N = make_pairs(1, seed=19)
    g = run_gpu(select(inp, slice(0, 0)), N, CONTACT_PARAMS)
    assert g["collision"].shape == (0,) and np.all(g["force"] == 0)
    o = oracle.contact(inp, CONTACT_PARAMS, N, "f32")
    g1 = run_gpu(inp, N, CONTACT_PARAMS)
    assert np.array_equal(g1["collision"], o["collision"])
    assert bits_equal(g1["force"], o["force"])


def test_device_tensors_in_place():
    from mwdiem_gb300 import gpu_fine_contact_detection as G
    inp, N = make_pairs(256, seed=20)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in inp.items()}
    F = torch.zeros((N, 3), dtype=torch.float32, device="cuda")
    T = torch.zeros_like(F)
    p = CONTACT_PARAMS
    F2, T2, hist, coll = G.Contact_detection_GPU(
        d["A_com"], d["B_com"], d["A_verts"], d["B_verts"], d["A_vel"], d["B_vel"], d["A_angvel"], d["B_angvel"],
        d["A_nv"], d["B_nv"], d["A_id"], d["B_id"], d["hist"], p["Kn"], p["en"], p["et"], p["mu"], p["Kn_wall"],
        p["en_wall"], p["et_wall"], p["mu_wall"], p["num_particles_wall"], F, T, p["num_vertices_max"], d["qA"],
        d["qB"], p["timestep"], d["IsA"], d["IsB"])
    assert F2 is F and T2 is T and hist is d["hist"]
    o = oracle.contact(inp, p, N, "f32")
    assert bits_equal(F.cpu().numpy(), o["force"])
    assert np.array_equal(coll.cpu().numpy(), o["collision"])


@pytest.mark.parametrize("lanes", [8, 32])
def test_epa_beyond_128_faces_resolves_like_the_oracle(lanes):
    # a deep overlap of two 32-64-vertex hulls whose EPA creates 129 faces in all: an append-only face
    # list of 128 entries stopped it with EPA_OVERFLOW; the compacted list holds only the live faces
    # (at most 2 x 30 - 4 = 56 within the reference's iteration limit) and finishes it, as the oracle,
    # which has no limit on faces created, does
    inp, N = make_pairs(2000, seed=242, V=64, n_min=32, n_max=64, dist=(0.3, 1.2))
    p = dict(CONTACT_PARAMS, num_vertices_max=64)
    sub = select(inp, np.arange(1040, 1070))
    o = oracle.contact(sub, p, N, "f32")
    assert o["counters"][14, 9] == 129 and not o["status"][14] & oracle.ST_EPA_OVERFLOW
    assert o["collision"][14] == 1
    # with creation capped at 128 faces the same pair overflows
    assert oracle.contact(sub, p, N, "f32", face_cap=128)["status"][14] & oracle.ST_EPA_OVERFLOW
    g = run_gpu(sub, N, p, lanes=lanes)
    assert not g["status"] & 2, "EPA_OVERFLOW"
    assert np.array_equal(g["collision"], o["collision"])
    assert bits_equal(g["diag"], o["diag"][:, :10])
    assert bits_equal(g["force"], o["force"]) and bits_equal(g["torque"], o["torque"])


@pytest.mark.parametrize("lanes", [1 | (16 << 8) | (1 << 16), 8 | (32 << 8)])
def test_epa_beyond_128_faces_in_the_two_pass_narrow_phase(lanes):
    # the same pair in the device step's two-pass narrow phase: its EPA pass stops the pair when the
    # append-only face list is full and a retry kernel runs it again with the compacting EPA; the
    # result must be the oracle's, bit for bit, with the work counted once
    from mwdiem_gb300.pairbench import PairScene
    inp, N = make_pairs(2000, seed=242, V=64, n_min=32, n_max=64, dist=(0.3, 1.2))
    p = dict(CONTACT_PARAMS, num_vertices_max=64)
    sub = select(inp, np.arange(1040, 1070))
    ps = PairScene.from_arrays(sub, p, lanes=lanes)
    ps.narrow(count_work=True)
    torch.cuda.synchronize()
    P = 30
    local = dict(sub, A_id=(2 * np.arange(P)).astype(np.int32), B_id=(2 * np.arange(P) + 1).astype(np.int32))
    o = oracle.contact(local, p, 2 * P, "f32")
    assert o["counters"][14, 9] == 129
    assert not int(ps.w["status"].item()) & 2, "EPA_OVERFLOW"
    assert np.array_equal(ps.w["collision"].cpu().numpy(), o["collision"])
    assert bits_equal(ps.t["force"][:, :3].cpu().numpy(), o["force"])
    assert bits_equal(ps.t["torque"][:, :3].cpu().numpy(), o["torque"])
    got = tuple(int(x) for x in ps.w["counters"].cpu().numpy())
    nsup = o["counters"][:, 0].astype(np.int64)
    want = (int((nsup * (local["A_nv"].astype(np.int64) + local["B_nv"])).sum()),
            int(o["counters"][:, 9][o["collision"] == 1].astype(np.int64).sum()), int(nsup.sum()))
    assert got == want
