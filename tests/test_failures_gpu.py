"""Failure handling of the device code, injected from the host: an undersized pair buffer, an oversize
hull, a non-finite particle and a full history table.  Each call ends normally with a status bit set
(and an exception where the Python layer checks the word); nothing is written out of bounds and the
other particles are unaffected.  No test here faults, traps or hangs the GPU: every capacity below is
checked by the kernels before they write."""
import numpy as np
import pytest
import torch

from helpers import CONTACT_PARAMS, make_pairs
from mwdiem_gb300 import _lib, scene

pytestmark = pytest.mark.gpu


def dense(n=400, seed=7, vel=0.3):
    sp = scene.pour_scene(n=n, seed=seed, box=16.0, spacing=2.1, pool=48)
    sp.velocities = np.random.default_rng(seed).normal(size=(n, 3)) * vel
    return sp


def oriented(p):
    return set(map(tuple, np.asarray(p).reshape(-1, 2).tolist()))


def test_pair_buffer_overflow_is_reported_and_bounded():
    from mwdiem_gb300.sim import Simulator
    sp = dense()
    full = Simulator(sp)
    full.broadphase()
    want = oriented(full.pairs().cpu().numpy())
    cap = len(want) // 4
    small = Simulator(sp, pair_cap=cap)
    small.step(1)
    torch.cuda.synchronize()
    assert int(small.w["n_pairs"].item()) == len(want)  # the count, beyond the capacity
    assert small.status() & _lib.ST_PAIR_OVERFLOW
    with pytest.raises(_lib.MwdError):
        small.check_status()
    kept = oriented(small.w["pairs"].cpu().numpy())
    assert len(kept) == cap and kept <= want  # the pairs that fit are genuine candidates
    assert small.nonfinite_rows() == 0


def test_oversize_hull_flags_the_pair_only():
    # a pair claiming more vertices than the staging capacity is skipped with BAD_SHAPE; the other
    # pairs of the call are computed as usual
    from mwdiem_gb300 import gpu_fine_contact_detection as G
    inp, N = make_pairs(64, seed=41, V=32)
    good = dict(inp)
    bad = {k: np.array(v, copy=True) for k, v in inp.items()}
    bad["A_nv"][5] = 40  # > num_vertices_max = 32
    out = []
    for d in (good, bad):
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        F, T, hist, coll = G.Contact_detection_GPU(
            d["A_com"], d["B_com"], d["A_verts"], d["B_verts"], d["A_vel"], d["B_vel"], d["A_angvel"], d["B_angvel"],
            d["A_nv"], d["B_nv"], d["A_id"], d["B_id"], d["hist"].copy(), CONTACT_PARAMS["Kn"], CONTACT_PARAMS["en"],
            CONTACT_PARAMS["et"], CONTACT_PARAMS["mu"], CONTACT_PARAMS["Kn_wall"], CONTACT_PARAMS["en_wall"],
            CONTACT_PARAMS["et_wall"], CONTACT_PARAMS["mu_wall"], CONTACT_PARAMS["num_particles_wall"],
            np.zeros((N, 3), np.float32), np.zeros((N, 3), np.float32), 32, d["qA"], d["qB"],
            CONTACT_PARAMS["timestep"], d["IsA"], d["IsB"], status=status)
        torch.cuda.synchronize()
        out.append((np.asarray(coll), int(status.item())))
    (c0, s0), (c1, s1) = out
    assert not s0 & _lib.ST_BAD_SHAPE
    assert s1 & _lib.ST_BAD_SHAPE
    assert c1[5] == -1
    others = np.arange(len(c0)) != 5
    assert np.array_equal(c0[others], c1[others])


def test_non_finite_particle_is_isolated():
    # a particle whose centre is NaN gets no cell (CELL_RANGE) and no pairs; the step finishes and
    # every other particle moves exactly as without it (deterministic sums)
    from mwdiem_gb300.sim import Simulator
    sp = dense(n=300, seed=9)
    ref = Simulator(sp, deterministic=True)
    bad = Simulator(sp, deterministic=True)
    W = sp.n_walls
    victim = W + 17
    ref.broadphase()
    touching = {int(x) for p in ref.pairs().cpu().numpy().tolist() for x in p if victim in p}
    bad.t["pos"][victim, :3] = float("nan")
    for s in (ref, bad):
        s.step(3)
    torch.cuda.synchronize()
    assert bad.status() & _lib.ST_CELL_RANGE
    assert bad.nonfinite_rows() >= 1
    pos_r, pos_b = ref.t["pos"].cpu().numpy(), bad.t["pos"].cpu().numpy()
    unaffected = np.ones(len(pos_r), bool)
    unaffected[list(touching | {victim})] = False  # the victim and its initial neighbours
    assert np.isfinite(pos_b[unaffected]).all()
    # particles far from the victim (no contact with it) follow the same trajectories
    far = unaffected & (np.linalg.norm(pos_r[:, :3] - pos_r[victim, :3], axis=1) > 8.0)
    far[:W] = False
    assert far.sum() > 50
    assert np.array_equal(pos_r[far], pos_b[far])


def test_full_history_table_is_reported():
    # a persistent-history table too small for the contacts of a step: HIST_OVERFLOW, bounded probing
    from mwdiem_gb300.sim import Simulator
    sp = dense(n=400, seed=21, vel=0.3)
    sim = Simulator(sp, deterministic=True, persistent_history=True)
    sim.work.hist_cap = 4  # a prefix of the allocated tables (a power of two)
    sim.step(2)
    torch.cuda.synchronize()
    assert sim.status() & _lib.ST_HIST_OVERFLOW
    assert sim.nonfinite_rows() == 0
