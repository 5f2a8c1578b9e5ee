"""Parity on the inputs the benchmark times, through the device step itself.

  * pour20k: bench.py's own scene (20,000 hulls, its 140,005-cell table scanned tile by tile), at
    step 0 and after 25 graph-replayed steps, with both lane settings the autotuner picks for it;
  * a batch of 16 scenes (one of 50,000 particles; cubes, tetrahedra and hulls) in one state, with
    the dense and with the occupancy-compressed cell table;
  * the narrow-phase workload of 4M independent random pairs: a sample of 131,072 pairs;
  * the kernel's own work counters (the roofline's numerator) against the oracle's per-pair counts.

Bars (the oracle is the reference's per-step CPU path, oracle/stepper.py and oracle.contact):
  * candidate pairs: the reference's oriented set, wall pairs included (MWDiem.py:808-817,
    LIBRARY_Coarse_contact_detection.py:84-155), computed from the device's own FP64 centres;
  * the bounding-sphere filter drops only pairs the oracle classifies "no contact";
  * contact flags: identical to the FP32 oracle fed the device's world vertices;
  * per-particle force and torque sums: within 1e-5 of the largest with float atomics, bit-identical
    with deterministic sums;
  * work counters: equal, count for count.
"""
import numpy as np
import pytest
import torch

import bench
import oracle
import stepper
from mwdiem_gb300 import scene

pytestmark = pytest.mark.gpu

GJK8_EPA32G = 8 | (32 << 8) | (1 << 16)
GJK1_EPA16G = 1 | (16 << 8) | (1 << 16)


def oriented(p):
    return set(map(tuple, np.asarray(p).reshape(-1, 2).tolist()))


def bits_equal(a, b):
    a, b = np.array(a, dtype=np.float32), np.array(b, dtype=np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    a[na] = 0
    b[nb] = 0
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


def device_pairs(sim, cull):
    """The broad phase's list from the simulator's current state, with or without the sphere filter."""
    sim.work.cull_pairs = 1 if cull else 0
    sim.broadphase()
    sim.check_status()
    return sim.pairs().cpu().numpy().copy()


def check_scene_rows(sim, spec, r0, r1, pairs_full, pairs_cut, coll_cut):
    """Candidate sets and flags of the scene occupying rows [r0, r1) of `sim` against the oracle.
    Returns the oracle's output on the scene's culled list (local row numbers) and that list."""
    ref = stepper.RefStepper(spec)
    pos = sim.t["pos"][r0:r1, :3].cpu().numpy()
    ref.st["com"][:] = pos
    want = ref.candidate_pairs()
    mine = pairs_full[(pairs_full[:, 0] >= r0) & (pairs_full[:, 0] < r1)] - r0
    assert len(mine) == len(want)
    assert oriented(mine) == oriented(want)
    sel = (pairs_cut[:, 0] >= r0) & (pairs_cut[:, 0] < r1)
    cut = pairs_cut[sel]
    kept = oriented(cut - r0)
    assert kept <= oriented(mine)
    inp = stepper.gather_from_sim(sim, mine + r0, ref.V)
    inp["A_id"], inp["B_id"] = mine[:, 0].astype(np.int32), mine[:, 1].astype(np.int32)
    o_full = oracle.contact(inp, ref.params, r1 - r0, "f32")
    dropped = np.array([tuple(p) not in kept for p in mine.tolist()], dtype=bool)
    assert np.all(o_full["collision"][dropped] == 0)
    flag = dict(zip(map(tuple, mine.tolist()), o_full["collision"].tolist()))
    got = dict(zip(map(tuple, (cut - r0).tolist()), coll_cut[sel].tolist()))
    assert all(flag[k] == v for k, v in got.items())
    return o_full, cut - r0, ref


def pour_checkpoint(sim, spec, det):
    """One full step at the simulator's state (broad phase, narrow phase, integrator), checked."""
    W = spec.n_walls
    full = device_pairs(sim, cull=False)
    cut = device_pairs(sim, cull=True)
    sim.narrow_force()
    torch.cuda.synchronize()
    coll = sim.w["collision"][: len(cut)].cpu().numpy()
    o_full, _, ref = check_scene_rows(sim, spec, 0, sim.n, full, cut, coll)
    assert (coll == 1).sum() > 0   # at rest on a 2.6-spaced lattice: ~50 contacts at step 0, ~10 later
    F = sim.t["force"][:, :3].cpu().numpy()
    T = sim.t["torque"][:, :3].cpu().numpy()
    assert np.all(F[:W] == 0)
    assert np.abs(F[W:] - o_full["force"][W:]).max() <= 1e-5 * np.abs(o_full["force"][W:]).max()
    assert np.abs(T[W:] - o_full["torque"][W:]).max() <= 1e-5 * np.abs(o_full["torque"][W:]).max()
    # deterministic sums on a copy of the state: bit-identical to the oracle's serial loop over the
    # same (cell-ordered) list
    det.load_from(sim)
    det.broadphase()
    dp = det.pairs().cpu().numpy()
    assert oriented(dp) == oriented(cut)
    det.narrow_force()
    torch.cuda.synchronize()
    o = oracle.contact(stepper.gather_from_sim(det, dp, ref.V), ref.params, det.n, "f32")
    assert bits_equal(det.t["force"][W:, :3].cpu().numpy(), o["force"][W:])
    assert bits_equal(det.t["torque"][W:, :3].cpu().numpy(), o["torque"][W:])
    det.t["force"].zero_()
    det.t["torque"].zero_()
    sim.integrate()
    sim.check_status()
    return int((coll == 1).sum())


class _Copy:
    """A deterministic-mode simulator that takes another simulator's state."""

    def __init__(self, spec, lanes):
        from mwdiem_gb300.sim import Simulator
        self.sim = Simulator(spec, lanes=lanes, collect_collisions=True, cull_pairs=True, deterministic=True)

    def load_from(self, other):
        for k in other.MUTABLE + ("world_verts", "info"):
            self.sim.t[k].copy_(other.t[k])

    def __getattr__(self, k):
        return getattr(self.sim, k)


@pytest.mark.parametrize("lanes", [GJK8_EPA32G, GJK1_EPA16G])
def test_pour20k_bench_scene_matches_oracle(lanes):
    from mwdiem_gb300.sim import Simulator
    spec = bench.build_scene(bench.SCENE["seed"])
    assert spec.n_particles == bench.N_PARTICLES
    sim = Simulator(spec, lanes=lanes, collect_collisions=True, cull_pairs=True)
    assert sim.total_cells > 65536   # the tiled cell scan
    det = _Copy(spec, lanes)
    contacts0 = pour_checkpoint(sim, spec, det)
    # 25 more steps the benchmark's way: one captured step graph, replayed
    sim.capture(1)
    sim.replay(24)
    torch.cuda.synchronize()
    assert sim.nonfinite_rows() == 0
    contacts25 = pour_checkpoint(sim, spec, det)
    print(f"pour20k lanes {lanes:#x}: contacts {contacts0} at step 0, {contacts25} at step 26")


@pytest.mark.parametrize("table", ["dense", "compressed"])
def test_batched_subset_matches_oracle(table):
    # the broad phase with either cell table (automatic: dense)
    from mwdiem_gb300.sim import Simulator
    specs = scene.batched_scenes(n_scenes=1, total=50_000, n_lo=50_000, n_hi=50_000, seed=11) + \
        scene.batched_scenes(n_scenes=15, total=60_000, seed=12)
    assert max(sp.n_particles for sp in specs) == 50_000
    sim = Simulator(specs, collect_collisions=True, cull_pairs=True, cell_table=table)
    assert sim.total_cells > 65536 and sim.cell_table_in_use == table
    for step in range(2):
        full = device_pairs(sim, cull=False)
        cut = device_pairs(sim, cull=True)
        sim.narrow_force()
        torch.cuda.synchronize()
        coll = sim.w["collision"][: len(cut)].cpu().numpy()
        F = sim.t["force"][:, :3].cpu().numpy()
        kinds = set()
        for i, sp in enumerate(specs):
            r0, r1 = sim.layout.row_begin[i], sim.layout.row_end[i]
            o, _, _ = check_scene_rows(sim, sp, r0, r1, full, cut, coll)
            W = sp.n_walls
            fo = o["force"][W:]
            if np.abs(fo).max() > 0:
                assert np.abs(F[r0 + W:r1] - fo).max() <= 1e-5 * np.abs(fo).max()
            nv = np.diff(sim.vert_off_host)[r0 + W:r1]
            kinds |= set(np.unique(nv).tolist())
        assert {4, 8} <= kinds and max(kinds) >= 12   # tetrahedra, cubes and hulls
        assert (coll == 1).sum() > 10   # scenes start at rest on lattices: ~100 contacts
        # advance a few steps between the two checks
        sim.integrate()
        sim.step(3)
        torch.cuda.synchronize()
    sim.check_status()


def test_compressed_cell_table_lists_the_dense_tables_pairs():
    # pour20k with both cell tables in deterministic mode (the list in cell order): the same sorted
    # rows, the same pair lists entry for entry, and the same states step after step
    from mwdiem_gb300.sim import Simulator
    spec = bench.build_scene(bench.SCENE["seed"])
    a = Simulator(spec, cull_pairs=True, deterministic=True, cell_table="dense")
    b = Simulator(spec, cull_pairs=True, deterministic=True, cell_table="compressed")
    assert a.cell_table_in_use == "dense" and b.cell_table_in_use == "compressed"
    assert Simulator(spec).cell_table_in_use == "dense"   # automatic: the dense table (140k cells)
    for _ in range(3):
        for cull in (False, True):
            pa, pb = device_pairs(a, cull), device_pairs(b, cull)
            assert len(pa) > 1000 and np.array_equal(pa, pb)
            assert torch.equal(a.w["sorted"], b.w["sorted"])
        assert int(b.w["cell_count"].abs().sum()) == 0   # left zero, as the dense table's counts
        a.step(10)
        b.step(10)
        for k in a.MUTABLE:
            assert torch.equal(a.t[k], b.t[k]), k
    a.check_status()
    b.check_status()


@pytest.mark.parametrize("box,table,cells", [(1500.0, "compressed", 5_000_000), (8000.0, "auto", 1 << 27)])
def test_compressed_cell_table_on_a_sparse_domain(box, table, cells):
    # 5,000 hulls in a 1,550-wide box (5.4M cells; the compressed table on request) and in an
    # 8,050-wide one (beyond 2^27 cells: the automatic choice).  The compressed table's arrays take a
    # small fraction of the dense table's memory and list the reference's oriented candidates
    from mwdiem_gb300.sim import Simulator
    sp = scene.pour_scene(n=5000, seed=3, box=box)
    sim = Simulator(sp, cull_pairs=False, cell_table=table)
    assert sim.cell_table_in_use == "compressed" and sim.total_cells > cells
    assert sim.w["cell_count"].numel() + sim.w["cell_start"].numel() < 0.15 * (2 * sim.total_cells + 1)
    for _ in range(2):
        pairs = device_pairs(sim, cull=False)
        ref = stepper.RefStepper(sp)
        ref.st["com"][:] = sim.t["pos"][:, :3].cpu().numpy()
        want = ref.candidate_pairs()
        assert len(pairs) == len(want) > 1000 and oriented(pairs) == oriented(want)
        sim.step(5)
        torch.cuda.synchronize()
    sim.check_status()


def test_narrow_4m_pairs_sample_matches_oracle():
    # the narrow-phase benchmark's own pairs (bench.py: 4M pairs, seed 1) and its lane setting
    from mwdiem_gb300.pairbench import PairScene
    n = 1 << 22
    ps = PairScene(n, seed=1, lanes=GJK1_EPA16G)
    ps.narrow()
    torch.cuda.synchronize()
    coll = ps.w["collision"].cpu().numpy()
    assert set(np.unique(coll)) <= {-1, 0, 1}
    idx = np.sort(np.random.default_rng(5).choice(n, size=131072, replace=False))
    o = oracle.contact(ps.gather(idx), ps.params, 2 * n, "f32")
    assert np.array_equal(coll[idx], o["collision"])
    rows = np.concatenate([2 * idx, 2 * idx + 1])
    F = ps.t["force"][:, :3].cpu().numpy()
    T = ps.t["torque"][:, :3].cpu().numpy()
    assert bits_equal(F[rows], o["force"][rows]) and bits_equal(T[rows], o["torque"][rows])
    del ps
    torch.cuda.empty_cache()


def spheres_apart_host(pa, pb):
    """The narrow phase's bounding-sphere pre-test (common.cuh spheres_apart) in float32, same order."""
    f = np.float32
    d = (pb[:, :3] - pa[:, :3]).astype(f)
    mag = np.abs(pa[:, :3].astype(f)).max(1) + np.abs(pb[:, :3].astype(f)).max(1)
    r = (pa[:, 3] + pb[:, 3]).astype(f) * f(1.001) + f(1e-5) * mag + f(1e-6)
    return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2] > r * r


def oracle_work(o, inp, run):
    """(vertex dot products, EPA faces, support queries) of the oracle over the pairs in `run`."""
    nsup = o["counters"][run, 0].astype(np.int64)
    dots = int((nsup * (inp["A_nv"][run].astype(np.int64) + inp["B_nv"][run])).sum())
    faces = int(o["counters"][run, 9][o["collision"][run] == 1].astype(np.int64).sum())
    return dots, faces, int(nsup.sum())


@pytest.mark.parametrize("lanes", [8, GJK1_EPA16G])
def test_work_counters_equal_oracle_counts_pairs(lanes):
    from mwdiem_gb300.pairbench import PairScene
    ps = PairScene(6000, seed=3, pool=96, lanes=lanes)
    ps.narrow(count_work=True)
    torch.cuda.synchronize()
    got = tuple(int(x) for x in ps.w["counters"].cpu().numpy())
    idx = np.arange(6000)
    inp = ps.gather(idx)
    o = oracle.contact(inp, ps.params, 12000, "f32")
    assert not np.any(o["status"] & oracle.ST_EPA_OVERFLOW)
    pos = ps.t["pos"].cpu().numpy()
    run = ~spheres_apart_host(pos[0::2], pos[1::2])   # the pairs the kernel runs GJK on
    assert 0 < (~run).sum() < 6000
    assert got == oracle_work(o, inp, run)
    # with the list marked as pre-filtered every pair runs GJK
    ps.work.cull_pairs = 1
    ps.t["force"].zero_()
    ps.t["torque"].zero_()
    ps.narrow(count_work=True)
    torch.cuda.synchronize()
    got_all = tuple(int(x) for x in ps.w["counters"].cpu().numpy())
    assert got_all == oracle_work(o, inp, np.ones(6000, dtype=bool))


@pytest.mark.parametrize("lanes", [GJK8_EPA32G, GJK1_EPA16G])
def test_work_counters_equal_oracle_counts_pour(lanes):
    from mwdiem_gb300.sim import Simulator
    spec = bench.build_scene(bench.SCENE["seed"])
    sim = Simulator(spec, lanes=lanes, collect_collisions=True, cull_pairs=True)
    sim.step(5)
    sim.broadphase()
    pairs = sim.pairs().cpu().numpy()
    got = sim.count_narrow_work()
    ref = stepper.RefStepper(spec)
    inp = stepper.gather_from_sim(sim, pairs, ref.V)
    o = oracle.contact(inp, ref.params, sim.n, "f32")
    assert not np.any(o["status"] & oracle.ST_EPA_OVERFLOW)
    assert got == oracle_work(o, inp, np.ones(len(pairs), dtype=bool))
