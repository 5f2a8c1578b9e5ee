"""Device-resident step (``mwd_step``: broad phase -> narrow phase + force -> integrator) against the
reference's per-step CPU path restated in oracle/stepper.py (Linked_cell_hash + wall test, the FP32
contact kernel, the FP64 Verlet kernel).

Bars:
  * candidate pairs: the same set of oriented pairs as the reference path, from the same state;
  * contact flags: identical to the FP32 oracle fed the GPU's own world-frame vertices;
  * contact forces before integration: within 1e-5 of the largest force (float atomics reorder sums);
  * short horizon (<= 100 steps) against the FP64 reference path: positions within 2e-6 of the scene
    size, velocities within 1e-3 of the largest speed, quaternions within 1e-4 (FP32 state on the GPU).
"""
import numpy as np
import pytest
import torch

import oracle
import stepper
from helpers import head_on_cubes
from mwdiem_gb300 import scene

pytestmark = pytest.mark.gpu


def dense_scene(n=600, seed=0, spacing=2.05, vel=0.5):
    sp = scene.pour_scene(n=n, seed=seed, box=16.0, spacing=spacing, pool=48)
    rng = np.random.default_rng(seed + 100)
    sp.velocities = rng.normal(size=(n, 3)) * vel
    return sp


def oriented(p):
    return set(map(tuple, np.asarray(p).reshape(-1, 2).tolist()))


def test_pairs_flags_forces_step0():
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene()
    sim = Simulator(sp, collect_collisions=True, cull_pairs=False)
    ref = stepper.RefStepper(sp)
    sim.broadphase()
    pairs = sim.pairs().cpu().numpy()
    want = ref.candidate_pairs()
    assert len(pairs) == len(want)
    assert oriented(pairs) == oriented(want)
    sim.narrow_force()
    torch.cuda.synchronize()
    coll = sim.w["collision"][: len(pairs)].cpu().numpy()
    inp = stepper.gather_from_sim(sim, pairs, ref.V)
    o = oracle.contact(inp, ref.params, sim.n, "f32")
    assert np.array_equal(coll, o["collision"])
    assert (coll == 1).sum() > 50
    W = sp.n_walls
    F = sim.t["force"][:, :3].cpu().numpy()
    T = sim.t["torque"][:, :3].cpu().numpy()
    scale = np.abs(o["force"][W:]).max()
    assert np.abs(F[W:] - o["force"][W:]).max() <= 1e-5 * scale
    assert np.abs(T[W:] - o["torque"][W:]).max() <= 1e-5 * np.abs(o["torque"][W:]).max()
    assert np.all(F[:W] == 0)
    sim.check_status()


# (scene, steps): the dense scene starts with overlaps at speeds ~10 and is compared over 20 steps;
# over longer horizons its trajectories separate because the contact law is discontinuous at first
# touch (the damping term Gn u_n does not vanish with the depth), so a contact that starts one step
# earlier in FP32 than in FP64 changes the force by O(1).  The 100-step comparison uses a scene whose
# contacts start gently.
@pytest.mark.parametrize("kind,steps", [("dense", 20), ("gentle", 100)])
def test_short_horizon_vs_fp64_reference_path(kind, steps):
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=400, seed=3) if kind == "dense" else dense_scene(n=400, seed=3, spacing=2.45, vel=0.05)
    sim = Simulator(sp)
    ref = stepper.RefStepper(sp)
    for _ in range(steps):
        ref.step()
    sim.step(steps)
    torch.cuda.synchronize()
    W = sp.n_walls
    g = sim.reference_state()
    size = 16.0
    dpos = np.abs(g["com"][W:] - ref.st["com"][W:]).max()
    vmax = np.abs(ref.st["v"][W:]).max()
    dvel = np.abs(g["v"][W:] - ref.st["v"][W:]).max()
    dq = np.abs(g["q"][W:] - ref.st["q"][W:]).max()
    print(f"{kind} steps {steps}: |dpos| {dpos:.3e} |dv| {dvel:.3e} (vmax {vmax:.3e}) |dq| {dq:.3e}")
    assert dpos <= 2e-6 * size
    assert dvel <= 1e-3 * vmax
    assert dq <= 1e-4


def test_host_round_trip_matches_device_stepping():
    # the public host-buffer path (state in pinned host memory, one copy each way per call) gives the
    # same state as stepping on the device (deterministic sums, so bit for bit)
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=300, seed=5, spacing=2.3, vel=0.2)
    a = Simulator(sp, deterministic=True)
    b = Simulator(sp, deterministic=True)
    host = a.host_state()
    assert a.host_state_bytes() == sum(host[k].numel() * host[k].element_size() for k in a.MUTABLE)
    for _ in range(4):
        a.step_host(host, 2)
    b.step(8)
    torch.cuda.synchronize()
    for k in a.MUTABLE:
        assert torch.equal(host[k], b.t[k].cpu()), k


@pytest.mark.parametrize("mirror", [True, False])
def test_host_graph_matches_device_stepping(mirror):
    # the captured host step (centres copied in first, the broad phase overlapping the copy of the
    # rest of the state; the state back through the integrator's mirrored writes or by a copy) gives
    # the state of plain device steps, bit for bit (deterministic sums)
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=300, seed=8, spacing=2.3, vel=0.2)
    a = Simulator(sp, deterministic=True)
    b = Simulator(sp, deterministic=True)
    host = a.host_state()
    a.capture_host(host, mirror=mirror)         # one warm-up step through the plain host path
    assert a.host_graph_mirrored == mirror
    for _ in range(6):
        a.step_host(host, 1)     # graph replays
    b.step(7)
    torch.cuda.synchronize()
    assert a.steps_done == 7
    for k in a.MUTABLE:
        assert torch.equal(host[k], b.t[k].cpu()), k
    with pytest.raises(ValueError):
        a.capture_host({"_buffer": torch.zeros(16, dtype=torch.uint8).pin_memory()})


def test_snapshot_resume_continues_identically(tmp_path):
    # save after 5 steps, load into a fresh simulator of the same scene, 5 more steps on both:
    # identical states (deterministic sums), persistent history included
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=300, seed=6, spacing=2.2, vel=0.3)
    a = Simulator(sp, deterministic=True, persistent_history=True)
    a.step(5)
    f = tmp_path / "snap.npz"
    a.save(f)
    b = Simulator(sp, deterministic=True, persistent_history=True)
    b.load(f)
    assert b.steps_done == 5
    a.step(5)
    b.step(5)
    torch.cuda.synchronize()
    for k in a.SNAPSHOT:
        assert torch.equal(a.t[k], b.t[k]), k
    plain = Simulator(sp)
    plain.save(tmp_path / "plain.npz")
    with pytest.raises(ValueError):
        b.load(tmp_path / "plain.npz")  # no history tables in it


def test_graph_replay_matches_stepping():
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=500, seed=5)
    a = Simulator(sp)
    b = Simulator(sp)
    a.step(11)
    b.capture(steps_per_replay=5)   # one warm-up step + 2 replays of 5
    b.replay(2)
    torch.cuda.synchronize()
    pa, pb = a.positions().cpu().numpy(), b.positions().cpu().numpy()
    assert np.abs(pa - pb).max() <= 1e-6 * 16.0
    assert a.n_pairs() == b.n_pairs()


def test_multi_step_overlap_is_exact():
    # one call of ten steps rewrites each step's world vertices during the next step's broad phase, on
    # a second stream; with deterministic sums it must give the bits of ten one-step calls, eagerly
    # and from a ten-step graph
    from mwdiem_gb300.sim import Simulator
    sp = scene.pour_scene(n=6000, seed=17, box=40.0, spacing=2.05, pool=48)
    sp.velocities = np.random.default_rng(117).normal(size=(6000, 3)) * 0.5
    a = Simulator(sp, deterministic=True)
    b = Simulator(sp, deterministic=True)
    c = Simulator(sp, deterministic=True)
    for _ in range(11):
        a.step(1)
    b.step(1)
    b.step(10)
    c.capture(steps_per_replay=10)   # one eager warm-up step, then the graph
    c.replay(1)
    torch.cuda.synchronize()
    assert a.n_pairs() > 100
    for k in ("pos", "q", "vel", "w", "world_verts"):
        ta = a.t[k].cpu().numpy()
        for o in (b, c):
            assert np.array_equal(ta, o.t[k].cpu().numpy(), equal_nan=True), k


def test_one_kernel_integrator_matches_two_passes():
    # from two full waves of blocks the integrator updates each block's rows and then their vertices in
    # one kernel; it must give the bits of the row pass + vertex pass, and a ten-step call (which then
    # runs without the vertex-pass overlap) those of ten one-step calls
    from mwdiem_gb300 import _lib
    from mwdiem_gb300.sim import Simulator
    specs = scene.batched_scenes(n_scenes=10, total=340_000, n_lo=34_000, n_hi=34_000, seed=5)
    a = Simulator(specs, deterministic=True)
    b = Simulator(specs, deterministic=True)
    assert _lib.lib().mwd_integrate_kernels(a.n) == 1 and _lib.lib().mwd_integrate_kernels(20_000) == 2
    for _ in range(3):
        for s in (a, b):
            s.broadphase()
            s.narrow_force()
        a.integrate()
        b.integrate_rows()
        b.world_vertices()
        torch.cuda.synchronize()
        for k in a.MUTABLE + ("force", "torque", "world_verts"):
            assert torch.equal(a.t[k], b.t[k]), k
    assert a.n_pairs() > 1000
    c = Simulator(specs, deterministic=True)
    d = Simulator(specs, deterministic=True)
    c.step(10)
    for _ in range(10):
        d.step(1)
    torch.cuda.synchronize()
    for k in ("pos", "q", "vel", "w", "world_verts"):
        assert torch.equal(c.t[k], d.t[k]), k
    a.check_status()


def test_multi_step_calls_from_two_threads():
    # two host threads, each stepping its own simulator ten steps per call on its own stream (each
    # thread has its own overlap stream and events): the bits of the same calls made one after another
    import threading
    from mwdiem_gb300.sim import Simulator
    specs = [dense_scene(n=500, seed=31), dense_scene(n=700, seed=32)]
    ref = [Simulator(sp, deterministic=True) for sp in specs]
    for r in ref:
        r.step(10)
    torch.cuda.synchronize()
    sims = [Simulator(sp, deterministic=True) for sp in specs]
    torch.cuda.synchronize()  # their set-up ran on the default stream
    errors = []

    def run(sim):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                sim.step(10)
            s.synchronize()
        except Exception as e:  # reported by the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(sim,)) for sim in sims]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    torch.cuda.synchronize()
    assert not errors, errors
    for r, sim in zip(ref, sims):
        for k in ("pos", "q", "vel", "world_verts"):
            assert np.array_equal(r.t[k].cpu().numpy(), sim.t[k].cpu().numpy(), equal_nan=True), k


def test_batched_equals_separate():
    from mwdiem_gb300.sim import Simulator
    specs = [dense_scene(n=n, seed=s) for n, s in ((300, 7), (700, 8), (120, 9))]
    batch = Simulator(specs)
    batch.broadphase()
    bp = batch.pairs().cpu().numpy()
    off = 0
    for i, sp in enumerate(specs):
        one = Simulator(sp)
        one.broadphase()
        p1 = one.pairs().cpu().numpy()
        r0, r1 = batch.layout.row_begin[i], batch.layout.row_end[i]
        mine = bp[(bp[:, 0] >= r0) & (bp[:, 0] < r1)] - r0
        assert oriented(mine) == oriented(p1)
        off += r1 - r0
    batch.step(30)
    for i, sp in enumerate(specs):
        one = Simulator(sp)
        one.step(30)
        torch.cuda.synchronize()
        rows = batch.particle_rows(i)
        d = np.abs(batch.positions()[rows].cpu().numpy() - one.positions(0).cpu().numpy()).max()
        assert d <= 1e-6 * 16.0


def test_two_pass_equals_single_pass():
    # the GJK pass + EPA pass split must not change any decision: same flags, same forces up to the
    # float-atomic summation order
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=800, seed=11)
    one = Simulator(sp, collect_collisions=True, two_pass=False)
    two = Simulator(sp, collect_collisions=True, two_pass=True)
    for s in (one, two):
        s.broadphase()
        s.narrow_force()
    torch.cuda.synchronize()
    n = one.n_pairs()
    assert n == two.n_pairs()
    # the device step's pair list holds the same pairs in a run-dependent order: compare by pair
    f1 = dict(zip(map(tuple, one.pairs().cpu().numpy().tolist()), one.w["collision"][:n].cpu().numpy().tolist()))
    f2 = dict(zip(map(tuple, two.pairs().cpu().numpy().tolist()), two.w["collision"][:n].cpu().numpy().tolist()))
    assert f1 == f2 and sum(v == 1 for v in f1.values()) > 100
    F1, F2 = one.t["force"].cpu().numpy(), two.t["force"].cpu().numpy()
    assert np.abs(F1 - F2).max() <= 1e-5 * np.abs(F1).max()
    T1, T2 = one.t["torque"].cpu().numpy(), two.t["torque"].cpu().numpy()
    assert np.abs(T1 - T2).max() <= 1e-5 * np.abs(T1).max()


def test_sphere_filter_drops_only_noncontacts():
    # with cull_pairs the broad phase lists a subset of the reference's candidates; every dropped
    # candidate must be one the FP32 oracle, fed the GPU's own vertices, classifies "no contact"
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=700, seed=12)
    full = Simulator(sp, collect_collisions=True, cull_pairs=False)
    cut = Simulator(sp, collect_collisions=True, cull_pairs=True)
    full.broadphase()
    cut.broadphase()
    pf = full.pairs().cpu().numpy()
    pc = cut.pairs().cpu().numpy()
    kept = oriented(pc)
    assert kept <= oriented(pf) and len(kept) < len(pf)
    ref = stepper.RefStepper(sp)
    o = oracle.contact(stepper.gather_from_sim(full, pf, ref.V), ref.params, full.n, "f32")
    dropped = np.array([tuple(p) not in kept for p in pf.tolist()])
    assert np.all(o["collision"][dropped] == 0)
    assert np.all(o["counters"][dropped, 0] == 1)   # settled by the first support query
    cut.narrow_force()
    full.narrow_force()
    torch.cuda.synchronize()
    F1, F2 = full.t["force"].cpu().numpy(), cut.t["force"].cpu().numpy()
    assert np.abs(F1 - F2).max() <= 1e-5 * np.abs(F1).max()


def test_wall_test_band_defers_to_fp64():
    # centres placed within float rounding of the wall range (|n . (p - c)| = wall_range + eps): the
    # device step's FP32 wall test must hand these to its FP64 test and list exactly the wall pairs
    # of MWDiem.py:808-811
    from mwdiem_gb300.sim import Simulator
    sp = scene.pour_scene(n=300, seed=4, box=16.0, spacing=2.6, pool=16)
    rng = np.random.default_rng(9)
    floor_c = np.asarray(sp.walls[0][1], float)
    rng_w = 6.0 * sp.max_particlesize
    eps = np.array([0.0, 1e-12, -1e-12, 1e-9, -1e-9, 1e-7, -1e-7, 1e-6, -1e-6, 1e-5, -1e-5, 1e-4, -1e-4, 1e-3, -1e-3])
    k = len(eps) * 4
    sp.centres = sp.centres.copy()
    sp.centres[:k, 2] = floor_c[2] + rng_w + np.tile(eps, 4)
    sp.centres[:k, 0] = rng.uniform(-6, 6, size=k)
    sp.centres[:k, 1] = rng.uniform(-6, 6, size=k)
    sim = Simulator(sp, cull_pairs=False)
    sim.broadphase()
    got = {tuple(p) for p in sim.pairs().cpu().numpy().tolist() if p[1] < sp.n_walls}
    ref = stepper.RefStepper(sp)
    want = {tuple(p) for p in ref.candidate_pairs().tolist() if p[1] < sp.n_walls}
    assert got == want
    near = {sp.n_walls + i for i in range(k)}
    assert {p for p in want if p[0] in near and p[1] == 0}, "the band rows should include floor pairs"


@pytest.mark.parametrize("lanes", [8, 1 | (16 << 8) | (1 << 16)])
def test_deterministic_sums_equal_serial_loop(lanes):
    # deterministic mode: each particle's force and torque are summed in pair-list order, so they are
    # bit-identical to the oracle's serial loop over the same list (the reference's host build order)
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=700, seed=13)
    sim = Simulator(sp, collect_collisions=True, cull_pairs=False, deterministic=True, lanes=lanes)
    sim.broadphase()
    pairs = sim.pairs().cpu().numpy()
    sim.narrow_force()
    torch.cuda.synchronize()
    ref = stepper.RefStepper(sp)
    o = oracle.contact(stepper.gather_from_sim(sim, pairs, ref.V), ref.params, sim.n, "f32")
    coll = sim.w["collision"][: len(pairs)].cpu().numpy()
    assert np.array_equal(coll, o["collision"]) and (coll == 1).sum() > 100
    W = sp.n_walls
    F = sim.t["force"][W:, :3].cpu().numpy()
    T = sim.t["torque"][W:, :3].cpu().numpy()
    assert np.array_equal(F, o["force"][W:], equal_nan=True)
    assert np.array_equal(T, o["torque"][W:], equal_nan=True)


def test_deterministic_mode_is_reproducible():
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=500, seed=14)
    runs = []
    for _ in range(2):
        sim = Simulator(sp, deterministic=True)
        sim.step(20)
        torch.cuda.synchronize()
        runs.append((sim.t["pos"].cpu().numpy(), sim.t["q"].cpu().numpy(), sim.pairs().cpu().numpy(),
                     sim.t["vel"].cpu().numpy()))
    # NaN rows (the reference's contact law can produce them in violent scenes) compare equal to NaN
    diff = ~((runs[0][0] == runs[1][0]) | (np.isnan(runs[0][0]) & np.isnan(runs[1][0]))).all(1)
    print("rows differing:", int(diff.sum()), "non-finite rows:", int((~np.isfinite(runs[0][0])).any(1).sum()))
    assert np.array_equal(runs[0][2], runs[1][2])
    assert not diff.any()
    assert np.array_equal(runs[0][1], runs[1][1], equal_nan=True)
    assert np.array_equal(runs[0][3], runs[1][3], equal_nan=True)


def test_settling_config1_short_horizon():
    # the settling scene (125 unit cubes on a 5^3 lattice at spacing 1.5, random orientations, onto a floor,
    # dt 1e-4): rotated cubes reach 0.87 from their centres, so neighbours overlap from step 0 and the
    # reference path's motion turns violent within the first hundred steps; the FP32 device step is
    # compared with the FP64 reference path over the first 20 steps
    from mwdiem_gb300.sim import Simulator
    sp = scene.settling_scene()
    sim = Simulator(sp, collect_collisions=True)
    ref = stepper.RefStepper(sp)
    steps = 20
    for _ in range(steps):
        ref.step()
    sim.step(steps)
    torch.cuda.synchronize()
    assert (ref.last_collision == 1).sum() > 20
    W = sp.n_walls
    g = sim.reference_state()
    size = 10.0
    dpos = np.abs(g["com"][W:] - ref.st["com"][W:]).max()
    vmax = np.abs(ref.st["v"][W:]).max()
    dvel = np.abs(g["v"][W:] - ref.st["v"][W:]).max()
    dq = np.abs(g["q"][W:] - ref.st["q"][W:]).max()
    print(f"settling scene, {steps} steps: |dpos| {dpos:.3e} |dv| {dvel:.3e} (vmax {vmax:.3e}) |dq| {dq:.3e}")
    assert dpos <= 2e-6 * size
    assert dvel <= 1e-3 * vmax
    assert dq <= 1e-4


@pytest.mark.parametrize("lanes", [8, 1 | (16 << 8) | (1 << 16)])
def test_persistent_history_matches_oracle_over_steps(lanes):
    # the history of every pair in contact carries over to the next step (the reference drops it,
    # MWDiem.py:953-966); checked step by step against the oracle's stride-4 history variant fed the
    # same pair list and a host dictionary of the histories, with bit-exact (deterministic) sums
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=400, seed=21, vel=0.3)
    sim = Simulator(sp, collect_collisions=True, cull_pairs=False, deterministic=True, persistent_history=True,
                    lanes=lanes)
    ref = stepper.RefStepper(sp)
    W = sp.n_walls
    table = {}
    reused = 0
    for step in range(6):
        sim.broadphase()
        pairs = sim.pairs().cpu().numpy()
        inp = stepper.gather_from_sim(sim, pairs, ref.V)
        hist = np.zeros((len(pairs), 4), np.float32)
        for k, (a, b) in enumerate(pairs.tolist()):
            v = table.get((min(a, b), max(a, b)))
            if v is not None:
                hist[k, :3] = v if a < b else -v
                reused += 1
        inp["hist"] = hist
        o = oracle.contact(inp, ref.params, sim.n, "f32", hist_stride4=True)
        sim.narrow_force()
        torch.cuda.synchronize()
        coll = sim.w["collision"][: len(pairs)].cpu().numpy()
        assert np.array_equal(coll, o["collision"])
        assert np.array_equal(sim.t["force"][W:, :3].cpu().numpy(), o["force"][W:], equal_nan=True)
        assert np.array_equal(sim.t["torque"][W:, :3].cpu().numpy(), o["torque"][W:], equal_nan=True)
        new = {}
        for k in np.nonzero(o["collision"] == 1)[0]:
            a, b = int(pairs[k, 0]), int(pairs[k, 1])
            v = o["hist"][k, :3].astype(np.float32)
            new[(min(a, b), max(a, b))] = v if a < b else -v
        got = sim.history_table()
        assert set(got) == set(new)
        for key, v in new.items():
            assert np.array_equal(got[key], v, equal_nan=True), key
        table = new
        sim.integrate()
    assert reused > 50, "contacts should carry their history across steps"


def test_physical_law_sums_equal_oracle():
    # the physical-mass contact law (effective masses, midpoint contact point): per-particle sums in
    # pair-list order, bit-identical to the oracle's serial loop running the same law
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=600, seed=17)
    sp.law = "physical"
    sim = Simulator(sp, collect_collisions=True, cull_pairs=False, deterministic=True)
    sim.broadphase()
    pairs = sim.pairs().cpu().numpy()
    sim.narrow_force()
    torch.cuda.synchronize()
    ref = stepper.RefStepper(sp)
    o = oracle.contact(stepper.gather_from_sim(sim, pairs, ref.V), ref.params, sim.n, "f32",
                       inv_mass=stepper.inv_mass_from_sim(sim, pairs))
    coll = sim.w["collision"][: len(pairs)].cpu().numpy()
    assert np.array_equal(coll, o["collision"]) and (coll == 1).sum() > 100
    W = sp.n_walls
    assert np.array_equal(sim.t["force"][W:, :3].cpu().numpy(), o["force"][W:], equal_nan=True)
    assert np.array_equal(sim.t["torque"][W:, :3].cpu().numpy(), o["torque"][W:], equal_nan=True)
    sim.check_status()


@pytest.mark.parametrize("kind,steps", [("dense", 20), ("gentle", 100)])
def test_physical_law_short_horizon(kind, steps):
    # the physical law against the FP64 reference path running the same law (principal-axes body
    # frames, vertices turned by each step's rotation), same scenes and bars as the reference law
    from mwdiem_gb300.sim import Simulator
    sp = dense_scene(n=400, seed=3) if kind == "dense" else dense_scene(n=400, seed=3, spacing=2.45, vel=0.05)
    sp.law = "physical"
    sim = Simulator(sp, collect_collisions=True)
    ref = stepper.RefStepper(sp)
    for _ in range(steps):
        ref.step()
    sim.step(steps)
    torch.cuda.synchronize()
    W = sp.n_walls
    g = sim.reference_state()
    dpos = np.abs(g["com"][W:] - ref.st["com"][W:]).max()
    vmax = np.abs(ref.st["v"][W:]).max()
    dvel = np.abs(g["v"][W:] - ref.st["v"][W:]).max()
    dq = np.abs(g["q"][W:] - ref.st["q"][W:]).max()
    print(f"physical law, {kind} {steps} steps: |dpos| {dpos:.3e} |dv| {dvel:.3e} (vmax {vmax:.3e}) |dq| {dq:.3e}")
    assert (ref.last_collision == 1).sum() > 5
    assert dpos <= 2e-6 * 16.0
    assert dvel <= 1e-3 * vmax
    assert dq <= 1e-4
    sim.check_status()


def test_physical_law_restitution():
    # a normal impact of two cubes of mass 4 rebounds with the restitution en of the law; the
    # reference's law, which uses mu = 0.5 as the effective mass (the true one is 2), damps it less
    # (and its contact point (cpA - cpB) / 2 spins the cubes)
    from mwdiem_gb300.sim import Simulator
    got = {}
    for law in ("physical", "reference"):
        sp = head_on_cubes(law)
        sim = Simulator(sp)
        sim.step(1500)  # contact starts after ~400 steps and lasts ~300 (tc = 0.0147 s, dt 5e-5)
        torch.cuda.synchronize()
        W = sp.n_walls
        v = sim.t["vel"][W:W + 2, :3].cpu().numpy()
        got[law] = -(v[0, 0] - v[1, 0]) / 1.0
    print("restitution:", got, "en", head_on_cubes("physical").en)
    en = head_on_cubes("physical").en
    assert abs(got["physical"] - en) < 0.02
    assert abs(got["reference"] - en) > 0.1


def test_inlet_rows_enter_on_schedule():
    # particles entering during the run (MWDiem.py:685-714): rows wait outside the broad phase and the
    # integrator and enter per_spawn at a time every period steps, also inside a captured graph
    from mwdiem_gb300.sim import InletSpec, Simulator
    sp = dense_scene(n=300, seed=31, vel=0.0)
    inl = InletSpec(period=5, per_spawn=2, initial=200, lo=(-5.0, -5.0, 15.5), hi=(5.0, 5.0, 17.5), seed=1)
    W = sp.n_walls
    eager = Simulator(sp, inlet=inl)
    assert int(eager.active_rows()[W:].sum()) == 200
    waiting0 = ~eager.active_rows().cpu().numpy()
    start = eager.t["pos"].cpu().numpy().copy()
    eager.step(30)
    torch.cuda.synchronize()
    act = eager.active_rows().cpu().numpy()
    assert act[W:].sum() == 200 + 2 * 6          # spawns at steps 0, 5, ..., 25
    entered = np.nonzero(act & waiting0)[0]
    assert np.array_equal(entered, np.arange(W + 200, W + 212))
    pos = eager.t["pos"].cpu().numpy()
    spawn = eager.inlet_t["spawn_pos"].cpu().numpy()
    # entered at rest at the spawn points (two entering together may overlap and push each other)
    assert np.all(np.abs(pos[entered, :3] - spawn[entered, :3]) < 0.05)
    assert np.all(pos[entered, 2] > 15.0)
    still = np.nonzero(~act)[0]
    assert np.array_equal(pos[still], start[still])                        # waiting rows untouched
    pairs = eager.pairs().cpu().numpy()
    assert not np.isin(pairs, still).any()
    graph = Simulator(sp, inlet=inl)
    graph.capture(1)                              # one eager step, then replays of the captured step
    graph.replay(29)
    torch.cuda.synchronize()
    assert np.array_equal(graph.active_rows().cpu().numpy(), act)
    assert np.abs(graph.t["pos"].cpu().numpy()[act] - pos[act]).max() <= 1e-6 * 16.0


def test_inlet_run_matches_reference_path():
    # the inlet's physics, not only its schedule: the reference path (oracle/stepper.py) runs the same
    # activation schedule with the same spawn points (MWDiem.py:685-714), and the 30-step run of the
    # device step must stay within the short-horizon bars of the reference path, rows entering
    # (some of them overlapping on arrival) included
    from mwdiem_gb300.sim import InletSpec, Simulator
    sp = dense_scene(n=300, seed=31, vel=0.0)
    inl = InletSpec(period=5, per_spawn=2, initial=200, lo=(-5.0, -5.0, 15.5), hi=(5.0, 5.0, 17.5), seed=1)
    W = sp.n_walls
    sim = Simulator(sp, inlet=inl, collect_collisions=True)
    spawn = sim.inlet_t["spawn_pos"][:, :3].cpu().numpy()
    ref = stepper.RefStepper(sp, inlet=(inl.period, inl.per_spawn, W + inl.initial, spawn))
    steps = 30
    for _ in range(steps):
        ref.step()
    sim.step(steps)
    torch.cuda.synchronize()
    act = sim.active_rows().cpu().numpy()
    assert int(act.sum()) == ref.active_end == W + 200 + 2 * 6
    rows = np.nonzero(act)[0]
    rows = rows[rows >= W]
    g = sim.reference_state()
    dpos = np.abs(g["com"][rows] - ref.st["com"][rows]).max()
    vmax = np.abs(ref.st["v"][rows]).max()
    dvel = np.abs(g["v"][rows] - ref.st["v"][rows]).max()
    dq = np.abs(g["q"][rows] - ref.st["q"][rows]).max()
    entered = np.arange(W + 200, W + 212)
    moved = np.abs(ref.st["v"][entered]).max()
    print(f"inlet, {steps} steps: |dpos| {dpos:.3e} |dv| {dvel:.3e} (vmax {vmax:.3e}) |dq| {dq:.3e}; "
          f"entered rows' largest speed {moved:.3e}")
    assert dpos <= 2e-6 * 16.0
    assert dvel <= 1e-3 * vmax
    assert dq <= 1e-4
    sim.check_status()
