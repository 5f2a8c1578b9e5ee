#!/usr/bin/env python
"""Benchmark: device-resident DEM steps of the 20,000-hull pour on one GB300 (particle-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = broad phase + narrow phase + contact force + integrator over the whole scene (one CUDA
graph replay).  The scene fits in L2 (~20 MB of state), so L2 is flushed (a 256 MB write) before
every timed step; each step is timed with CUDA events on the stream it runs on and the times are
summed.  `e2e` is the same step through the public host-buffer API (state copied from pinned host
memory to the device and back every step).  `roofline` covers the kernel that dominates the step.
`--impl reference` times the reference's own CPU path (oracle/stepper.py: its kernels compiled
for the host from their source when that build is available, else the oracle's restatement) on
this machine's host cores, on the same scene.  Under torchrun every rank runs an independent
replica (the scene does not shard; no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

N_PARTICLES = 20000
SCENE = dict(n=N_PARTICLES, seed=0, box=40.0, spacing=2.6, jitter=0.1, n_min=12, n_max=32, r_min=0.8, r_max=1.2,
             zeta=0.3, kn=1e5, mu=0.5, dt=5e-5)
WORKLOAD = ("pour20k: 20,000 convex hulls of U{12..32} points on a sphere of radius U[0.8,1.2], jittered "
            "lattice (spacing 2.6) in a 40x40 box, random orientations, at rest, gravity; kn 1e5, damping "
            "ratio 0.3 (en=et=0.372), mu 0.5, dt 5e-5")
class host_prints_to_stderr:
    """The reference's kernels report some cases with printf (e.g. "No min depth found!",
    gpu_fine_contact_detection.cu:437); while they run on the host their C-level stdout goes to
    stderr, so that stdout carries only this script's JSON line."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        os.dup2(2, 1)
        return self

    def __exit__(self, *exc):
        import ctypes
        ctypes.CDLL(None).fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)
        return False


METRIC = "particle-steps/s"
WINDOW_STEPS = 500  # the pour configuration runs 500 steps
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) of one GJK-pass and one EPA-pass
# launch of this step, from one capture of the eager first step: 5.185 MB + 0.169 MB (the writes stay
# in L2).  ncu cannot run inside this timing, so the figure is carried here.
NARROW_DRAM_BYTES_PER_LAUNCH = 5.184512e6 + 0.169472e6
# broad phase 4 (assign, cell scan, place, append) + GJK pass + EPA pass + EPA overflow reruns +
# integrator rows + vertices
KERNELS_PER_STEP = 9


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--lanes", type=lanes_arg, default=8,
                    help="lanes per pair: an integer, or a setting such as gjk8/epa32g (with --no-tune)")
    ap.add_argument("--no-tune", action="store_true", help="use --lanes instead of the autotuner's choice")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-breakdown", action="store_true")
    ap.add_argument("--pairs", type=int, default=1 << 22,
                    help="also time the narrow phase on this many independent random pairs (0: skip)")
    ap.add_argument("--pairs-only", action="store_true", help="only the independent-pair narrow-phase timing")
    ap.add_argument("--pairs-lanes", default=None,
                    help="lanes per pair for the pair timing, e.g. gjk1/epa16g (default: the sweep's best)")
    ap.add_argument("--batch-compare", action="store_true",
                    help="256 independent scenes (~2M particles): one batched graph step vs per-scene launches")
    ap.add_argument("--calibration", action="store_true",
                    help="differentiable calibration: 2,000 hulls, 5,000 steps, forward vs forward + adjoint")
    ap.add_argument("--settling", action="store_true",
                    help="the 125-cube settling scene (dt 1e-4, 2000 steps): the reference CPU path (oracle "
                         "restatement, one core) and the device step")
    ap.add_argument("--calib-steps", type=int, default=5000)
    ap.add_argument("--calib-particles", type=int, default=2000)
    ap.add_argument("--contact-point", default="midpoint", choices=["reference", "midpoint"],
                    help="calibration's torque-arm contact point: the reference's (cpA - cpB)/2 spins particles "
                         "far from the origin up until the 5,000-step pour flies apart, so the midpoint is the default")
    ap.add_argument("--batch-only", action="store_true",
                    help="only the 256-scene batched step with --lanes (no tuning, no sequential comparison)")
    ap.add_argument("--graph-steps", type=int, default=1, help="steps per captured graph (--batch-only)")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-total", type=int, default=2_000_000)
    ap.add_argument("--batch-seq-steps", type=int, default=3,
                    help="steps of the sequential per-scene baseline in the batched section")
    ap.add_argument("--no-extras", action="store_true",
                    help="leave out the batched, calibration and settling sections of the default run")
    return ap.parse_args()


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        # nvidia-smi numbers the GPUs of the machine; CUDA numbers the visible ones
        vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
        self.index = vis[index] if index < len(vis) else str(index)
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "20", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_scene(seed):
    from mwdiem_gb300 import scene
    p = dict(SCENE, seed=seed)
    return scene.pour_scene(**p)


def ref_kind(spec, V):
    """The reference path on the host: its kernels compiled from their own source when that build is
    available for this scene ('reference'), else the oracle's restatement ('port')."""
    import stepper
    try:
        return stepper.RefStepper(spec, V=V, kind="reference", nthreads=os.cpu_count() or 1), "reference"
    except Exception:
        return stepper.RefStepper(spec, V=V, kind="port", nthreads=1), "port"


def cpu_path_rate(spec, max_seconds=20.0, max_steps=5, one_core_steps=2):
    """Particle-steps/s of the reference path on the host (bounded sample: whole steps of the scene),
    on all host cores and, beside it, on one ("one_core": the reference's own serial loops)."""
    s, kind = ref_kind(spec, None)
    n = spec.n_particles
    with host_prints_to_stderr():
        s.step()  # warm-up (allocations, library load)
        t0 = time.perf_counter()
        steps = 0
        while steps < max_steps:
            s.step()
            steps += 1
            if time.perf_counter() - t0 > max_seconds:
                break
        dt = time.perf_counter() - t0
        one = None
        if kind == "reference" and one_core_steps > 0:
            s.nthreads = 1
            t1 = time.perf_counter()
            for _ in range(one_core_steps):
                s.step()
            one = {"value": n * one_core_steps / (time.perf_counter() - t1), "unit": METRIC, "cores": 1,
                   "kind": kind, "sample": f"{one_core_steps} more full steps, one thread"}
    cores = (os.cpu_count() or 1) if kind == "reference" else 1
    out = {"value": n * steps / dt, "unit": METRIC, "cores": cores, "kind": kind,
           "sample": f"{steps} full steps of the {n}-particle pour after 1 warm-up step"}
    if one is not None:
        out["one_core"] = one
    return out, s


def narrow_flops(sim):
    """Algorithmic FP32 operations of one narrow-phase launch on the current pair list, counted by
    the kernel itself (work counters on): 5 per vertex per support query (3 multiplies + 2 adds of
    the dot product) plus ~60 per EPA face built (cross product, normalisation, inside test)."""
    dots, faces, queries = sim.count_narrow_work()
    return 5.0 * dots + 60.0 * faces, dict(vertex_dots=dots, epa_faces=faces, support_queries=queries)


def lib_integrate_kernels(n):
    from mwdiem_gb300._lib import lib
    return int(lib().mwd_integrate_kernels(int(n)))


def integrate_bytes(sim):
    # per row: reads pos, dx_all (2 x 32 B), 14 float4 (224 B), info + vert_off (8 B);
    # writes pos, dx_all (64 B), 9 float4 state + 2 zeroed accumulators (176 B); per vertex 16 B in, 16 B out
    return sim.n * (64 + 224 + 8 + 64 + 176) + sim.state.n_verts * 32


class Window:
    """The pour is timed over its first WINDOW_STEPS steps (the configuration's length): the mutable
    state is restored to the initial state whenever a window ends."""

    def __init__(self, sim, length):
        self.sim = sim
        self.length = int(length)
        self.snap = {k: sim.t[k].clone() for k in sim.MUTABLE + ("force", "torque", "world_verts")}
        self.pos = 0

    def restore(self):
        for k, v in self.snap.items():
            self.sim.t[k].copy_(v)
        self.sim.w["status"].zero_()
        self.pos = 0

    def before_step(self):
        if self.pos >= self.length:
            self.restore()
        self.pos += 1


def main():
    args = parse()
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args)
    torch.cuda.set_device(local)
    if args.pairs_only:
        print(json.dumps({"narrow_pairs": pairs_rate(args.pairs, args.lanes, with_cpu=not args.no_cpu_baseline,
                                                     fixed=args.pairs_lanes)}), flush=True)
        return 0
    if args.batch_compare:
        print(json.dumps({"batch": batch_compare(args)}), flush=True)
        return 0
    if args.batch_only:
        print(json.dumps({"batch_only": batch_only(args)}), flush=True)
        return 0
    if args.calibration:
        print(json.dumps({"calibration": calibration(args)}), flush=True)
        return 0
    if args.settling:
        print(json.dumps({"settling": settling(args)}), flush=True)
        return 0
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from mwdiem_gb300 import _lib
    from mwdiem_gb300.sim import Simulator

    spec = build_scene(seed=SCENE["seed"] + rank)
    sim = Simulator(spec, lanes=args.lanes)
    V = sim.max_verts
    window = Window(sim, WINDOW_STEPS)
    from mwdiem_gb300 import autotune
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    # tuned the way the step is timed: each step after an L2 flush
    tuning = {} if args.no_tune else autotune.tune_lanes(sim, steps=6, flush=flush)
    sim.capture(steps_per_replay=1)
    window.restore()
    # clocks are sampled every 20 ms from the start of the warm-up (kept under the same load for at
    # least 0.5 s, so the sampler is running) to the end of the timed region
    clocks = ClockSampler(local)
    clocks.start()
    t_warm = time.perf_counter()
    done = 0
    while done < max(3, args.warmup) or time.perf_counter() - t_warm < 0.5:
        flush.zero_()
        window.before_step()
        sim.replay(1)
        done += 1
        if done % 20 == 0:
            torch.cuda.synchronize()
    torch.cuda.synchronize()
    window.restore()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.zero_()
        window.before_step()
        ev[i][0].record(stream)
        sim.replay(1)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    value, total_ms = job_rate(sum(a.elapsed_time(b) for a, b in ev), N_PARTICLES * args.steps, world, "cuda")
    status = sim.check_status()
    n_pairs = sim.n_pairs()
    nonfinite = sim.nonfinite_rows()

    # e2e: state from pinned host memory in, result back out, every step (from the initial state), one
    # captured graph per step: centres in, broad phase while the rest of the state comes in, narrow
    # phase, integrator, state out (Simulator.capture_host)
    window.restore()
    host = sim.host_state()
    nbytes = sim.host_state_bytes()
    ne = max(1, args.e2e_steps)

    def host_steps():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(ne):
            sim.step_host(host, 1)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    # for comparison: copy in, the step graph, copy out, one after another
    sim.step_host(host, 1)
    torch.cuda.synchronize()
    plain_value, _ = job_rate(host_steps(), N_PARTICLES * ne, world, "cuda")
    sim.capture_host(host)
    sim.step_host(host, 1)
    torch.cuda.synchronize()
    e2e_value, _ = job_rate(host_steps(), N_PARTICLES * ne, world, "cuda")
    # bytes back to the host per step: the whole state by a copy, or the rows the integrator updates
    # (the particles, 208 B each) when it writes them to the mapped host buffer itself
    back = N_PARTICLES * (nbytes // sim.n) if sim.host_graph_mirrored else nbytes
    e2e = {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": back,
           "state_back": "written to the mapped host buffer by the integrator's row pass" if sim.host_graph_mirrored
           else "copied after the integrator's row pass", "copies_around_step_graph": plain_value}

    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles": N_PARTICLES, "walls": spec.n_walls,
                       "candidate_pairs_per_step": n_pairs, "lanes_per_pair": autotune.describe(sim.lanes),
                       "block_size": autotune.block_size(sim.lanes),
                       "lanes_tuning_ms": {autotune.describe(k): v for k, v in tuning.items()}, "cuda_graph": True,
                       "l2": "flushed (256 MB write) before every timed step", "parallelism": f"replicas x{world}",
                       "window": f"steps 0..{WINDOW_STEPS - 1} of the pour from its initial state (the state is "
                                 f"restored every {WINDOW_STEPS} steps, outside the timed events)"},
            "e2e": e2e, "gpu_launches": KERNELS_PER_STEP * args.steps, "clocks": clk,
            "status": _lib.status_names(status), "nonfinite_rows": nonfinite,
            "steps_simulated": sim.steps_done}

    if rank == 0 and not args.no_breakdown:
        window.restore()
        line["breakdown"], line["roofline"] = breakdown(sim, V, flush)
    if rank == 0 and args.pairs > 0:
        del sim
        torch.cuda.empty_cache()
        line["narrow_pairs"] = pairs_rate(args.pairs, args.lanes)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cb, _ = cpu_path_rate(build_scene(SCENE["seed"]))
            line["cpu_baseline"] = cb
        except Exception as e:  # report, do not fail the GPU measurement
            line["cpu_baseline"] = {"error": str(e)[:200]}
    if rank == 0 and world == 1 and not args.no_extras:
        # the other configurations of the metric, each with its own clock record
        line["dropin"] = dropin_rate(line["ms_per_step"])
        for key, fn in (("batched", batch_compare), ("calibration", calibration), ("settling", settling)):
            torch.cuda.empty_cache()
            try:
                line[key] = fn(args)
            except Exception as e:  # report, do not fail the headline measurement
                line[key] = {"error": f"{type(e).__name__}: {str(e)[:300]}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def dropin_rate(device_ms_per_step, steps=3):
    """The pour through the reference's own per-step loop over the drop-in modules (mwdiem_gb300.dropin:
    host arrays, every module call copying its arguments in and out, the per-pair gather in numpy):
    what a user who only swaps the reference's imports runs.  Host wall clock per step (each step ends
    with the state back in host memory), after one warm-up step."""
    import torch
    from mwdiem_gb300.dropin import ReferenceLoop
    try:
        loop = ReferenceLoop(build_scene(SCENE["seed"]))
        loop.step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            loop.step()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / steps
    except Exception as e:  # report, do not fail the headline measurement
        return {"error": f"{type(e).__name__}: {str(e)[:300]}"}
    n = N_PARTICLES
    return {"value": n / (ms * 1e-3), "unit": METRIC, "ms_per_step": ms, "steps": steps,
            "candidate_pairs": int(len(loop.last_pairs)),
            "device_resident_over_dropin": ms / device_ms_per_step,
            "path": "cell keys + wall test + Linked_cell_hash (GPU, host arrays) -> per-pair gather (numpy) -> "
                    "Contact_detection_GPU -> Verlet_GPU, every call copying its numpy arguments in and out"}


def job_rate(local_ms, units_per_rank, world, device):
    """Whole-job throughput of `world` independent replicas (one per GPU, the same work each): the
    units all ranks processed over the slowest rank's time (max over ranks).  Returns (units/s, ms)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    return units_per_rank * world / (ms * 1e-3), ms


def breakdown(sim, V, flush, reps=10):
    """Per-stage device time (CUDA events on the launching stream, L2 flushed before each stage's
    step) and the roofline of the dominant stage."""
    import torch
    from mwdiem_gb300 import _lib
    stream = torch.cuda.current_stream()
    acc = {"broad": 0.0, "narrow": 0.0, "integrate": 0.0}
    for _ in range(reps):
        flush.zero_()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        evs[0].record(stream)
        sim.broadphase()
        evs[1].record(stream)
        sim.narrow_force()
        evs[2].record(stream)
        sim.integrate()
        evs[3].record(stream)
        torch.cuda.synchronize()
        acc["broad"] += evs[0].elapsed_time(evs[1])
        acc["narrow"] += evs[1].elapsed_time(evs[2])
        acc["integrate"] += evs[2].elapsed_time(evs[3])
    ms = {k: v / reps for k, v in acc.items()}
    pk = peaks()
    import ctypes as C
    scratch = torch.zeros(8 * 1024, dtype=torch.float32, device="cuda")
    tf = C.c_double(0)
    _lib.check(_lib.lib().mwd_probe_fp32(20000, scratch.data_ptr(), C.byref(tf), None))
    fp32_peak = tf.value
    flops, work = narrow_flops(sim)
    ib = integrate_bytes(sim)
    out = {"ms": ms, "n_pairs": sim.n_pairs(), "narrow_fp32_tflops": flops / (ms["narrow"] * 1e-3) / 1e12,
           "narrow_fp32_peak_tflops_measured": fp32_peak,
           "integrate_gbs": ib / (ms["integrate"] * 1e-3) / 1e9, "narrow_work": work}
    dom = max(ms, key=ms.get)
    if dom == "narrow":
        a = flops / (ms["narrow"] * 1e-3) / 1e12
        roof = {"kernel": "gjk_pass_kernel + epa_pass_kernel", "bound": "fp32", "achieved": a, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": a / fp32_peak if fp32_peak else None,
                "traffic": NARROW_DRAM_BYTES_PER_LAUNCH,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch of each pass of the "
                                  "eager first step (not measured in this run)",
                "note": "latency-bound: ~13k candidate pairs, each a chain of dependent support queries; the "
                        "GJK pass issues on ~40% of cycles, the EPA pass waits on its few longest pairs",
                "peak_source": "measured in this run (mwd_probe_fp32: FMUL+FADD chains, no FMA)"}
    elif dom == "integrate":
        hbm = pk.get("hbm_gbs", 6800.0)
        a = ib / (ms["integrate"] * 1e-3) / 1e9
        roof = {"kernel": "integrate_kernel", "bound": "hbm", "achieved": a, "peak": hbm, "unit": "GB/s",
                "frac": a / hbm, "traffic": None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in pk else "fallback 6800"}
    else:
        hbm = pk.get("hbm_gbs", 6800.0)
        n, P = sim.n, sim.n_pairs()
        bbytes = n * (32 + 4 + 4 + 4 + 4 + 4 + 8) + sim.total_cells * 12 + P * (8 + 8 + 8)
        a = bbytes / (ms["broad"] * 1e-3) / 1e9
        roof = {"kernel": "broad phase (4 kernels)", "bound": "hbm", "achieved": a, "peak": hbm, "unit": "GB/s",
                "frac": a / hbm, "traffic": None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in pk else "fallback 6800"}
    return out, roof


def pairs_cpu_rate(ps, n_pairs, sample=30_000, max_seconds=20.0):
    """Pairs/s of the reference's contact kernel on the host (its own source compiled for the host,
    all cores; else the oracle's restatement, one core) on a random sample of the same pairs.  The
    reference's EPA writes past its 50-face arrays on some deep overlaps (its host build then
    crashes), so the sample keeps the pairs the oracle finishes within 50 faces."""
    import numpy as np
    import oracle
    k = min(n_pairs, sample)
    idx = np.sort(np.random.default_rng(0).choice(n_pairs, size=k, replace=False))
    inp = ps.gather(idx)
    inp["A_id"] = (2 * np.arange(k)).astype(np.int32)
    inp["B_id"] = (2 * np.arange(k) + 1).astype(np.int32)
    params = dict(ps.params, num_particles_wall=0)
    # the pairs whose EPA stays within the reference's 50 faces (oracle with that capacity, clean status)
    ok = np.nonzero(oracle.contact(inp, params, 2 * k, "f32", face_cap=50)["status"] == 0)[0]
    inp = {kk: np.ascontiguousarray(v[ok]) for kk, v in inp.items()}
    inp["A_id"] = (2 * np.arange(len(ok))).astype(np.int32)
    inp["B_id"] = (2 * np.arange(len(ok)) + 1).astype(np.int32)
    dropped = k - len(ok)
    k = len(ok)
    kind, cores = "reference", os.cpu_count() or 1
    try:
        ref = oracle.RefContact(params, "f32")
        run = lambda d: ref.run(d, 2 * k, nthreads=cores)  # noqa: E731
        run({kk: v[:64] for kk, v in inp.items()})
    except Exception:
        kind, cores = "port", 1
        run = lambda d: oracle.contact(d, params, 2 * k, "f32")  # noqa: E731
    with host_prints_to_stderr():
        done, t0 = 0, time.perf_counter()
        for a in range(0, k, 10_000):
            run({kk: v[a:a + 10_000] for kk, v in inp.items()})
            done += min(10_000, k - a)
            if time.perf_counter() - t0 > max_seconds:
                break
        dt = time.perf_counter() - t0
        one = None
        if kind == "reference":
            # the same kernel on one thread, the first 5,000 pairs of the sample
            k1 = min(k, 5_000)
            t1 = time.perf_counter()
            ref.run({kk: v[:k1] for kk, v in inp.items()}, 2 * k, nthreads=1)
            one = {"value": k1 / (time.perf_counter() - t1), "unit": "pairs/s", "cores": 1, "kind": kind,
                   "sample": f"the first {k1} pairs of the sample, one thread"}
    out = {"value": done / dt, "unit": "pairs/s", "cores": cores, "kind": kind,
           "sample": f"{done} of the {n_pairs} pairs (random, same seed; {dropped} pairs whose EPA overruns the "
                     f"reference's 50 faces or stops at its iteration cap left out), in chunks of 10,000"}
    if one is not None:
        out["one_core"] = one
    return out


def lanes_arg(text):
    return parse_lanes(text) if "/" in str(text) else int(text)


def parse_lanes(text):
    """'gjk1/epa16g' or 'gjk1/epa16g/b64x256' -> the lanes word (GJK lanes | EPA lanes << 8 | hulls
    read in place << 16 | block-size codes of the GJK and EPA passes << 20, << 22)."""
    import re
    m = re.fullmatch(r"gjk(\d+)/epa(\d+)(g?)(?:/b(\d+)x(\d+))?", text)
    if not m:
        raise SystemExit(f"bad lanes setting {text!r}; expected e.g. gjk1/epa16g or gjk1/epa16g/b64x128")
    w = int(m.group(1)) | (int(m.group(2)) << 8) | ((1 << 16) if m.group(3) else 0)
    if m.group(4):
        code = {128: 0, 64: 1, 256: 2}
        try:
            w |= (code[int(m.group(4))] << 20) | (code[int(m.group(5))] << 22)
        except KeyError:
            raise SystemExit(f"bad block sizes in {text!r}; each is 64, 128 or 256")
    return w


def pairs_rate(n_pairs, lanes, reps=5, with_cpu=True, fixed=None):
    """GJK/EPA pairs/s of the device-step narrow phase on independent random pairs (hulls of 8-64
    vertices, radius U[0.8,1.2], centre distance U[0.5,2.2] (rA+rB)/2; inputs ~10 GB, far above L2)."""
    import ctypes as C

    import torch
    from mwdiem_gb300 import _lib
    from mwdiem_gb300.pairbench import PairScene
    from mwdiem_gb300 import autotune
    ps = PairScene(n_pairs, seed=1, lanes=lanes)
    stream = torch.cuda.current_stream()
    sweep = {}
    cands = tuple(parse_lanes(t) for t in ("gjk8/epa8", "gjk8/epa16", "gjk4/epa16", "gjk4/epa16g", "gjk4/epa8g",
                                           "gjk8/epa16g", "gjk1/epa16", "gjk1/epa16g", "gjk1/epa8g", "gjk1/epa32g"))
    if fixed is not None:
        cands = (parse_lanes(fixed),)
    for cand in cands:
        ps.lanes = cand
        ps.narrow()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            ps.narrow()
        e1.record(stream)
        torch.cuda.synchronize()
        sweep[autotune.describe(cand)] = e0.elapsed_time(e1) / reps
    if fixed is None:
        # block sizes of the two passes at the fastest lane setting
        top = min(sweep, key=sweep.get)
        top_word = [c for c in cands if autotune.describe(c) == top][0]
        extra = tuple(c for c in autotune.block_candidates(top_word) if c not in cands)
        cands = cands + extra
        for cand in extra:
            ps.lanes = cand
            ps.narrow()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                ps.narrow()
            e1.record(stream)
            torch.cuda.synchronize()
            sweep[autotune.describe(cand)] = e0.elapsed_time(e1) / reps
    best = min(sweep, key=sweep.get)
    ms = sweep[best]
    ps.lanes = [c for c in cands if autotune.describe(c) == best][0]
    ps.narrow(count_work=True)
    torch.cuda.synchronize()
    dots, faces, queries = (int(x) for x in ps.w["counters"].cpu().numpy())
    coll = ps.w["collision"].cpu().numpy()
    flops = 5.0 * dots + 60.0 * faces
    scratch = torch.zeros(8 * 1024, dtype=torch.float32, device="cuda")
    tf = C.c_double(0)
    _lib.check(_lib.lib().mwd_probe_fp32(20000, scratch.data_ptr(), C.byref(tf), None))
    ach = flops / (ms * 1e-3) / 1e12
    cpu = pairs_cpu_rate(ps, n_pairs) if with_cpu else None
    return {"pairs": n_pairs, "ms_per_launch": ms, "pairs_per_s": n_pairs / (ms * 1e-3), "cpu_baseline": cpu,
            "contact_fraction": float((coll == 1).mean()), "support_queries": queries, "vertex_dots": dots,
            "epa_faces": faces, "lanes_per_pair": best, "block_size": autotune.block_size(ps.lanes),
            "lanes_sweep_ms": sweep, "two_pass": True,
            "roofline": {"kernel": "gjk_pass + epa_pass", "bound": "fp32", "achieved": ach, "peak": tf.value,
                         "unit": "TFLOP/s", "frac": ach / tf.value if tf.value else None,
                         "peak_source": "measured in this run (mwd_probe_fp32)"}}


def batch_compare(args):
    """Batched scenes: 256 independent boxes with log-uniform particle counts in 100..50,000 (~2M in
    all; cubes, tetrahedra and hulls), dt 5e-5.  Batched = all scenes in one state, one launch per
    stage, the step captured in CUDA graphs, lanes chosen by the autotuner.  Sequential = one
    simulator per scene, stepped one after another with plain launches (the same kernels), timed over
    --batch-seq-steps steps.  Contact sets: the batch's candidate list scene by scene equals each
    scene's own simulator's, and, for a sample of scenes, the reference path's (the cpu_baseline leg,
    which also times that path on those scenes)."""
    import torch
    from mwdiem_gb300 import autotune, scene
    from mwdiem_gb300.sim import Simulator
    t0 = time.perf_counter()
    specs = scene.batched_scenes(n_scenes=args.batch_scenes, total=args.batch_total, seed=0)
    n_total = sum(sp.n_particles for sp in specs)
    batch = Simulator(specs, lanes=args.lanes)
    singles = [Simulator(sp, lanes=args.lanes) for sp in specs]
    build_s = time.perf_counter() - t0
    # identical contact sets, scene by scene, at the initial state (bounding-sphere filter on)
    batch.broadphase()
    bp = batch.pairs().cpu().numpy()
    same = True
    for i, one in enumerate(singles):
        one.broadphase()
        p1 = one.pairs().cpu().numpy()
        r0, r1 = batch.layout.row_begin[i], batch.layout.row_end[i]
        mine = bp[(bp[:, 0] >= r0) & (bp[:, 0] < r1)] - r0
        if set(map(tuple, mine.tolist())) != set(map(tuple, p1.tolist())):
            same = False
    # the full candidate list (filter off), compared with the reference path's on a sample of scenes
    batch.work.cull_pairs = 0
    batch.broadphase()
    full = batch.pairs().cpu().numpy()
    batch.work.cull_pairs = 1
    cpu = batch_cpu_baseline(specs, batch.layout, full)
    torch.cuda.synchronize()
    tune = autotune.tune_lanes(batch, steps=3)
    K = max(1, args.steps)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    # one step per graph, then ten: inside a ten-step graph each step's world-vertex pass runs beside
    # the next step's broad phase (mwd_step's overlap); the arrays (~1.5 GB) are far larger than L2
    ms_batch_1 = autotune.time_steps(batch, steps=K, reps=3)
    ms_batch = autotune.time_steps(batch, steps=max(K, 10), reps=3, per=10)
    stream = torch.cuda.current_stream()
    for one in singles:
        one.lanes = batch.lanes
        one.step(1)
    torch.cuda.synchronize()
    Ks = max(1, args.batch_seq_steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(Ks):
        for one in singles:
            one.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_seq = e0.elapsed_time(e1) / Ks
    clk = clocks.stop()
    stages = batch_stages(batch)
    from mwdiem_gb300._lib import status_names
    return {"workload": "256 boxes, particle counts log-uniform in 100..50,000 (~2M), shapes 1/3 each cube, regular "
                        "tetrahedron, hull of 12-32 points; kn 1e5, damping ratio 0.3, mu 0.5, dt 5e-5",
            "scenes": len(specs), "particles": int(n_total),
            "counts_min_max": [int(min(sp.n_particles for sp in specs)), int(max(sp.n_particles for sp in specs))],
            "build_s": build_s, "lanes_tuning_ms": {autotune.describe(k): v for k, v in tune.items()},
            "lanes": autotune.describe(batch.lanes), "block_size": autotune.block_size(batch.lanes),
            "ms_per_step_batched": ms_batch, "graph_steps_batched": 10,
            "steps_timed_batched": 3 * max(K, 10), "ms_per_step_batched_graph1": ms_batch_1,
            "ms_per_step_sequential": ms_seq, "steps_timed_sequential": Ks,
            "particle_steps_per_s_batched": n_total / (ms_batch * 1e-3),
            "particle_steps_per_s_sequential": n_total / (ms_seq * 1e-3),
            "batched_over_sequential": ms_seq / ms_batch, "identical_contact_sets": same,
            "identical_contact_sets_vs_reference": cpu.get("identical_contact_sets"),
            "status": status_names(batch.status()), "pairs_batched": int(len(bp)), "candidates_unfiltered": int(len(full)),
            "stages": stages, "clocks": clk, "cpu_baseline": cpu}


def batch_cpu_baseline(specs, layout, full, n_sample=8, max_seconds=15.0):
    """The reference path (oracle/stepper.py, its own kernels built for the host where available) on a
    sample of the batch's scenes -- the largest and seven drawn at random -- one step each from the
    initial state: its candidate sets must equal the batch's scene by scene, and its particle-steps/s
    over the sample is the CPU baseline of this configuration."""
    import oracle_sets
    order = oracle_sets.batch_sample(specs, n_sample)
    same, done, parts, t_cpu, kind = True, [], 0, 0.0, None
    with host_prints_to_stderr():
        for i in order:
            s, kind = ref_kind(specs[i], None)
            t0 = time.perf_counter()
            s.step()
            t_cpu += time.perf_counter() - t0
            r0, r1 = layout.row_begin[i], layout.row_end[i]
            mine = full[(full[:, 0] >= r0) & (full[:, 0] < r1)] - r0
            if len(mine) != len(s.last_pairs) or \
                    set(map(tuple, mine.tolist())) != set(map(tuple, s.last_pairs.tolist())):
                same = False
            done.append(i)
            parts += specs[i].n_particles
            if t_cpu > max_seconds:
                break
    cores = (os.cpu_count() or 1) if kind == "reference" else 1
    return {"value": parts / t_cpu, "unit": METRIC, "cores": cores, "kind": kind, "identical_contact_sets": same,
            "sample": f"one step from the initial state of each of scenes {done} ({parts} particles)"}


def batch_stages(sim, reps=5):
    """Per-stage device time of the batched step (CUDA events around each stage's launches; its
    arrays, ~1.5 GB, are far larger than L2) and the HBM roofline of the integrator, the stage whose
    traffic is fixed by the algorithm: per row 536 B (state read and written), per vertex 32 B (body
    vertex in, world vertex out)."""
    import torch
    stream = torch.cuda.current_stream()
    acc = {"broad": 0.0, "narrow": 0.0, "integrate": 0.0}
    for _ in range(reps):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        evs[0].record(stream)
        sim.broadphase()
        evs[1].record(stream)
        sim.narrow_force()
        evs[2].record(stream)
        sim.integrate()
        evs[3].record(stream)
        torch.cuda.synchronize()
        for k, (a, b) in zip(acc, ((0, 1), (1, 2), (2, 3))):
            acc[k] += evs[a].elapsed_time(evs[b])
    ms = {k: v / reps for k, v in acc.items()}
    hbm = peaks().get("hbm_gbs", 6800.0)
    ib = integrate_bytes(sim)
    a = ib / (ms["integrate"] * 1e-3) / 1e9
    one = lib_integrate_kernels(sim.n) == 1
    return {"ms": ms, "integrate_roofline": {"kernel": "integrate_kernel" if one else "integrate_rows_kernel + world_verts_kernel", "bound": "hbm",
                                            "bytes_per_step": ib, "achieved": a, "peak": hbm, "unit": "GB/s",
                                            "frac": a / hbm}}


def settling(args, steps=2000, cpu_seconds=15.0):
    """The settling scene: 125 randomly rotated unit cubes on a 5^3 lattice (spacing 1.5) onto a floor,
    dt 1e-4, 2000 steps.  The reference CPU path (wall test + Linked_cell_hash + per-pair gather +
    contact kernel FP32 + Verlet kernel FP64, as the oracle restates them) is timed on one host core
    for the whole run or ~20 s, whichever ends first; the device step (graph replay) runs all 2000
    steps."""
    import torch
    import stepper
    from mwdiem_gb300 import scene
    from mwdiem_gb300.sim import Simulator
    spec = scene.settling_scene()
    n = spec.n_particles
    out = {"workload": "settling125: 125 unit cubes (density 1), 5x5x5 lattice at spacing 1.5, jitter 0.1, "
                       "random orientations, floor 10x10, kn 1e5, damping ratio 0.3, mu 0.5, dt 1e-4",
           "particles": n, "steps": steps}
    # The reference's own contact kernel (built for the host) is not run here: once the cubes' contacts
    # need more than 50 EPA faces it writes past its T[50]/V[50] arrays (gpu_fine_contact_detection.cu:
    # 359-362, 519-539), which crashed the process on the Arm host.  The oracle's restatement computes
    # the same results with bounded arrays, on one core.
    s = stepper.RefStepper(spec, kind="port")
    t0 = time.perf_counter()
    done = 0
    while done < steps and time.perf_counter() - t0 < cpu_seconds:
        s.step()
        done += 1
    dt = time.perf_counter() - t0
    out["cpu_1core"] = {"value": n * done / dt, "unit": METRIC, "cores": 1, "kind": "port",
                        "sample": f"the first {done} of the {steps} steps"}
    sim = Simulator(spec)
    window = Window(sim, steps)
    per = 20  # steps per captured graph
    sim.capture(steps_per_replay=per)
    sim.replay(3)  # warm-up
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    reps, times = 5, []
    for _ in range(reps):
        window.restore()  # the run from its initial state, outside the timed events
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.replay(steps // per)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    ms = sorted(times)[reps // 2]
    out["gpu"] = {"value": n * steps / (ms * 1e-3), "unit": METRIC, "ms_per_step": ms / steps,
                  "dtype": "f32 state, f64 centres", "graph_steps": per, "status": sim.status(),
                  "sample": f"the {steps} steps from the initial state, median of {reps} runs", "clocks": clk}
    return out


def batch_only(args):
    """The 256-scene batched step alone: all scenes in one state, the step captured in one CUDA graph,
    --lanes fixed, --warmup then --steps replays timed with CUDA events."""
    import torch
    from mwdiem_gb300 import scene
    from mwdiem_gb300.sim import Simulator
    specs = scene.batched_scenes(n_scenes=args.batch_scenes, total=args.batch_total, seed=0)
    n_total = sum(sp.n_particles for sp in specs)
    sim = Simulator(specs, lanes=args.lanes)
    per = max(1, args.graph_steps)
    n = max(1, -(-max(1, args.steps) // per))
    sim.capture(per)
    sim.replay(max(1, -(-args.warmup // per)))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.replay(n)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / (n * per)
    return {"scenes": len(specs), "particles": int(n_total), "lanes": args.lanes, "graph_steps": per, "ms_per_step": ms,
            "particle_steps_per_s": n_total / (ms * 1e-3), "status": sim.status()}


def calibration(args):
    """Calibration: 2,000 random hulls (12-32 points, radius U[0.8,1.2]) poured in a 20 x 20 box, 5,000
    steps at dt 5e-5.  Loss = MSE of the per-step centre of mass against a target trajectory of the
    same simulator with kn 2e5, damping ratio 0.2, mu 0.4; gradients with respect to kn, damping
    ratio, mu and the initial velocities, checkpoints every 100 steps.  Times the differentiable
    forward alone and forward + adjoint (CUDA events, same stream), and the plain FP32 step of the
    same scene; the FP64 finite-difference check runs at 16 particles x 50 steps."""
    import numpy as np
    import torch
    from mwdiem_gb300 import scene
    from mwdiem_gb300.diff import DiffEngine, law_from, rollout
    from mwdiem_gb300.sim import Simulator
    n, steps = args.calib_particles, args.calib_steps
    spec = scene.pour_scene(n=n, box=20.0, seed=0)
    eng = DiffEngine(spec, steps, ckpt_every=100, contact_point=args.contact_point)
    dev = eng.device
    W = eng.n_walls
    x0 = eng.initial_state()
    target, _ = eng.forward(x0, law_from(2e5, 0.2, 0.4).to(dev), steps)
    st_target = eng.status_word()
    stream = torch.cuda.current_stream()

    def run(backward):
        kn = torch.tensor(1e5, dtype=torch.float64, device=dev, requires_grad=True)
        zeta = torch.tensor(0.3, dtype=torch.float64, device=dev, requires_grad=True)
        mu = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
        v0 = torch.zeros((n, 3), dtype=torch.float64, device=dev, requires_grad=True)
        x = torch.cat([x0[:W], torch.cat([x0[W:, :3], v0, v0, x0[W:, 9:]], 1)], 0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        if backward:
            com, _ = rollout(eng, x, law_from(kn, zeta, mu).to(dev), steps)
            loss = ((com - target) ** 2).mean()
            loss.backward()
        else:
            with torch.no_grad():
                com, _ = rollout(eng, x, law_from(kn, zeta, mu).to(dev), steps)
                loss = ((com - target) ** 2).mean()
        e1.record(stream)
        torch.cuda.synchronize()
        g = None
        if backward:
            g = {"kn": float(kn.grad), "damping": float(zeta.grad), "mu": float(mu.grad),
                 "v0_norm": float(v0.grad.norm()), "finite": bool(torch.isfinite(v0.grad).all())}
        return e0.elapsed_time(e1), float(loss), g

    run(False)  # warm-up: graph capture
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    fwd = sorted(run(False)[0] for _ in range(3))[1]
    fb = []
    for _ in range(3):
        ms, loss, grads = run(True)
        fb.append(ms)
    clk = clocks.stop()
    fwd_bwd = sorted(fb)[1]
    contacts = int(eng.step_off[steps].item())
    st = eng.status_word()
    # the plain device step of the same scene (FP32 state, CUDA graph)
    sim = Simulator(spec)
    sim.capture(1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.replay(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    from mwdiem_gb300._lib import status_names
    return {"workload": "2,000 hulls of 12-32 points (radius U[0.8,1.2]) poured into a 20x20 box, 5,000 steps at "
                        "dt 5e-5; loss = MSE of the per-step centre of mass against the trajectory with kn 2e5, "
                        "damping ratio 0.2, mu 0.4; gradients w.r.t. kn, damping ratio, mu, initial velocities",
            "particles": n, "steps": steps, "checkpoint_every": 100, "contact_point": args.contact_point,
            "contacts_logged": contacts, "ms_forward": fwd, "ms_forward_adjoint": fwd_bwd,
            "adjoint_over_forward": fwd_bwd / fwd, "ms_plain_fp32_steps": plain_ms,
            "forward_over_plain": fwd / plain_ms, "loss": loss, "grads": grads,
            "status": status_names(st), "status_target": status_names(st_target), "clocks": clk,
            "timing": "median of 3 runs each (CUDA events on the launching stream) after one warm-up run",
            "fd_check_16x50": fd_check()}


def fd_check(steps=50):
    """Relative difference between the adjoint gradient and FP64 central differences (h = 1e-6
    relative) of the whole forward, 16 packed hulls x 50 steps, for kn, damping, mu and a random
    direction of the initial velocities."""
    import numpy as np
    import torch
    from mwdiem_gb300 import scene
    from mwdiem_gb300.diff import DiffEngine, law_from, rollout
    eng = DiffEngine(scene.packed_scene(16, seed=3), steps, ckpt_every=10)
    dev = eng.device
    W = eng.n_walls
    x0 = eng.initial_state()
    target, _ = eng.forward(x0, law_from(2e5, 0.2, 0.4).to(dev), steps)
    base = {"kn": 1e5, "zeta": 0.3, "mu": 0.5}
    v0 = x0[W:, 3:6].clone()
    d = torch.from_numpy(np.random.default_rng(7).normal(size=tuple(v0.shape))).to(dev)

    def loss(p, v):
        x = torch.cat([x0[:W], torch.cat([x0[W:, :3], v, v, x0[W:, 9:]], 1)], 0)
        com, _ = rollout(eng, x, law_from(p["kn"], p["zeta"], p["mu"]).to(dev), steps)
        return ((com - target) ** 2).mean()

    P = {k: torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=True) for k, v in base.items()}
    vv = v0.clone().requires_grad_(True)
    loss(P, vv).backward()
    an = {k: float(t.grad) for k, t in P.items()}
    an["v0"] = float((vv.grad * d).sum())
    out = {}
    with torch.no_grad():
        for k in ("kn", "zeta", "mu", "v0"):
            h = 1e-6 * (base[k] if k != "v0" else 1.0)
            vals = []
            for sgn in (1, -1):
                p = dict(base)
                v = v0
                if k == "v0":
                    v = v0 + sgn * h * d
                else:
                    p[k] = base[k] + sgn * h
                vals.append(float(loss(p, v)))
            fd = (vals[0] - vals[1]) / (2 * h)
            out[k] = {"adjoint": an[k], "fd": fd, "rel_err": abs(an[k] - fd) / abs(fd)}
    return out


def reference_arm(args):
    """The reference's CPU path on this host, same scene, same metric."""
    spec = build_scene(SCENE["seed"])
    s, kind = ref_kind(spec, None)
    cores = (os.cpu_count() or 1) if kind == "reference" else 1
    with host_prints_to_stderr():
        for _ in range(max(0, args.warmup)):
            s.step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.step()
        dt = time.perf_counter() - t0
    value = spec.n_particles * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles": spec.n_particles, "walls": spec.n_walls,
                       "path": "wall test + cell keys + Linked_cell_hash (C restatement) -> per-pair gather -> "
                               "contact kernel (FP32) -> Verlet kernel (FP64)"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": kind,
                             "sample": f"{args.steps} full steps of the {spec.n_particles}-particle pour"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
