"""Autotuner for the device-resident step.

Chooses the lanes per pair of the narrow phase's GJK pass (1, 4, 8 or 16) and EPA pass (8, 16 or 32),
whether the EPA pass stages the two hulls in shared memory or reads them in place, and then the
threads per block of each of the two passes (64, 128 or 256), by timing graph-captured steps of the
actual scene and keeping the fastest.  The cell size is not a tuning knob: it decides the
reference's candidate set (an 8-cell forward stencil misses some neighbour pairs, and which ones
depends on the cell size), so it stays what the scene defines (MWDiem.py:575-580).  The reference
hard-codes its launch geometry (gpu_fine_contact_detection.py:28-29, gpu_Verlet.py:26-27).
"""
from __future__ import annotations

import copy

import torch


def time_steps(sim, steps=5, reps=3, per=1, flush=None):
    """Median ms per graph-replayed step (after one captured warm-up step); `per` steps per graph
    (rounded up to whole graphs).  With `flush` (a tensor larger than L2), each graph replay is timed
    on its own after the tensor is overwritten, outside the timed events: the regime of a step whose
    state is not in L2."""
    sim.capture(per)
    n = max(1, -(-steps // per))
    stream = torch.cuda.current_stream()
    best = []
    for _ in range(reps):
        if flush is None:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim.replay(n)
            e1.record(stream)
            torch.cuda.synchronize()
            best.append(e0.elapsed_time(e1) / (n * per))
            continue
        evs = []
        for _ in range(n):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim.replay(1)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        best.append(sum(a.elapsed_time(b) for a, b in evs) / (n * per))
    best.sort()
    return best[len(best) // 2]


# lanes word: GJK-pass lanes | EPA-pass lanes << 8 | EPA hulls read in place (no staging) << 16 |
# block-size codes of the two passes << 20 and << 22 (0: 128 threads, 1: 64, 2: 256)
EPA_IN_PLACE = 1 << 16
GJK_BLOCK_SHIFT = 20
EPA_BLOCK_SHIFT = 22
BLOCK_THREADS = {0: 128, 1: 64, 2: 256}
DEFAULT_CANDIDATES = tuple(g | (e << 8) | f for g in (1, 4, 8, 16) for e in (8, 16, 32) for f in (0, EPA_IN_PLACE))


def block_size(lanes):
    """Threads per block of the GJK and EPA passes under a lanes word."""
    return {"gjk": BLOCK_THREADS[(lanes >> GJK_BLOCK_SHIFT) & 3], "epa": BLOCK_THREADS[(lanes >> EPA_BLOCK_SHIFT) & 3]}


def with_blocks(lanes, gjk_code, epa_code):
    mask = (3 << GJK_BLOCK_SHIFT) | (3 << EPA_BLOCK_SHIFT)
    return (lanes & ~mask) | (gjk_code << GJK_BLOCK_SHIFT) | (epa_code << EPA_BLOCK_SHIFT)


def block_candidates(lanes):
    return tuple(with_blocks(lanes, g, e) for g in (0, 1, 2) for e in (0, 1, 2))


def describe(lanes):
    s = f"gjk{lanes & 0xff}/epa{((lanes >> 8) & 0xff) or (lanes & 0xff)}"
    s += "g" if lanes & EPA_IN_PLACE else ""
    b = block_size(lanes)
    if b != {"gjk": 128, "epa": 128}:
        s += f"/b{b['gjk']}x{b['epa']}"
    return s


def tune_lanes(sim, candidates=DEFAULT_CANDIDATES, steps=5, blocks=True, flush=None):
    """Time the scene with each lanes-per-pair setting (GJK-pass lanes | EPA-pass lanes << 8) on a
    copy of its state, then the block sizes of the two passes at the fastest setting; set the fastest
    on `sim`, and return {setting: ms per step}.  The state of `sim` is restored afterwards.  `flush`:
    time every step with L2 overwritten first (time_steps)."""
    saved = {k: v.clone() for k, v in sim.t.items()}
    res = {}

    def run(lanes):
        sim.lanes = int(lanes)
        sim.graph = None
        res[lanes] = time_steps(sim, steps, flush=flush)
        for k, v in saved.items():
            sim.t[k].copy_(v)

    for lanes in candidates:
        run(lanes)
    if blocks:
        best = min(res, key=res.get)
        for lanes in block_candidates(best):
            if lanes not in res:
                run(lanes)
    best = min(res, key=res.get)
    sim.lanes = int(best)
    sim.graph = None
    for k, v in saved.items():
        sim.t[k].copy_(v)
    sim.w["status"].zero_()
    torch.cuda.synchronize()
    return res
