"""Autotuner for the device-resident step.

Chooses the lanes per pair of the narrow phase's GJK pass (1, 4, 8 or 16) and EPA pass (8, 16 or 32)
and whether the EPA pass stages the two hulls in shared memory or reads them in place, by timing graph-captured steps of the actual scene and keeping
the fastest.  The
cell size is not a tuning knob: it decides the reference's candidate set (an 8-cell forward stencil
misses some neighbour pairs, and which ones depends on the cell size), so it stays what the scene
defines (MWDiem.py:575-580).
"""
from __future__ import annotations

import copy

import torch


def time_steps(sim, steps=5, reps=3, per=1):
    """Median ms per graph-replayed step (after one captured warm-up step); `per` steps per graph
    (rounded up to whole graphs)."""
    sim.capture(per)
    n = max(1, -(-steps // per))
    stream = torch.cuda.current_stream()
    best = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.replay(n)
        e1.record(stream)
        torch.cuda.synchronize()
        best.append(e0.elapsed_time(e1) / (n * per))
    best.sort()
    return best[len(best) // 2]


# lanes word: GJK-pass lanes | EPA-pass lanes << 8 | EPA hulls read in place (no staging) << 16
EPA_IN_PLACE = 1 << 16
DEFAULT_CANDIDATES = tuple(g | (e << 8) | f for g in (1, 4, 8, 16) for e in (8, 16, 32) for f in (0, EPA_IN_PLACE))


def describe(lanes):
    s = f"gjk{lanes & 0xff}/epa{((lanes >> 8) & 0xff) or (lanes & 0xff)}"
    return s + ("g" if lanes & EPA_IN_PLACE else "")


def tune_lanes(sim, candidates=DEFAULT_CANDIDATES, steps=5):
    """Time the scene with each lanes-per-pair setting (GJK-pass lanes | EPA-pass lanes << 8) on a
    copy of its state, set the fastest on `sim`, and return {setting: ms per step}.  The state of
    `sim` is restored afterwards."""
    saved = {k: v.clone() for k, v in sim.t.items()}
    res = {}
    for lanes in candidates:
        sim.lanes = int(lanes)
        sim.graph = None
        res[lanes] = time_steps(sim, steps)
        for k, v in saved.items():
            sim.t[k].copy_(v)
    best = min(res, key=res.get)
    sim.lanes = int(best)
    sim.graph = None
    for k, v in saved.items():
        sim.t[k].copy_(v)
    sim.w["status"].zero_()
    torch.cuda.synchronize()
    return res
