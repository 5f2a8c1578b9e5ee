"""The reference path's inlet (oracle/stepper.py, MWDiem.py:685-714) on the CPU: rows wait outside
the broad phase and the integrator and enter per_spawn at a time every period steps, at rest at
their spawn points; the candidate pairs never name a waiting row."""
import numpy as np

import stepper
from mwdiem_gb300 import scene


def test_inlet_schedule_of_the_reference_path():
    sp = scene.pour_scene(n=40, seed=2, box=10.0, spacing=2.3, pool=8)
    W = sp.n_walls
    N = W + sp.n_particles
    spawn = np.zeros((N, 3))
    spawn[W + 30:] = np.random.default_rng(0).uniform([-3, -3, 20], [3, 3, 22], size=(10, 3))
    ref = stepper.RefStepper(sp, inlet=(4, 3, W + 30, spawn))
    start = ref.st["com"].copy()
    for step in range(10):
        ref.step()
        entered = min(3 * (step // 4 + 1), 10)
        assert ref.active_end == W + 30 + entered
        waiting = np.arange(ref.active_end, N)
        assert not np.isin(ref.last_pairs, waiting).any()
        assert np.array_equal(ref.st["com"][waiting], start[waiting])      # untouched while waiting
    new = np.arange(W + 30, ref.active_end)
    # entered at rest at their spawn points, then fell for a few steps under gravity
    assert np.all(np.abs(ref.st["com"][new] - spawn[new]) < 1e-3)
    assert np.all(ref.st["v"][new, 2] <= 0.0)
