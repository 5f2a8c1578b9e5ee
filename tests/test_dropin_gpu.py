"""The reference's per-step loop run over the drop-in modules (mwdiem_gb300/dropin.py: host arrays,
every module copying its arguments in and out) against the reference path of oracle/stepper.py
(the same loop over the oracle's kernels): the same candidate pairs every step, the same contact
flags, and states within the short-horizon bars after 10 steps."""
import numpy as np
import pytest

import stepper
from mwdiem_gb300 import scene

pytestmark = pytest.mark.gpu


def oriented(p):
    return set(map(tuple, np.asarray(p).reshape(-1, 2).tolist()))


def test_reference_loop_over_dropins_matches_reference_path():
    from mwdiem_gb300.dropin import ReferenceLoop
    sp = scene.pour_scene(n=300, seed=5, box=16.0, spacing=2.2, pool=24)
    sp.velocities = np.random.default_rng(5).normal(size=(300, 3)) * 0.3
    loop = ReferenceLoop(sp)
    ref = stepper.RefStepper(sp)
    contacts = 0
    for _ in range(10):
        loop.step()
        ref.step()
        assert oriented(loop.last_pairs) == oriented(ref.last_pairs)
        flags = dict(zip(map(tuple, ref.last_pairs.tolist()), ref.last_collision.tolist()))
        got = dict(zip(map(tuple, loop.last_pairs.tolist()), loop.last_collision.tolist()))
        assert got == flags
        contacts += int((ref.last_collision == 1).sum())
    assert contacts > 50
    W = sp.n_walls
    for k, bar in (("com", 2e-6 * 16.0), ("q", 1e-6)):
        assert np.abs(loop.st[k][W:] - ref.st[k][W:]).max() <= bar, k
    vmax = np.abs(ref.st["v"][W:]).max()
    assert np.abs(loop.st["v"][W:] - ref.st["v"][W:]).max() <= 1e-4 * vmax
