"""The device-step narrow phase on independent random pairs (the GJK/EPA pairs/s workload, hulls of
8-64 vertices, centre distance U[0.5,2.2] (rA+rB)/2) against the FP32 oracle: contact flags and the
per-row forces/torques (each row is in one pair) bit-identical on a sample; at full size the
size-independent properties (every pair decided, contact fraction in range, momentum balance)."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a, b = np.array(a), np.array(b, dtype=np.asarray(a).dtype)
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    a[na] = 0
    b[nb] = 0
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("two_pass,lanes", [(True, 8), (False, 16), (True, 4 | (16 << 8) | (1 << 16)),
                                            (True, 8 | (32 << 8) | (1 << 16)), (True, 1 | (16 << 8)),
                                            (True, 1 | (8 << 8) | (1 << 16)),
                                            (True, 1 | (32 << 8) | (1 << 16))])
def test_pairs_vs_oracle(two_pass, lanes):
    from mwdiem_gb300.pairbench import PairScene
    ps = PairScene(6000, seed=3, pool=96, lanes=lanes, two_pass=two_pass)
    ps.narrow()
    torch.cuda.synchronize()
    coll = ps.w["collision"].cpu().numpy()
    idx = np.arange(6000)
    o = oracle.contact(ps.gather(idx), ps.params, 12000, "f32")
    assert np.array_equal(coll, o["collision"])
    assert 0.3 < (coll == 1).mean() < 0.8
    F = ps.t["force"][:, :3].cpu().numpy()
    T = ps.t["torque"][:, :3].cpu().numpy()
    assert bits_equal(F, o["force"]) and bits_equal(T, o["torque"])


def test_pairs_large_properties():
    from mwdiem_gb300.pairbench import PairScene
    n = 1 << 20
    ps = PairScene(n, seed=4, pool=256)
    ps.narrow()
    torch.cuda.synchronize()
    coll = ps.w["collision"].cpu().numpy()
    assert set(np.unique(coll)) <= {-1, 0, 1}
    assert (coll == -1).sum() <= n * 1e-4
    frac = (coll == 1).mean()
    assert 0.3 < frac < 0.8
    F = ps.t["force"][:, :3].double()
    # normal forces are equal and opposite within each pair
    s = (F[0::2] + F[1::2]).abs().max().item()
    assert s <= 1e-3 * F.abs().max().item()
    # a sample still matches the oracle exactly
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(n, size=3000, replace=False))
    o = oracle.contact(ps.gather(idx), ps.params, 2 * n, "f32")
    assert np.array_equal(coll[idx], o["collision"])
