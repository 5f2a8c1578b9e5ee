"""The place pass's two-member shortcut (broad.cu pyset_pair_lo_first) restated in Python and checked
against CPython's own set iteration order: list({lo - base, hi - base}) built by inserting the smaller
id first, as the reference's dict-of-sets walk does (LIBRARY_Coarse_contact_detection.py:84-155)."""
import numpy as np


def pair_lo_first(lo, hi, base):
    """broad.cu pyset_pair_lo_first: slot of lo, then hi's probe sequence (no linear probes in an
    8-slot table; perturbation while the slot is taken)."""
    ia = (lo - base) & 7
    h = (hi - base) & 0xFFFFFFFF
    i = h & 7
    perturb = h
    steps = 0
    while i == ia:
        perturb >>= 5
        i = (i * 5 + 1 + perturb) & 7
        steps += 1
        assert steps <= 15
    return ia < i


def cpython_lo_first(lo, hi, base):
    s = set()
    s.add(lo - base)
    s.add(hi - base)
    return list(s)[0] == lo - base


def test_pair_order_matches_cpython():
    rng = np.random.default_rng(7)
    base = rng.integers(0, 1 << 20, 20000)
    lo = base + rng.integers(0, 1 << 16, 20000)
    gap = np.where(rng.uniform(size=20000) < 0.5, 8 * rng.integers(1, 1 << 12, 20000), rng.integers(1, 64, 20000))
    hi = lo + gap
    for a, b, c in zip(lo.tolist(), hi.tolist(), base.tolist()):
        assert pair_lo_first(a, b, c) == cpython_lo_first(a, b, c), (a, b, c)
    # every residue pair of the 8-slot table, with collisions and large ids
    for a in range(64):
        for b in range(a + 1, a + 200):
            assert pair_lo_first(a, b, 0) == cpython_lo_first(a, b, 0)
            assert pair_lo_first(a + 10**9, b + 10**9, 0) == cpython_lo_first(a + 10**9, b + 10**9, 0)
