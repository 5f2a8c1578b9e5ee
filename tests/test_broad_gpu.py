"""Broad phase on the GPU against the oracle's restatement of ``Linked_cell_hash`` (whose list is
identical to the reference's, test_oracle.py) and of the wall test / cell keys of MWDiem.py:808-816.
Bar: the same set of oriented pairs, bit-exact keys."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def pairset(p):
    return set(map(tuple, np.asarray(p).reshape(-1, 2).tolist()))


@pytest.mark.parametrize("seed,n,spread", [(0, 20000, 20.0), (1, 5000, 4.0), (2, 3000, 60.0)])
def test_linked_cell_hash_matches(seed, n, spread):
    from mwdiem_gb300 import LIBRARY_Coarse_contact_detection as CCD
    rng = np.random.default_rng(seed)
    W = 5
    com = np.zeros((n + W, 3))
    com[W:] = rng.uniform([-spread, -spread, -3], [spread, spread, 3 * spread], size=(n, 3))
    cs, nx, ny = 2.4, 17, 17
    keys_o = oracle.cell_keys(com, cs, cs, cs, nx, ny)
    keys_g = CCD.cell_keys(com, cs, cs, cs, nx, ny)
    assert np.array_equal(keys_o, keys_g)
    ref = oracle.linked_cell_hash(W, n + W, keys_o, nx, ny)
    got = CCD.Linked_cell_hash(None, nx, ny, W, n + W, [], keys_g)
    assert len(got) == len(ref)
    assert pairset(got) == pairset(ref)


def test_linked_cell_hash_many_rows_matches():
    # 700,000 rows: enough for the place pass's large-count instance (two-member cells by an atomic
    # exchange); 78k two-member and 121k larger cells; the oriented pairs compared as sorted int64 codes
    import torch
    from mwdiem_gb300 import _lib
    rng = np.random.default_rng(21)
    n = 700_000
    com = rng.uniform([-100, -100, -3], [100, 100, 60], size=(n, 3))
    keys = oracle.cell_keys(com, 2.0, 2.0, 2.0, 100, 100)
    ref = oracle.linked_cell_hash(0, n, keys, 100, 100).astype(np.int64)
    cap = len(ref) + 1024
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    pairs = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    k = torch.from_numpy(keys).cuda()
    _lib.check(_lib.lib().mwd_linked_cell_hash(0, n, k.data_ptr(), 100, 100, pairs.data_ptr(), cap, cnt.data_ptr(),
                                               st.data_ptr(), None))
    torch.cuda.synchronize()
    got = pairs[: int(cnt.item())].cpu().numpy().astype(np.int64)
    assert int(st.item()) == 0 and len(got) == len(ref)
    code = lambda p: np.sort((p[:, 0] << 32) | p[:, 1])
    assert np.array_equal(code(got), code(ref))


def test_linked_cell_hash_wide_key_range_matches():
    # a key range of ~7e8 cells (beyond the dense table's 2^28) for 60,000 ids: the compressed table
    from mwdiem_gb300 import LIBRARY_Coarse_contact_detection as CCD
    rng = np.random.default_rng(23)
    n = 60_000
    com = rng.uniform([-20000, -20000, -3], [20000, 20000, 3], size=(n, 3))
    com[: n // 2, :2] = rng.uniform(-150, 150, size=(n // 2, 2))  # a dense patch, so pairs exist
    keys = oracle.cell_keys(com, 2.0, 2.0, 2.0, 20000, 20000)
    assert keys.max() - keys.min() + 1 > (1 << 28)
    ref = oracle.linked_cell_hash(0, n, keys, 20000, 20000)
    got = CCD.Linked_cell_hash(None, 20000, 20000, 0, n, [], keys)
    assert len(ref) > 1000 and len(got) == len(ref) and pairset(got) == pairset(ref)


def test_crowded_cells_and_negative_keys():
    from mwdiem_gb300 import LIBRARY_Coarse_contact_detection as CCD
    rng = np.random.default_rng(3)
    n = 4000
    com = rng.normal(scale=3.0, size=(n, 3))  # many particles per cell, negative coordinates
    keys = oracle.cell_keys(com, 2.0, 2.0, 2.0, 7, 7)
    ref = oracle.linked_cell_hash(0, n, keys, 7, 7)
    got = CCD.Linked_cell_hash(None, 7, 7, 0, n, [], keys)
    assert pairset(got) == pairset(ref) and len(got) == len(ref)


def test_wall_pairs_match():
    from mwdiem_gb300 import LIBRARY_Coarse_contact_detection as CCD
    rng = np.random.default_rng(4)
    W, n = 5, 6000
    com = rng.uniform(-20, 20, size=(n + W, 3))
    wn = rng.normal(size=(W, 3))
    wn /= np.linalg.norm(wn, axis=1, keepdims=True)
    wc = rng.uniform(-5, 5, size=(W, 3))
    ref = oracle.wall_pairs(W, W, n + W, com, wn, wc, 14.4)
    got = CCD.wall_pairs(com, wn, wc, W, W, n + W, 14.4).cpu().numpy()
    assert np.array_equal(got, ref)  # wall-major order, as MWDiem.py:808-811


def test_empty_ranges():
    from mwdiem_gb300 import LIBRARY_Coarse_contact_detection as CCD
    keys = np.zeros(10, np.int64)
    assert CCD.Linked_cell_hash(None, 4, 4, 3, 3, [], keys) == []
    one = CCD.Linked_cell_hash(None, 4, 4, 3, 4, [], keys)
    assert one == []
    two = CCD.Linked_cell_hash(None, 4, 4, 3, 5, [], keys)
    assert pairset(two) == pairset(oracle.linked_cell_hash(3, 5, keys, 4, 4))


def test_very_crowded_cell_flags_status():
    # more members in one cell than the set-order emulation covers: same unordered pairs, status set
    import torch
    from mwdiem_gb300 import _lib
    n = 400
    keys = np.zeros(n, np.int64)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    pairs = torch.zeros((n * n, 2), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    k = torch.from_numpy(keys).cuda()
    _lib.check(_lib.lib().mwd_linked_cell_hash(0, n, k.data_ptr(), 4, 4, pairs.data_ptr(), n * n, cnt.data_ptr(),
                                               st.data_ptr(), None))
    torch.cuda.synchronize()
    got = pairs[: int(cnt.item())].cpu().numpy()
    ref = oracle.linked_cell_hash(0, n, keys, 4, 4)
    assert int(st.item()) & _lib.ST_CELL_CROWDED
    assert set(map(frozenset, got.tolist())) == set(map(frozenset, ref.tolist()))
