"""The C-ABI library builds, loads and exports every entry point include/mwdem.h declares (no
device calls: this runs without a GPU)."""
import re
from pathlib import Path

HEADER = Path(__file__).resolve().parents[1] / "include" / "mwdem.h"


def declared():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(mwd_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from mwdiem_gb300 import _lib
    h = _lib.lib()
    names = declared()
    assert len(names) >= 14
    for n in names:
        assert hasattr(h, n), n
    assert set(_lib.EXPORTED) <= set(names)
    assert h.mwd_version() >= 1


def test_host_side_material_constants():
    import ctypes
    import math
    from mwdiem_gb300 import _lib
    p = _lib.ContactParams(1e5, 0.372, 0.372, 0.5, 3e4, 0.5, 0.6, 0.3, 5e-5, 4, 0, 0, 0)
    m = (_lib.Material * 2)()
    _lib.check(_lib.lib().mwd_derive_material(ctypes.byref(p), m))
    # Gn = -2 mu / tc * ln(en) with tc = sqrt(mu (pi^2 + ln^2 en) / Kn): = 2 zeta sqrt(mu Kn)-like
    ln = math.log(0.372)
    tc = math.sqrt(0.5 * (math.pi ** 2 + ln * ln) / 1e5)
    assert abs(m[0].Gn - (-2 * 0.5 / tc * ln)) < 1e-3 * abs(m[0].Gn)
    assert abs(m[1].inv_mu - 1 / 0.3) < 1e-12
    assert m[0].Kn_f == 1e5 and abs(m[0].dt_f - 5e-5) < 1e-10


def test_errors_are_codes_not_aborts():
    import ctypes
    from mwdiem_gb300 import _lib
    rc = _lib.lib().mwd_contact_pairs(-1, 8, 1, *([None] * 20), None, None, None, None)
    assert rc == _lib.MWD_ERR_INVALID
    assert b"bad arguments" in _lib.lib().mwd_last_error()


def test_mirrored_row_pass_checks_its_block():
    # mwd_integrate_rows_mirror rejects, before any device call, a state array outside the mirrored
    # block and a mirror whose offset from the block is not a multiple of 32 bytes
    import ctypes
    import numpy as np
    from mwdiem_gb300 import _lib
    n = 4
    block = np.zeros(208 * n + 64, np.uint8)
    base = (block.ctypes.data + 31) // 32 * 32
    st = _lib.State()
    st.n = n
    off = 0
    for name, width in (("pos", 32), ("dx_all", 32), ("vel", 16), ("vel_half", 16), ("w_half_bf", 16),
                        ("w_bf", 16), ("w", 16), ("q", 16), ("q_half", 16), ("q_all", 16), ("q_acc", 16)):
        setattr(st, name, base + off)
        off += width * n
    st.vert_owner = st.xform = base      # only checked for presence before the launch
    scenes = mirror = base               # never dereferenced on these paths
    h = _lib.lib()
    rc = h.mwd_integrate_rows_mirror(ctypes.byref(st), scenes, None, mirror + 4096, base, off - 16, None)
    assert rc == _lib.MWD_ERR_INVALID and b"outside" in h.mwd_last_error()
    rc = h.mwd_integrate_rows_mirror(ctypes.byref(st), scenes, None, mirror + 4096 + 16, base, off, None)
    assert rc == _lib.MWD_ERR_INVALID and b"alignment" in h.mwd_last_error()
    st.xform = None
    rc = h.mwd_integrate_rows_mirror(ctypes.byref(st), scenes, None, mirror, base, off, None)
    assert rc == _lib.MWD_ERR_INVALID


def test_cell_table_choice():
    # which cell table mwd_broadphase uses (host logic, no device call): automatic and explicit dense
    # give the dense table; the compressed one only where its arrays fit inside the dense ones
    from mwdiem_gb300 import _lib
    h = _lib.lib()
    assert h.mwd_cell_table(2_000_000, 15_200_000, 0) == 1
    assert h.mwd_cell_table(2_000_000, 300_000_000, 0) == 2   # automatic: beyond 2^27 cells
    assert h.mwd_cell_table(2_000_000, 15_200_000, 1) == 1
    assert h.mwd_cell_table(2_000_000, 15_200_000, 2) == 2
    assert h.mwd_cell_table(20_000, 140_005, 2) == 2
    assert h.mwd_cell_table(20_000, 20_000 * 4 + 4095, 2) == 1   # below 4 n + 4096 cells
    assert h.mwd_cell_table(0, 1_000_000, 2) == 1


def test_cell_table_sizes():
    # the ints the cell_count / cell_start arrays need for the chosen table (host logic)
    import ctypes
    from mwdiem_gb300 import _lib
    h = _lib.lib()
    c, s = ctypes.c_int64(), ctypes.c_int64()
    assert h.mwd_cell_table_ints(20_000, 140_005, 0, ctypes.byref(c), ctypes.byref(s)) == 1
    assert (c.value, s.value) == (140_005, 140_006)
    assert h.mwd_cell_table_ints(5_005, 5_400_000, 2, ctypes.byref(c), ctypes.byref(s)) == 2
    words = (5_400_000 + 31) // 32
    pad = (words + 1 + 3) // 4 * 4
    rows = (5_005 + 1 + 3) // 4 * 4
    assert (c.value, s.value) == (pad + rows, 2 * pad + rows + 1)
    assert c.value + s.value < 0.15 * (2 * 5_400_000 + 1)
