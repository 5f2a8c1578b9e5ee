"""The lanes word of the narrow phase (GJK-pass lanes | EPA-pass lanes << 8 | hulls read in place
<< 16 | block-size codes of the two passes << 20 and << 22), as bench.py parses it and the autotuner
names it: the two are inverse on every setting the autotuner tries, and the header's bit positions
are the autotuner's."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_parse_and_describe_are_inverse():
    import bench
    from mwdiem_gb300 import autotune
    for base in autotune.DEFAULT_CANDIDATES:
        for lanes in (base,) + autotune.block_candidates(base):
            text = autotune.describe(lanes)
            assert bench.parse_lanes(text) == lanes, text
    assert autotune.block_size(bench.parse_lanes("gjk8/epa32g/b256x64")) == {"gjk": 256, "epa": 64}
    assert bench.parse_lanes("gjk1/epa16g") == 1 | (16 << 8) | (1 << 16)
    assert bench.lanes_arg("8") == 8


def test_bad_setting_is_refused():
    import bench
    with pytest.raises(SystemExit):
        bench.parse_lanes("gjk1-epa16")


def test_header_bit_positions():
    import re
    from mwdiem_gb300 import autotune
    text = (ROOT / "include" / "mwdem.h").read_text()
    defs = dict(re.findall(r"#define (MWD_LANES_\w+) \(?(?:1 << )?(\d+)\)?", text))
    assert int(defs["MWD_LANES_GJK_BLOCK_SHIFT"]) == autotune.GJK_BLOCK_SHIFT
    assert int(defs["MWD_LANES_EPA_BLOCK_SHIFT"]) == autotune.EPA_BLOCK_SHIFT
    assert 1 << int(defs["MWD_LANES_EPA_IN_PLACE"]) == autotune.EPA_IN_PLACE
