"""The lanes word of the narrow phase (GJK-pass lanes | EPA-pass lanes << 8 | hulls read in place
<< 16), as bench.py parses it and the autotuner names it: the two are inverse on every setting the
autotuner tries."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_parse_and_describe_are_inverse():
    import bench
    from mwdiem_gb300 import autotune
    for lanes in autotune.DEFAULT_CANDIDATES:
        text = autotune.describe(lanes)
        assert bench.parse_lanes(text) == lanes, text
    assert bench.parse_lanes("gjk1/epa16g") == 1 | (16 << 8) | (1 << 16)
    assert bench.lanes_arg("8") == 8


def test_bad_setting_is_refused():
    import bench
    with pytest.raises(SystemExit):
        bench.parse_lanes("gjk1-epa16")
