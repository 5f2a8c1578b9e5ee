"""Every struct of include/mwdem.h has the size and field offsets its ctypes mirror in
mwdiem_gb300/_lib.py assumes (a host C compiler lays the header out; no GPU needed)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

STRUCTS = {
    "mwd_contact_params": "ContactParams",
    "mwd_material": "Material",
    "mwd_verlet_params": "VerletParams",
    "mwd_state": "State",
    "mwd_scene": "Scene",
    "mwd_work": "Work",
    "mwd_contact_rec": "ContactRec",
    "mwd_diff": "Diff",
    "mwd_inlet": "Inlet",
}


def test_struct_layouts_match_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    from mwdiem_gb300 import _lib
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mwdem.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(_lib, pyname)
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            s, f, v = ln.split()
            got[(s, f)] = int(v)
    for cname, pyname in STRUCTS.items():
        cls = getattr(_lib, pyname)
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for f in cls._fields_:
            assert got[(cname, f[0])] == getattr(cls, f[0]).offset, (cname, f[0])
