"""The allocation-free narrow phase, mwd_contact_pairs_noalloc, against mwd_contact_pairs.

Some callers of this library cannot let it allocate device memory: an application whose own
allocator owns (nearly) all of the GPU's memory, a process given a fixed slice of device memory up
front, and a loop that cannot take the device-wide stall of the cudaFree that mwd_contact_pairs
makes when its scratch grows.  mwd_contact_pairs_noalloc serves them from a fixed-size array
compiled into the library instead of library-allocated scratch.  Both entry points are called here
through the C ABI on the same inputs, twice in a row with different inputs (the fixed array keeps
the first call's contents), and must agree bit for bit -- the bar the other contact tests use when
every particle is in one pair.  A child process then checks that a call allocates nothing: the
device's free memory and torch's allocator are unchanged across a 200,000-pair call, while the
same measurement sees the allocating entry point's cudaMalloc.

This file is collected last so that a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from helpers import CONTACT_PARAMS, make_pairs

pytestmark = pytest.mark.gpu

NAMES = ("A_com", "B_com", "A_verts", "B_verts", "A_vel", "B_vel", "A_angvel", "B_angvel", "A_nv", "B_nv", "A_id",
         "B_id")


def _bind():
    from mwdiem_gb300 import _lib
    h = _lib.lib()
    f = h.mwd_contact_pairs_noalloc
    f.restype = C.c_int
    f.argtypes = h.mwd_contact_pairs.argtypes
    return h, _lib


def _call(fn, inp, N, prm):
    d = {k: torch.from_numpy(np.ascontiguousarray(inp[k])).cuda() for k in inp}
    P = int(d["A_com"].shape[0])
    F = torch.zeros((N, 3), dtype=torch.float32, device="cuda")
    T = torch.zeros_like(F)
    hist = d["hist"].clone()
    coll = torch.full((P,), 7, dtype=torch.int32, device="cuda")
    diag = torch.zeros((P, 10), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = fn(P, int(inp["A_verts"].shape[1]), N, *[d[k].data_ptr() for k in NAMES], hist.data_ptr(), F.data_ptr(),
            T.data_ptr(), d["qA"].data_ptr(), d["qB"].data_ptr(), d["IsA"].data_ptr(), d["IsB"].data_ptr(),
            coll.data_ptr(), C.byref(prm), diag.data_ptr(), st.data_ptr(), None)
    torch.cuda.synchronize()
    return rc, {k: v.cpu().numpy() for k, v in dict(F=F, T=T, hist=hist, coll=coll, diag=diag, st=st).items()}


def _same(a, b):
    for k in a:
        x, y = np.array(a[k]), np.array(b[k])
        if x.dtype.kind == "f":
            nx, ny = np.isnan(x), np.isnan(y)
            assert np.array_equal(nx, ny), k
            x[nx] = 0
            y[ny] = 0
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), k


def test_noalloc_matches_allocating_entry_point_twice():
    h, _lib = _bind()
    p = CONTACT_PARAMS
    for seed, P, hist_mode in ((41, 3000, 0), (42, 700, 0), (43, 500, 1)):
        inp, N = make_pairs(P, seed=seed)
        inp["hist"] = (np.random.default_rng(seed).normal(size=(P, 4)) * 1e-4).astype(np.float32)
        prm = _lib.ContactParams(p["Kn"], p["en"], p["et"], p["mu"], p["Kn_wall"], p["en_wall"], p["et_wall"],
                                 p["mu_wall"], p["timestep"], p["num_particles_wall"], hist_mode, 8, 0)
        rc0, want = _call(h.mwd_contact_pairs, inp, N, prm)
        rc1, got = _call(h.mwd_contact_pairs_noalloc, inp, N, prm)
        assert rc0 == 0 and rc1 == 0, h.mwd_last_error()
        assert (want["coll"] == 1).sum() > 100
        _same(want, got)


def test_noalloc_rejects_oversize_calls():
    h, _lib = _bind()
    p = CONTACT_PARAMS
    prm = _lib.ContactParams(p["Kn"], p["en"], p["et"], p["mu"], p["Kn_wall"], p["en_wall"], p["et_wall"],
                             p["mu_wall"], p["timestep"], p["num_particles_wall"], 0, 8, 0)
    rc = h.mwd_contact_pairs_noalloc(_lib.NOALLOC_MAX_PAIRS + 1, 32, 10, *([None] * 20), C.byref(prm), None, None,
                                     None)
    assert rc == _lib.MWD_ERR_INVALID
    assert b"fixed scratch" in h.mwd_last_error()


# Run in a fresh interpreter, so that nothing this process did earlier (another test's call of
# mwd_contact_pairs growing its scratch) can hide an allocation.
_CHILD = r"""
import ctypes as C, json, sys
import numpy as np, torch
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/tests"]
from helpers import CONTACT_PARAMS, make_pairs
from mwdiem_gb300 import _lib
h = _lib.lib()
f = h.mwd_contact_pairs_noalloc
f.restype = C.c_int
f.argtypes = h.mwd_contact_pairs.argtypes
base, N0 = make_pairs(2000, seed=44)
reps = 100                                   # 200,000 pairs: the fixed scratch holds 262,144
inp = {k: np.concatenate([v] * reps) for k, v in base.items()}
inp["A_id"] = np.concatenate([base["A_id"] + r * N0 for r in range(reps)]).astype(np.int32)
inp["B_id"] = np.concatenate([base["B_id"] + r * N0 for r in range(reps)]).astype(np.int32)
N = N0 * reps
P = len(inp["A_id"])
names = ("A_com", "B_com", "A_verts", "B_verts", "A_vel", "B_vel", "A_angvel", "B_angvel", "A_nv", "B_nv",
         "A_id", "B_id")
d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in inp.items()}
F = torch.zeros((N, 3), dtype=torch.float32, device="cuda")
T = torch.zeros_like(F)
hist = d["hist"].clone()
coll = torch.zeros(P, dtype=torch.int32, device="cuda")
st = torch.zeros(1, dtype=torch.int32, device="cuda")
p = CONTACT_PARAMS
prm = _lib.ContactParams(p["Kn"], p["en"], p["et"], p["mu"], p["Kn_wall"], p["en_wall"], p["et_wall"],
                         p["mu_wall"], p["timestep"], p["num_particles_wall"], 0, 8, 0)
def call(fn, n):
    rc = fn(n, int(inp["A_verts"].shape[1]), N, *[d[k].data_ptr() for k in names], hist.data_ptr(), F.data_ptr(),
            T.data_ptr(), d["qA"].data_ptr(), d["qB"].data_ptr(), d["IsA"].data_ptr(), d["IsB"].data_ptr(),
            coll.data_ptr(), C.byref(prm), None, st.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0, h.mwd_last_error()
def snap():
    return torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
call(f, 1000)                 # loads the kernels and looks up the array's address
before = snap()
call(f, P)
after_noalloc = snap()
call(h.mwd_contact_pairs, P)  # control: its scratch is allocated on this first call
after_alloc = snap()
print(json.dumps(dict(before=before, noalloc=after_noalloc, alloc=after_alloc, contacts=int((coll == 1).sum()))))
"""


def test_noalloc_call_allocates_nothing():
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = str(Path(__file__).resolve().parents[1])
    r = subprocess.run([sys.executable, "-c", _CHILD, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    m = json.loads(r.stdout.strip().splitlines()[-1])
    assert m["contacts"] > 10000
    # the allocation-free call: device free memory and torch's allocator unchanged
    assert m["noalloc"] == m["before"], m
    # the allocating entry point's first call takes ~7.6 MB of scratch, which the same measurement sees
    assert m["alloc"][0] < m["noalloc"][0], m
