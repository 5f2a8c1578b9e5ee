"""Integrator over the reference's FP64 arrays on the GPU (``mwd_verlet_ref`` through the drop-in
``Verlet_GPU``) against the oracle's FP64 restatement.  The operation sequence is the reference's;
sin/cos come from different libraries (CUDA vs the C library), so the bar is 1e-12 relative per
quantity over 20 steps (each step feeds the next)."""
import numpy as np
import pytest
import torch

import oracle
from helpers import make_verlet_state

pytestmark = pytest.mark.gpu

ORDER = ("v12", "q", "wbf", "w12bf", "w", "q12", "v", "com", "verts", "qall", "dxall")


def gpu_step(st, dt, box, W, N, V):
    from mwdiem_gb300 import gpu_Verlet
    out = gpu_Verlet.Verlet_GPU(st["v"], st["v12"], st["w12bf"], st["q12"], st["q"], st["qall"], st["wbf"], st["w"],
                                st["F"], st["T"], st["verts"], st["com"], dt, st["mass"], N, st["Iinv"], st["I"],
                                st["dxall"], V, box[0], box[1], box[2], box[3], box[4], box[5], W, N - 2)
    return dict(zip(ORDER, out))


def test_verlet_matches_oracle_fp64():
    N, V, W, dt = 300, 32, 3, 1e-3
    st, box = make_verlet_state(N, V, seed=4, W=W)
    a = {k: v.copy() for k, v in st.items()}
    b = {k: v.copy() for k, v in st.items()}
    for _ in range(20):
        oracle.verlet_f64(a, dt, box, W, N - 2)
        out = gpu_step(b, dt, box, W, N, V)
        for k in ORDER:
            assert out[k] is b[k]  # in-place, like pycuda InOut
    for k in ("v", "v12", "w12bf", "wbf", "w", "com", "dxall", "q12", "q", "qall", "verts"):
        scale = max(np.abs(a[k]).max(), 1e-30)
        assert np.abs(a[k] - b[k]).max() <= 1e-12 * scale, k
    # rows outside [n_min, n_max) untouched
    assert np.array_equal(b["com"][:W], st["com"][:W])


def test_verlet_fly_away_reset():
    # gpu_Verlet.cu:338-352: a centre leaving the box stops the particle and undoes the move
    N, V, W, dt = 16, 8, 3, 1e-3
    st, box = make_verlet_state(N, V, seed=6, W=W)
    b = {k: v.copy() for k, v in st.items()}
    gpu_step(b, dt, box, W, N, V)
    assert np.all(b["v"][W + 1] == 0) and np.all(b["v12"][W + 1] == 0) and np.all(b["w"][W + 1] == 0)
    assert np.allclose(b["com"][W + 1], st["com"][W + 1], rtol=0, atol=1e-12)


def test_verlet_device_tensors():
    from mwdiem_gb300 import gpu_Verlet
    N, V, W, dt = 64, 16, 2, 5e-4
    st, box = make_verlet_state(N, V, seed=5, W=W)
    a = {k: v.copy() for k, v in st.items()}
    d = {k: torch.from_numpy(v.copy()).cuda() for k, v in st.items()}
    nres = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu_Verlet.Verlet_GPU(d["v"], d["v12"], d["w12bf"], d["q12"], d["q"], d["qall"], d["wbf"], d["w"], d["F"],
                          d["T"], d["verts"], d["com"], dt, d["mass"], N, d["Iinv"], d["I"], d["dxall"], V, *box, W,
                          N - 2, n_reset=nres)
    r = oracle.verlet_f64(a, dt, box, W, N - 2)
    assert int(nres.item()) == r == 1
    for k in ("com", "verts", "q", "v"):
        assert np.abs(d[k].cpu().numpy() - a[k]).max() <= 1e-12 * np.abs(a[k]).max()
