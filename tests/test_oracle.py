"""The oracle (oracle/mwdem_oracle.c, a CPU restatement) pinned against the reference:
  * the golden fixtures in tests/golden/, made by tests/golden/make_golden.py from the reference's own
    kernels (rendered + compiled for the CPU) and its own Python Linked_cell_hash;
  * when the reference checkout is present, the host-compiled reference on fresh random inputs.
Bar: bit-identical outputs."""
import ast
from pathlib import Path

import numpy as np
import pytest

import oracle
from helpers import CONTACT_PARAMS, make_pairs, make_verlet_state, select

G = Path(__file__).resolve().parent / "golden"


def bits_equal(a, b):
    """Bit-identical, except that NaNs compare by position only (payload bits differ between the CPU
    and the GPU, which produce different NaN encodings)."""
    a = np.array(a)
    b = np.array(b, dtype=a.dtype)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        na, nb = np.isnan(a), np.isnan(b)
        if not np.array_equal(na, nb):
            return False
        a[na] = 0
        b[nb] = 0
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def load_contact():
    z = np.load(G / "contact.npz")
    params = ast.literal_eval(str(z["params_json"]))
    inp = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    return z, params, inp, int(z["N"])


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_contact_golden(prec):
    z, params, inp, N = load_contact()
    o = oracle.contact(inp, params, N, prec)
    for k in ("collision", "force", "torque", "hist"):
        assert bits_equal(o[k], z[f"{prec}_{k}"]), k
    assert (z["f32_collision"] == 1).sum() > 50 and (z["f32_collision"] == 0).sum() > 50


def test_contact_golden_history_variants():
    z, params, inp, N = load_contact()
    inp = dict(inp, hist=z["hist_in"])
    o = oracle.contact(inp, params, N, "f32", hist_stride4=True)
    for k in ("collision", "force", "torque", "hist"):
        assert bits_equal(o[k], z[f"histfix_{k}"]), k
    o1 = oracle.contact(inp, params, N, "f32")
    for k in ("collision", "force", "torque", "hist"):
        assert bits_equal(o1[k], z[f"stride1_{k}"]), k


def test_physical_law_closed_form():
    # the physical-mass variant of the contact law (not in the reference) on a known answer: two
    # axis-aligned cubes overlapping by 0.1 along x, A approaching at 0.2, masses 4 and 2.  The normal
    # force is Kn depth + Gn u_n with Gn = -2 m_n ln en / tc, tc = sqrt(m_n (pi^2 + ln^2 en) / Kn),
    # m_n = 1 / (1/4 + 1/2); no tangential motion, so no tangential force; torques about the
    # midpoint contact point (cpA + cpB) / 2.
    from helpers import cube_pair_kat
    params = dict(CONTACT_PARAMS, num_particles_wall=0)
    inp = {k: np.asarray(v, np.float64) if np.asarray(v).dtype == np.float32 else v
           for k, v in cube_pair_kat(depth=0.1).items()}
    inp["A_vel"] = np.array([[0.2, 0.0, 0.0]])
    imA, imB = np.array([0.25]), np.array([0.5])
    o = oracle.contact(inp, params, 2, "f64", inv_mass=(imA, imB))
    assert o["collision"][0] == 1
    d = o["diag"][0]
    depth = d[0]  # 0.1 up to the float32 rounding of the fixture's vertices
    assert abs(depth - 0.1) < 1e-6
    mn = 1.0 / (0.25 + 0.5)
    Len = np.log(params["en"])
    tc = np.sqrt(mn * (np.pi ** 2 + Len ** 2) / params["Kn"])
    Gn = -2.0 * mn * Len / tc
    F = np.array([-(params["Kn"] * depth + Gn * 0.2), 0.0, 0.0])
    assert np.allclose(o["force"][0], F, rtol=1e-12, atol=1e-9)
    assert np.allclose(o["force"][1], -F, rtol=1e-12, atol=1e-9)
    cp = (d[4:7] + d[7:10]) / 2
    assert np.allclose(o["torque"][0], np.cross(cp - inp["A_com"][0], F), rtol=1e-9, atol=1e-9)
    assert np.allclose(o["torque"][1], np.cross(cp - inp["B_com"][0], -F), rtol=1e-9, atol=1e-9)
    # the reference's law on the same pair uses mu = 0.5 as the mass: a different damping force
    r = oracle.contact(inp, params, 2, "f64")
    assert abs(r["force"][0, 0] - F[0]) > 1.0
    # FP32 restatement of the physical law against the FP64 one
    o32 = oracle.contact(cube_pair_kat(depth=0.1) | {"A_vel": np.array([[0.2, 0.0, 0.0]], np.float32)}, params, 2,
                         "f32", inv_mass=(imA, imB))
    assert np.allclose(o32["force"], o["force"], rtol=1e-5, atol=1e-2)


def test_verlet_golden():
    z = np.load(G / "verlet.npz")
    st = {k[3:]: z[k].copy() for k in z.files if k.startswith("in_")}
    for _ in range(10):
        oracle.verlet_f64(st, float(z["dt"]), tuple(z["box"]), int(z["W"]), int(z["n_max"]))
    for k in st:
        assert bits_equal(st[k], z["out_" + k]), k


def test_broad_golden():
    z = np.load(G / "broad.npz")
    com, cs = z["com"], z["cs"]
    nx, ny, W = int(z["nx"]), int(z["ny"]), int(z["W"])
    keys = oracle.cell_keys(com, cs[0], cs[1], cs[2], nx, ny)
    assert np.array_equal(keys, z["keys"])
    cells = oracle.linked_cell_hash(W, com.shape[0], keys, nx, ny)
    assert np.array_equal(cells, z["cell_pairs"])  # same list, same order, same orientation
    walls = oracle.wall_pairs(W, W, com.shape[0], com, z["normals"], com[:W], float(z["wall_range"]))
    assert np.array_equal(walls, z["wall_pairs"])


def test_pyset_order_matches_cpython():
    rng = np.random.default_rng(0)
    for _ in range(3000):
        n = int(rng.integers(1, 33))
        ids = np.sort(rng.choice(int(rng.choice([40, 1000, 10 ** 6])), size=n, replace=False))
        s = set()
        for i in ids:
            s.add(int(i))
        assert list(s) == oracle.pyset_order(ids).tolist()


ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not present")


@ref
def test_oracle_vs_live_reference():
    inp, N = make_pairs(600, seed=31, unique_ids=False, n_particles=300)
    keep = oracle.contact(inp, CONTACT_PARAMS, N, "f32", face_cap=50)["status"] == 0
    inp = select(inp, keep)
    r = oracle.RefContact(CONTACT_PARAMS, "f32").run(inp, N, snapshot=True)
    o = oracle.contact(inp, CONTACT_PARAMS, N, "f32")
    for k in ("collision", "force", "torque", "hist"):
        assert bits_equal(o[k], r[k]), k
    st, box = make_verlet_state(40, 32, seed=32)
    vp = dict(timestep_size=1e-3, num_particles=40, num_vertices_max=32, syssize_x_max=box[0],
              syssize_x_min=box[1], syssize_y_max=box[2], syssize_y_min=box[3], syssize_z_max=box[4],
              syssize_z_min=box[5], num_part_min=3, num_part_max=38)
    a = {k: v.copy() for k, v in st.items()}
    b = {k: v.copy() for k, v in st.items()}
    R = oracle.RefVerlet(vp)
    for _ in range(5):
        oracle.verlet_f64(a, 1e-3, box, 3, 38)
        R.run(b)
    for k in a:
        assert bits_equal(a[k], b[k]), k
