"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference checkout exists; its location comes from the first argument, else from
$MWDEM_REFERENCE_ROOT, else from oracle/build_ref.py's default:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

Sources of truth (nothing here is restated by hand except the 3-line wall test):
  * contact_*.npz  -- the reference's contact_detection kernel (LIBRARIES/gpu_fine_contact_detection.cu)
    rendered with its own Jinja call and compiled for the CPU by oracle/build_ref.py, run serially;
    every pair reads the history array as it was on entry (what a GPU warp sees).
  * verlet.npz     -- the reference's Verlet kernel (LIBRARIES/gpu_Verlet.cu), same recipe.
  * broad.npz      -- LIBRARY_Coarse_contact_detection.Linked_cell_hash imported from the reference and
    run in this CPython; the wall candidates follow MWDiem.py:808-811.

Pairs whose EPA needs more than the reference's 50 faces are left out: the reference writes past its
T[50]/n[50]/dist[50] arrays there (undefined behaviour, a crash on the CPU).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))

import build_ref  # noqa: E402
import oracle  # noqa: E402
from helpers import cube_pair_kat, make_pairs, make_verlet_state, select  # noqa: E402

PARAMS = dict(Kn=1e5, en=0.372, et=0.372, mu=0.5, Kn_wall=3e4, en_wall=0.5, et_wall=0.6, mu_wall=0.3,
              num_vertices_max=16, num_particles_wall=6, timestep=5e-5)


def contact_inputs():
    a, N = make_pairs(260, seed=101, V=16, n_min=6, n_max=16, dist=(0.4, 2.0), unique_ids=False,
                      n_particles=90)
    b, _ = make_pairs(60, seed=102, V=16, n_min=6, n_max=16, dist=(2.2, 3.5), unique_ids=False, n_particles=90)
    k = cube_pair_kat(0.1, V=16)
    k["A_id"][:] = 7
    k["B_id"][:] = 8
    # identical shapes at the same place (degenerate simplex, CorrectFlat path)
    d = select(a, slice(0, 12))
    d["B_com"] = d["A_com"].copy()
    d["B_verts"] = d["A_verts"].copy()
    d["B_nv"] = d["A_nv"].copy()
    inp = {key: np.concatenate([a[key], b[key], k[key], d[key]]) for key in a}
    ok = oracle.contact(inp, PARAMS, N, "f32", face_cap=50)["status"] == 0
    ok &= oracle.contact(inp, PARAMS, N, "f64", face_cap=50)["status"] == 0
    return select(inp, ok), N


def main():
    if len(sys.argv) > 1:
        build_ref.set_reference_root(sys.argv[1])
    if not build_ref.reference_available():
        raise SystemExit("reference checkout not found")
    inp, N = contact_inputs()
    r32 = oracle.RefContact(PARAMS, "f32").run(inp, N, snapshot=True)
    r64 = oracle.RefContact(PARAMS, "f64").run(inp, N, snapshot=True)
    rng = np.random.default_rng(103)
    hist_in = (rng.normal(size=inp["hist"].shape) * 1e-4).astype(np.float32)
    inp_h = dict(inp, hist=hist_in)
    rh = oracle.RefContact(PARAMS, "histfix").run(inp_h, N, snapshot=False)
    r1 = oracle.RefContact(PARAMS, "f32").run(inp_h, N, snapshot=True)
    np.savez_compressed(HERE / "contact.npz", N=N, params_json=np.array(repr(PARAMS)), hist_in=hist_in,
                        **{"in_" + k: v for k, v in inp.items()},
                        **{"f32_" + k: v for k, v in r32.items()}, **{"f64_" + k: v for k, v in r64.items()},
                        **{"histfix_" + k: v for k, v in rh.items()}, **{"stride1_" + k: v for k, v in r1.items()})

    # integrator: 10 steps of the reference kernel
    Nv, V, W, dt = 24, 16, 2, 1e-3
    st, box = make_verlet_state(Nv, V, seed=104, W=W)
    vp = dict(timestep_size=dt, num_particles=Nv, num_vertices_max=V, syssize_x_max=box[0], syssize_x_min=box[1],
              syssize_y_max=box[2], syssize_y_min=box[3], syssize_z_max=box[4], syssize_z_min=box[5],
              num_part_min=W, num_part_max=Nv - 2)
    ref = oracle.RefVerlet(vp)
    s = {k: v.copy() for k, v in st.items()}
    for _ in range(10):
        ref.run(s)
    np.savez_compressed(HERE / "verlet.npz", dt=dt, box=np.array(box), W=W, n_max=Nv - 2,
                        **{"in_" + k: v for k, v in st.items()}, **{"out_" + k: v for k, v in s.items()})

    # broad phase: the reference's Linked_cell_hash in this interpreter, and MWDiem.py:808-811
    sys.path.insert(0, str(build_ref.REFERENCE_ROOT / "LIBRARIES"))
    import LIBRARY_Coarse_contact_detection as CCD

    class P:
        def __init__(self, i):
            self.particle_id = i

    n, Wb = 1200, 4
    com = np.zeros((n + Wb, 3))
    com[Wb:] = rng.uniform([-10, -10, -2], [10, 10, 25], size=(n, 3))
    com[:Wb] = rng.uniform(-3, 3, size=(Wb, 3))
    normals = rng.normal(size=(Wb, 3))
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    csx, csy, csz, nx, ny = 2.3, 2.4, 2.5, 9, 9
    xc = (com[:, 0] / csx).astype(int)
    yc = (com[:, 1] / csy).astype(int)
    zc = (com[:, 2] / csz).astype(int)
    keys = xc + yc * nx + zc * nx * ny
    rng_w = 6 * 1.2
    wall = []
    for k in range(Wb):
        for j in range(Wb, n + Wb):
            if abs(np.dot(normals[k], com[j] - com[k])) < rng_w:
                wall.append([j, k])
    cells = CCD.Linked_cell_hash([P(i) for i in range(n + Wb)], nx, ny, Wb, n + Wb, [], keys)
    np.savez_compressed(HERE / "broad.npz", com=com, normals=normals, cs=np.array([csx, csy, csz]),
                        nx=nx, ny=ny, W=Wb, wall_range=rng_w, keys=keys,
                        wall_pairs=np.array(wall, np.int32).reshape(-1, 2),
                        cell_pairs=np.array(cells, np.int32).reshape(-1, 2))
    print("contact pairs", inp["A_com"].shape[0], "collisions", int((r32["collision"] == 1).sum()),
          "wall pairs", len(wall), "cell pairs", len(cells))


if __name__ == "__main__":
    main()
