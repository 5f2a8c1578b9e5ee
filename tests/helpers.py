"""Seeded synthetic inputs shared by the tests, the golden-fixture script and the benchmark."""
from __future__ import annotations

import numpy as np

from mwdiem_gb300 import scene as scene_mod
from mwdiem_gb300 import shapes

CONTACT_PARAMS = dict(Kn=1e5, en=0.372, et=0.372, mu=0.5, Kn_wall=1e5, en_wall=0.372, et_wall=0.372,
                      mu_wall=0.5, num_vertices_max=32, num_particles_wall=4, timestep=5e-5)


def hull_pool(rng, n_shapes, n_min, n_max, r_min=0.8, r_max=1.2):
    return [shapes.random_hull(rng, n_min, n_max, r_min, r_max) for _ in range(n_shapes)]


def make_pairs(P, seed, V=32, n_min=8, n_max=32, dist=(0.5, 2.2), vel=0.5, angvel=2.0, pool=64, box=50.0,
               unique_ids=True, n_particles=None):
    """Per-pair arrays in the reference's layout (MWDiem.py:847-903): random hulls of n_min..n_max
    points on a sphere of radius U[0.8,1.2], random orientation, centre distance
    U[dist]*(r1+r2)/2 along a random direction.  With unique_ids every particle appears in one pair
    only, so float atomics have a single term per particle."""
    rng = np.random.default_rng(seed)
    shp = hull_pool(rng, pool, n_min, min(n_max, V))
    N = n_particles or (2 * P + 8)
    A_com = np.zeros((P, 3)); B_com = np.zeros((P, 3))
    A_v = np.zeros((P, V, 3)); B_v = np.zeros((P, V, 3))
    A_nv = np.zeros(P, np.int32); B_nv = np.zeros(P, np.int32)
    IsA = np.zeros(P); IsB = np.zeros(P)
    ia = rng.integers(len(shp), size=P)
    ib = rng.integers(len(shp), size=P)
    for p in range(P):
        sa, sb = shp[ia[p]], shp[ib[p]]
        qa, qb = shapes.random_quaternion(rng), shapes.random_quaternion(rng)
        ca = rng.uniform(-box, box, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        cb = ca + d * rng.uniform(*dist) * (sa.radius + sb.radius) / 2
        A_com[p] = ca
        B_com[p] = cb
        A_v[p, :sa.num_vertices] = ca + sa.vertices @ shapes.quat_to_matrix(qa).T
        B_v[p, :sb.num_vertices] = cb + sb.vertices @ shapes.quat_to_matrix(qb).T
        A_nv[p] = sa.num_vertices
        B_nv[p] = sb.num_vertices
        IsA[p] = sa.inertia_size
        IsB[p] = sb.inertia_size
    if unique_ids:
        ids = rng.permutation(N)[:2 * P].astype(np.int32)
        A_id, B_id = ids[:P], ids[P:]
    else:
        A_id = rng.integers(N, size=P).astype(np.int32)
        B_id = ((A_id + 1 + rng.integers(N - 1, size=P)) % N).astype(np.int32)
    inp = dict(A_com=A_com, B_com=B_com, A_verts=A_v, B_verts=B_v,
               A_vel=rng.normal(size=(P, 3)) * vel, B_vel=rng.normal(size=(P, 3)) * vel,
               A_angvel=rng.normal(size=(P, 3)) * angvel, B_angvel=rng.normal(size=(P, 3)) * angvel,
               A_nv=A_nv, B_nv=B_nv, A_id=A_id, B_id=B_id, hist=np.zeros((P, 4)),
               qA=np.array([shapes.random_quaternion(rng) for _ in range(P)]).reshape(P, 4),
               qB=np.array([shapes.random_quaternion(rng) for _ in range(P)]).reshape(P, 4), IsA=IsA, IsB=IsB)
    return {k: (v.astype(np.float32) if v.dtype == np.float64 else v) for k, v in inp.items()}, N


def cube_pair_kat(depth=0.1, V=8, lateral=(0.05, 0.03)):
    """Two unit cubes overlapping by `depth` along x (the known-answer case |F| = Kn * depth).

    B is also shifted sideways by `lateral` (y, z): with lateral=(0, 0) the two cubes are exactly
    aligned and the reference's EPA starts from a degenerate polytope whose four faces all fail the
    inside test, returning depth 1e30 and a NaN normal (reproduced, not corrected)."""
    c = shapes.cube(1.0)
    off = np.array([1.0 - depth, lateral[0], lateral[1]])
    A = c.vertices.copy()
    B = c.vertices + off
    inp = dict(A_com=np.zeros((1, 3)), B_com=off[None].copy(),
               A_verts=np.zeros((1, V, 3)), B_verts=np.zeros((1, V, 3)),
               A_vel=np.zeros((1, 3)), B_vel=np.zeros((1, 3)), A_angvel=np.zeros((1, 3)), B_angvel=np.zeros((1, 3)),
               A_nv=np.array([8], np.int32), B_nv=np.array([8], np.int32), A_id=np.array([0], np.int32),
               B_id=np.array([1], np.int32), hist=np.zeros((1, 4)), qA=np.array([[1.0, 0, 0, 0]]),
               qB=np.array([[1.0, 0, 0, 0]]), IsA=np.array([c.inertia_size]), IsB=np.array([c.inertia_size]))
    inp["A_verts"][0, :8] = A
    inp["B_verts"][0, :8] = B
    return {k: (v.astype(np.float32) if v.dtype == np.float64 else v) for k, v in inp.items()}


def select(inp, idx):
    return {k: np.ascontiguousarray(np.asarray(v)[idx]) for k, v in inp.items()}


def make_verlet_state(N, V, seed, W=3, box=5.0, dt=1e-3):
    """Reference-layout FP64 integrator arrays (MWDiem.py:603-646) with random motion and loads."""
    rng = np.random.default_rng(seed)
    st = {k: np.zeros((N, 3)) for k in ("v", "v12", "w12bf", "wbf", "w", "F", "T", "com", "dxall")}
    for k in ("q12", "q", "qall"):
        st[k] = np.tile([1.0, 0, 0, 0], (N, 1))
    st["verts"] = np.zeros((N, V, 3))
    st["mass"] = np.zeros(N)
    st["Iinv"] = np.zeros((N, 3, 3))
    st["I"] = np.zeros((N, 3, 3))
    for i in range(N):
        s = shapes.random_hull(rng, 8, min(V, 24))
        c = rng.uniform(-box + 1, box - 1, 3)
        st["com"][i] = c
        st["verts"][i, :s.num_vertices] = c + s.vertices
        st["mass"][i] = s.mass
        st["I"][i] = s.inertia_bf
        st["Iinv"][i] = s.inertia_bf_inv
    st["v12"][:] = rng.normal(size=(N, 3))
    st["w12bf"][:] = rng.normal(size=(N, 3)) * 3
    st["w"][:] = rng.normal(size=(N, 3)) * 3
    st["F"][:] = rng.normal(size=(N, 3)) * 10
    st["T"][:] = rng.normal(size=(N, 3))
    # one particle leaves the box on its first step (fly-away reset, gpu_Verlet.cu:338-352)
    st["com"][W + 1] = [box - 0.01, 0, 0]
    st["v12"][W + 1] = [1e4, 0, 0]
    bx = (box, -box, box, -box, box, -box)
    return st, bx


def head_on_cubes(law, density=4.0, v=0.5):
    """Two unit cubes (mass 4) meeting head-on along x at relative speed 2v, no gravity, in a 10 x 10
    box."""
    # cube A turned so that a body diagonal points along +x, its corner hitting the face of the
    # axis-aligned cube B: a corner-face contact whose normal and contact point lie (almost) on the
    # line of centres, so the impact is normal and nearly torque-free (a face-face contact from one
    # contact point would tip the cubes)
    axis = np.array([0.0, 1.0, -1.0]) / np.sqrt(2.0)
    th = np.arccos(1.0 / np.sqrt(3.0))
    q = np.concatenate([[np.cos(th / 2)], np.sin(th / 2) * axis])
    A = scene_mod.body_from_shape(shapes.cube(1.0, density), q)
    B = scene_mod.body_from_shape(shapes.cube(1.0, density))
    walls = scene_mod.box_walls(10.0, 10.0, 10.0, 2.0)
    centres = np.array([[-0.01 - np.sqrt(3.0) / 2, 0.0, 5.0], [0.51, 0.02, 5.013]])
    return scene_mod.SceneSpec(walls=walls, bodies=[A, B], centres=centres,
                               velocities=np.array([[v, 0.0, 0.0], [-v, 0.0, 0.0]]), gravity=(0.0, 0.0, 0.0),
                               max_particlesize=float(2 * shapes.cube(1.0).radius), law=law)
