"""ctypes front end of the oracle (``liboracle.so``) and of the host-compiled reference kernels
(``oracle/_ref``).

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU reference arm -- never by the product package ``mwdiem_gb300``.

Array conventions are the reference's own (``MWDiem.py:847-903`` for the per-pair contact inputs,
``MWDiem.py:603-631`` for the integrator state).
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
if str(HERE) not in sys.path:
    sys.path.insert(0, str(HERE))
import build as _build  # noqa: E402
import build_ref as _build_ref  # noqa: E402

DIAG = 19        # per-pair diagnostics: depth, normal(3), cpA(3), cpB(3), F(3), TA(3), TB(3)
NCOUNT = 10      # per-pair counters: support calls, GJK tetra iterations, EPA iterations, face ids (6), faces used
ST_EPA_NOCONV = 1
ST_EPA_OVERFLOW = 2
ST_GJK_NOCONV = 4


class ContactParams(C.Structure):
    _fields_ = [("Kn", C.c_double), ("en", C.c_double), ("et", C.c_double), ("mu", C.c_double),
                ("Kn_wall", C.c_double), ("en_wall", C.c_double), ("et_wall", C.c_double),
                ("mu_wall", C.c_double), ("dt", C.c_double), ("n_wall", C.c_int),
                ("hist_stride4", C.c_int), ("face_cap", C.c_int), ("physical", C.c_int)]


class VerletParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("box", C.c_double * 6), ("n_min", C.c_int), ("n_max", C.c_int),
                ("V", C.c_int), ("physical", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(_build.build()))
        P = C.c_void_p
        for name in ("orc_contact_f32", "orc_contact_f64"):
            f = getattr(_lib, name)
            f.restype = None
            f.argtypes = [C.c_int, C.c_int] + [P] * 20 + [C.POINTER(ContactParams), P, P, P, P, P]
        _lib.orc_verlet_f64.restype = C.c_int
        _lib.orc_verlet_f64.argtypes = [C.c_int] + [P] * 16 + [C.POINTER(VerletParams)]
        _lib.orc_cell_keys.restype = None
        _lib.orc_cell_keys.argtypes = [C.c_int, P, C.c_double, C.c_double, C.c_double, C.c_int64, C.c_int64, P]
        _lib.orc_wall_pairs.restype = C.c_int64
        _lib.orc_wall_pairs.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, C.c_double, P, C.c_int64]
        _lib.orc_linked_cell_hash.restype = C.c_int64
        _lib.orc_linked_cell_hash.argtypes = [C.c_int, C.c_int, P, C.c_int64, C.c_int64, P, C.c_int64]
        _lib.orc_pyset_order.restype = C.c_int
        _lib.orc_pyset_order.argtypes = [C.c_int, P, P]
        _lib.orc_face_capacity.restype = C.c_int
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


CONTACT_INPUTS = ("A_com", "B_com", "A_verts", "B_verts", "A_vel", "B_vel", "A_angvel", "B_angvel",
                  "A_nv", "B_nv", "A_id", "B_id", "hist", "qA", "qB", "IsA", "IsB")


def contact_params(p: dict, hist_stride4=False, face_cap=0, physical=False) -> ContactParams:
    return ContactParams(float(p["Kn"]), float(p["en"]), float(p["et"]), float(p["mu"]),
                         float(p["Kn_wall"]), float(p["en_wall"]), float(p["et_wall"]), float(p["mu_wall"]),
                         float(p["timestep"]), int(p["num_particles_wall"]), int(bool(hist_stride4)),
                         int(face_cap), int(bool(physical)))


def contact(inp: dict, params: dict, n_particles: int, precision="f32", force=None, torque=None,
            hist_stride4=False, face_cap=0, inv_mass=None):
    """Run the oracle narrow phase + force over per-pair arrays.

    ``inp`` holds the arrays named in ``CONTACT_INPUTS`` (shapes as in ``MWDiem.py:887-903``).
    ``inv_mass=(imA, imB)``, per-pair inverse masses (0 for a wall side), selects the physical-mass
    contact law instead of the reference's.
    Returns a dict with force, torque (n_particles,3), hist (P,4), collision (P,), diag (P,19),
    status (P,), counters (P,9).
    """
    dt = np.float32 if precision == "f32" else np.float64
    n = int(np.asarray(inp["A_com"]).shape[0])
    V = int(np.asarray(inp["A_verts"]).shape[1]) if n else 1
    a = {k: _c(inp[k], np.int32 if k in ("A_nv", "B_nv", "A_id", "B_id") else dt) for k in CONTACT_INPUTS}
    hist = a["hist"].copy()
    F = np.zeros((n_particles, 3), dt) if force is None else _c(force, dt).copy()
    T = np.zeros((n_particles, 3), dt) if torque is None else _c(torque, dt).copy()
    coll = np.zeros(n, np.int32)
    diag = np.zeros((n, DIAG), dt)
    status = np.zeros(n, np.int32)
    counters = np.zeros((n, NCOUNT), np.int32)
    prm = contact_params(params, hist_stride4, face_cap, physical=inv_mass is not None)
    imA = imB = None
    if inv_mass is not None:
        imA, imB = (_c(x, dt) for x in inv_mass)
    fn = lib().orc_contact_f32 if precision == "f32" else lib().orc_contact_f64
    if n:
        fn(n, V, _p(a["A_com"]), _p(a["B_com"]), _p(a["A_verts"]), _p(a["B_verts"]), _p(a["A_vel"]),
           _p(a["B_vel"]), _p(a["A_angvel"]), _p(a["B_angvel"]), _p(a["A_nv"]), _p(a["B_nv"]),
           _p(a["A_id"]), _p(a["B_id"]), _p(hist), _p(F), _p(T), _p(a["qA"]), _p(a["qB"]), _p(a["IsA"]),
           _p(a["IsB"]), _p(coll), C.byref(prm), _p(diag), _p(status), _p(counters), _p(imA), _p(imB))
    return dict(force=F, torque=T, hist=hist, collision=coll, diag=diag, status=status, counters=counters)


VERLET_ARRAYS = ("v", "v12", "w12bf", "q12", "q", "qall", "wbf", "w", "F", "T", "verts", "com", "mass",
                 "Iinv", "I", "dxall")


def verlet_params(dt, box, n_min, n_max, V, physical=False) -> VerletParams:
    vp = VerletParams()
    vp.dt = float(dt)
    for i in range(6):
        vp.box[i] = float(box[i])
    vp.n_min, vp.n_max, vp.V = int(n_min), int(n_max), int(V)
    vp.physical = int(bool(physical))
    return vp


def verlet_f64(state: dict, dt, box, n_min, n_max, physical=False) -> int:
    """One FP64 integrator step in place over reference-layout arrays; returns resets.
    ``physical``: the vertices turn by the step's rotation (the physical contact law's integrator)
    instead of by the whole orientation as in the reference."""
    for k in VERLET_ARRAYS:
        a = state[k]
        assert a.dtype == np.float64 and a.flags.c_contiguous, k
    N = state["v"].shape[0]
    V = state["verts"].shape[1]
    prm = verlet_params(dt, box, n_min, n_max, V, physical)
    return lib().orc_verlet_f64(N, *[_p(state[k]) for k in VERLET_ARRAYS], C.byref(prm))


def cell_keys(com, csx, csy, csz, nx, ny):
    com = _c(com, np.float64)
    keys = np.zeros(com.shape[0], np.int64)
    lib().orc_cell_keys(com.shape[0], _p(com), csx, csy, csz, int(nx), int(ny), _p(keys))
    return keys


def wall_pairs(n_wall, n_lo, n_hi, com, wall_n, wall_c, rng):
    com = _c(com, np.float64)
    wall_n = _c(wall_n, np.float64)
    wall_c = _c(wall_c, np.float64)
    cap = max(1, n_wall * max(0, n_hi - n_lo))
    out = np.zeros((cap, 2), np.int32)
    n = lib().orc_wall_pairs(n_wall, n_lo, n_hi, _p(com), _p(wall_n), _p(wall_c), float(rng), _p(out), cap)
    return out[:n].copy()


def linked_cell_hash(n_lo, n_hi, keys, nx, ny, cap=None):
    keys = _c(keys, np.int64)
    if cap is None:
        cap = 1 << 16
    while True:
        out = np.zeros((cap, 2), np.int32)
        n = lib().orc_linked_cell_hash(n_lo, n_hi, _p(keys), int(nx), int(ny), _p(out), cap)
        if n <= cap:
            return out[:n].copy()
        cap = int(n)


def pyset_order(ids):
    ids = _c(ids, np.int64)
    out = np.zeros_like(ids)
    rc = lib().orc_pyset_order(len(ids), _p(ids), _p(out))
    if rc != 0:
        raise ValueError("set too large for the emulation")
    return out


# ---------------------------------------------------------------- host-compiled reference kernels

class RefContact:
    """The reference's ``contact_detection`` compiled for the host with ``params`` baked in."""

    def __init__(self, params: dict, variant="f32"):
        self.params = dict(params)
        self.variant = variant
        self.dtype = np.float64 if variant == "f64" else np.float32
        self.lib = C.CDLL(str(_build_ref.ensure_built("contact", self.params, variant)))
        P = C.c_void_p
        self.lib.ref_contact_run.restype = None
        self.lib.ref_contact_run.argtypes = [C.c_int, C.c_int, C.c_int] + [P] * 22

    def run(self, inp: dict, n_particles: int, nthreads=1, snapshot=True, force=None, torque=None):
        dt = self.dtype
        n = int(np.asarray(inp["A_com"]).shape[0])
        a = {k: _c(inp[k], np.int32 if k in ("A_nv", "B_nv", "A_id", "B_id") else dt) for k in CONTACT_INPUTS}
        V = a["A_verts"].shape[1] if n else 1
        assert V == int(self.params["num_vertices_max"]), "rendered for another num_vertices_max"
        hist = a["hist"].copy()
        F = np.zeros((n_particles, 3), dt) if force is None else _c(force, dt).copy()
        T = np.zeros((n_particles, 3), dt) if torque is None else _c(torque, dt).copy()
        coll = np.zeros(n, np.int32)
        pid = np.zeros((n, 2), np.int32)
        scratch = np.zeros((max(n, 1), 4), dt)
        if n:
            self.lib.ref_contact_run(n, int(nthreads), int(bool(snapshot)), _p(a["A_com"]), _p(a["B_com"]),
                                     _p(a["A_verts"]), _p(a["B_verts"]), _p(a["A_vel"]), _p(a["B_vel"]),
                                     _p(a["A_angvel"]), _p(a["B_angvel"]), _p(a["A_nv"]), _p(a["B_nv"]),
                                     _p(a["A_id"]), _p(a["B_id"]), _p(hist), _p(F), _p(T), _p(a["qA"]),
                                     _p(a["qB"]), _p(pid), _p(coll), _p(a["IsA"]), _p(a["IsB"]), _p(scratch))
        return dict(force=F, torque=T, hist=hist, collision=coll)


class RefVerlet:
    """The reference's ``Verlet`` kernel compiled for the host with ``params`` baked in
    (keys as ``gpu_Verlet.py:63-73``)."""

    def __init__(self, params: dict):
        self.params = dict(params)
        self.lib = C.CDLL(str(_build_ref.ensure_built("verlet", self.params, "f32")))
        P = C.c_void_p
        self.lib.ref_verlet_run.restype = None
        self.lib.ref_verlet_run.argtypes = [C.c_int, C.c_int] + [P] * 16

    def run(self, state: dict, nthreads=1):
        for k in VERLET_ARRAYS:
            a = state[k]
            assert a.dtype == np.float64 and a.flags.c_contiguous, k
        n = state["v"].shape[0]
        self.lib.ref_verlet_run(n, int(nthreads), *[_p(state[k]) for k in VERLET_ARRAYS])


def ref_available():
    return _build_ref.reference_available()
