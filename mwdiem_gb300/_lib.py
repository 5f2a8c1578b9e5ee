"""ctypes binding of ``libmwdem.so`` (C ABI in ``include/mwdem.h``).

The library is the only compute path: if it cannot be loaded the import of any GPU entry point
raises.  Structures below mirror the header field for field.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

MWD_OK = 0
MWD_ERR_INVALID = 1
MWD_ERR_CUDA = 2
MWD_ERR_UNSUPPORTED = 3
MWD_ERR_NOMEM = 4

ST_EPA_NOCONV = 1
ST_EPA_OVERFLOW = 2
ST_GJK_NOCONV = 4
ST_PAIR_OVERFLOW = 8
ST_CELL_RANGE = 16
ST_CELL_CROWDED = 32
ST_BAD_SHAPE = 64
ST_DEGENERATE_FACE = 128
ST_LOG_OVERFLOW = 256
ST_FLY_RESET = 512
ST_HIST_OVERFLOW = 1024

EPA_FACE_CAP = 128
EPA_COUNT_INTS = 256  # ints of mwd_work.epa_count: EPA record count, work queue, overflow retry list
EPA_VERT_CAP = 32
HULL_CAP = 64
CELL_CAP = 306
NOALLOC_MAX_PAIRS = 1 << 18

STATUS_NAMES = {ST_EPA_NOCONV: "EPA_NOCONV", ST_EPA_OVERFLOW: "EPA_OVERFLOW", ST_GJK_NOCONV: "GJK_NOCONV",
                ST_PAIR_OVERFLOW: "PAIR_OVERFLOW", ST_CELL_RANGE: "CELL_RANGE", ST_CELL_CROWDED: "CELL_CROWDED",
                ST_BAD_SHAPE: "BAD_SHAPE", ST_DEGENERATE_FACE: "DEGENERATE_FACE", ST_LOG_OVERFLOW: "LOG_OVERFLOW",
                ST_FLY_RESET: "FLY_RESET", ST_HIST_OVERFLOW: "HIST_OVERFLOW"}


class MwdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libmwdem error {code}: {msg}")
        self.code = code


class ContactParams(C.Structure):
    _fields_ = [("Kn", C.c_double), ("en", C.c_double), ("et", C.c_double), ("mu", C.c_double),
                ("Kn_wall", C.c_double), ("en_wall", C.c_double), ("et_wall", C.c_double),
                ("mu_wall", C.c_double), ("dt", C.c_double), ("n_wall", C.c_int32),
                ("hist_mode", C.c_int32), ("lanes", C.c_int32), ("deterministic", C.c_int32),
                ("law", C.c_int32), ("pad", C.c_int32)]


CELL_TABLE_AUTO = 0
CELL_TABLE_DENSE = 1
CELL_TABLE_COMPRESSED = 2

LAW_REFERENCE = 0
LAW_PHYSICAL = 1


class Material(C.Structure):
    _fields_ = [("Kn_f", C.c_float), ("mu_f", C.c_float), ("Gn", C.c_float), ("ln_et", C.c_float),
                ("dt_f", C.c_float), ("ln_en", C.c_float), ("Xn", C.c_float), ("Xt", C.c_float),
                ("mu", C.c_double), ("inv_mu", C.c_double), ("KtA", C.c_double), ("physical", C.c_int32),
                ("inv_mu_hi", C.c_float), ("inv_mu_lo", C.c_float), ("KtA_hi", C.c_float), ("KtA_lo", C.c_float),
                ("pad", C.c_int32)]


class VerletParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("box", C.c_double * 6), ("n_min", C.c_int32), ("n_max", C.c_int32),
                ("V", C.c_int32), ("pad", C.c_int32)]


_P = C.c_void_p


class State(C.Structure):
    _fields_ = [(n, _P) for n in ("pos", "dx_all", "vel", "vel_half", "w_half_bf", "w_bf", "w", "q", "q_half",
                                  "q_all", "q_acc", "force", "torque", "ext_force", "ext_torque", "inertia",
                                  "inv_inertia", "info", "wall_normal", "vert_off", "body_verts", "world_verts")] + \
               [("n", C.c_int32), ("n_verts", C.c_int32), ("max_verts", C.c_int32), ("pad", C.c_int32),
                ("vert_owner", _P), ("xform", _P)]


class Scene(C.Structure):
    _fields_ = [("cs", C.c_double * 3), ("box", C.c_double * 6), ("dt", C.c_double), ("wall_range", C.c_double),
                ("nx", C.c_int64), ("ny", C.c_int64), ("key_min", C.c_int64), ("n_keys", C.c_int64),
                ("cell_base", C.c_int64), ("row_begin", C.c_int32), ("wall_end", C.c_int32),
                ("row_end", C.c_int32), ("pad", C.c_int32), ("law", ContactParams), ("mat", Material * 2),
                ("inv_cs", C.c_float * 3), ("pad2", C.c_int32)]


class Work(C.Structure):
    _fields_ = [(n, _P) for n in ("cell_count", "cell_start", "cell_of", "sorted", "pair_count", "pairs",
                                  "scan_tmp", "n_pairs", "status", "collision")] + \
               [("work_counters", _P), ("epa_count", _P), ("epa_rec", _P),
                ("epa_cap", C.c_int64), ("sorted_pos", _P), ("sorted_cell", _P), ("cull_pairs", C.c_int32),
                ("cell_table", C.c_int32), ("total_cells", C.c_int64),
                ("pair_cap", C.c_int64), ("face_ids", _P), ("deterministic", C.c_int32),
                ("pad2", C.c_int32), ("det_scratch", _P), ("hist_cap", C.c_int64), ("hist_keys", _P),
                ("hist_vals", _P), ("hist_parity", _P), ("inlet", _P)]


INFO_INACTIVE = 1 << 30


class Inlet(C.Structure):
    _fields_ = [("period", C.c_int32), ("per_spawn", C.c_int32), ("row_end", C.c_int32), ("pad", C.c_int32),
                ("next_row", _P), ("step", _P), ("spawn_pos", _P)]


DIFF_ROW = 32
# FP64 state row of the differentiable step (include/mwdem.h): slices by name
DIFF_SLICES = {"c": slice(0, 3), "v": slice(3, 6), "v_half": slice(6, 9), "w_half_bf": slice(9, 12),
               "w_bf": slice(12, 15), "w": slice(15, 18), "q": slice(18, 22), "q_half": slice(22, 26),
               "q_acc": slice(26, 30)}


class ContactRec(C.Structure):
    _fields_ = [("A", C.c_int32), ("B", C.c_int32), ("fa", C.c_int32 * 3), ("fb", C.c_int32 * 3)]


class Diff(C.Structure):
    _fields_ = [("n", C.c_int32), ("n_particles", C.c_int32), ("n_steps", C.c_int32), ("ckpt_every", C.c_int32),
                ("contact_point", C.c_int32), ("pad", C.c_int32), ("dt", C.c_double), ("box", C.c_double * 6)] + \
               [(n, _P) for n in ("inertia", "inv_inertia", "ext", "body_verts", "vert_off", "info", "law", "F", "T",
                                  "rec")] + \
               [("rec_cap", C.c_int64)] + \
               [(n, _P) for n in ("step_off", "step_count", "t_dev", "sync", "com", "ckpt", "status", "t_base")]


_lock = threading.Lock()
_handle = None


def lib():
    """Load (building first if needed) ``libmwdem.so``.  Raises if it cannot be built or loaded."""
    global _handle
    if _handle is not None:
        return _handle
    with _lock:
        if _handle is not None:
            return _handle
        path = _build.build()
        h = C.CDLL(str(path))
        i32, i64, d = C.c_int32, C.c_int64, C.c_double
        sig = {
            "mwd_last_error": (C.c_char_p, []),
            "mwd_version": (C.c_int, []),
            "mwd_num_sms": (i32, []),
            "mwd_scan_tmp_ints": (i64, [i64]),
            "mwd_cell_table": (i32, [i64, i64, i32]),
            "mwd_integrate_kernels": (i32, [i64]),
            "mwd_cell_table_ints": (i32, [i64, i64, i32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
            "mwd_derive_material": (C.c_int, [C.POINTER(ContactParams), C.POINTER(Material)]),
            "mwd_contact_pairs": (C.c_int, [i64, i32, i32] + [_P] * 20 + [C.POINTER(ContactParams), _P, _P, _P]),
            "mwd_verlet_ref": (C.c_int, [i32] + [_P] * 16 + [C.POINTER(VerletParams), _P, _P]),
            "mwd_cell_keys": (C.c_int, [i32, _P, d, d, d, i64, i64, _P, _P]),
            "mwd_wall_pairs": (C.c_int, [i32, i32, i32, _P, _P, _P, d, _P, i64, _P, _P, _P]),
            "mwd_linked_cell_hash": (C.c_int, [i32, i32, _P, i64, i64, _P, i64, _P, _P, _P]),
            "mwd_broadphase": (C.c_int, [C.POINTER(State), _P, _P, i32, C.POINTER(Work), _P]),
            "mwd_narrow_force": (C.c_int, [C.POINTER(State), _P, C.POINTER(Work), i32, _P]),
            "mwd_integrate": (C.c_int, [C.POINTER(State), _P, _P, _P]),
            "mwd_step": (C.c_int, [C.POINTER(State), _P, _P, i32, C.POINTER(Work), i32, i32, _P]),
            "mwd_refresh_vertices": (C.c_int, [C.POINTER(State), _P]),
            "mwd_integrate_rows": (C.c_int, [C.POINTER(State), _P, _P, _P]),
            "mwd_world_vertices": (C.c_int, [C.POINTER(State), _P]),
            "mwd_integrate_rows_mirror": (C.c_int, [C.POINTER(State), _P, _P, _P, _P, i64, _P]),
            "mwd_host_mapped": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
            "mwd_probe_fp32": (C.c_int, [i32, _P, C.POINTER(C.c_double), _P]),
            "mwd_contact_pairs_noalloc": (C.c_int, [i64, i32, i32] + [_P] * 20 +
                                          [C.POINTER(ContactParams), _P, _P, _P]),
            "mwd_det_scratch_bytes": (i64, [i32, i64]),
            "mwd_inlet_step": (C.c_int, [C.POINTER(State), C.POINTER(Inlet), _P]),
            "mwd_diff_collect": (C.c_int, [C.POINTER(Diff), C.POINTER(Work), _P]),
            "mwd_diff_force": (C.c_int, [C.POINTER(Diff), _P, i32, _P]),
            "mwd_diff_integrate": (C.c_int, [C.POINTER(Diff), _P, _P, _P, C.POINTER(State), i32, _P]),
            "mwd_diff_mirror": (C.c_int, [C.POINTER(Diff), _P, C.POINTER(State), _P]),
            "mwd_diff_adjoint": (C.c_int, [C.POINTER(Diff), _P, _P, i32, _P, _P, _P, _P, _P, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _handle = h
        return h


EXPORTED = ("mwd_last_error", "mwd_version", "mwd_num_sms", "mwd_scan_tmp_ints", "mwd_cell_table", "mwd_cell_table_ints", "mwd_integrate_kernels",
            "mwd_derive_material",
            "mwd_contact_pairs", "mwd_verlet_ref", "mwd_cell_keys", "mwd_wall_pairs", "mwd_linked_cell_hash",
            "mwd_broadphase", "mwd_narrow_force", "mwd_integrate", "mwd_step", "mwd_refresh_vertices",
            "mwd_integrate_rows", "mwd_world_vertices", "mwd_integrate_rows_mirror", "mwd_host_mapped", "mwd_probe_fp32",
            "mwd_contact_pairs_noalloc", "mwd_det_scratch_bytes", "mwd_inlet_step", "mwd_diff_collect", "mwd_diff_force", "mwd_diff_integrate",
            "mwd_diff_mirror", "mwd_diff_adjoint")


def check(rc: int):
    if rc != MWD_OK:
        msg = lib().mwd_last_error()
        raise MwdError(rc, msg.decode() if msg else "")


def lib_path() -> Path:
    return _build.LIB


def status_names(word: int):
    return [name for bit, name in STATUS_NAMES.items() if word & bit]
