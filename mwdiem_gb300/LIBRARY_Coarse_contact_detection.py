"""Drop-in for ``LIBRARIES/LIBRARY_Coarse_contact_detection.py`` plus the inline broad-phase code
of ``MWDiem.py:808-816``.

* ``Linked_cell_hash(particle, numcells_x, numcells_y, num_part_min, num_part_max, pairstocheck,
  hashh_arr)`` appends the cell candidates to ``pairstocheck`` and returns it
  (``LIBRARY_Coarse_contact_detection.py:84-155``).  The appended pairs are the reference's pairs
  exactly, same-cell pairs oriented in CPython set order; they are listed cell by cell instead of in
  the dict's insertion order.
* ``cell_keys`` is ``MWDiem.py:813-816``; ``wall_candidates`` is ``MWDiem.py:808-811``.
* ``linked_cell_pairs`` / ``wall_pairs`` are the device-array forms (CUDA tensors in and out).

All of them run on the GPU (``libmwdem.so``).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _dev
from ._lib import check, lib


def _run_pairs(call, cap):
    n_out = torch.zeros(1, dtype=torch.int64, device="cuda")
    while True:
        pairs = torch.empty((max(cap, 1), 2), dtype=torch.int32, device="cuda")
        call(pairs, cap, n_out)
        torch.cuda.current_stream().synchronize()
        n = int(n_out.item())
        if n < cap or cap == 0 and n == 0:
            return pairs[:n]
        if n == cap:
            # may have been truncated: the total is clamped to cap; grow and retry once more
            cap = cap * 2
            continue
        cap = n


def linked_cell_pairs(keys, num_part_min, num_part_max, numcells_x, numcells_y, cap=None):
    """Cell candidates as an (P,2) int32 CUDA tensor; ``keys`` indexed by particle row."""
    _dev.require_cuda()
    k = keys if _dev.is_device(keys) else torch.from_numpy(np.ascontiguousarray(np.asarray(keys).reshape(-1),
                                                                                  dtype=np.int64)).cuda()
    k = k.reshape(-1).to(torch.int64).contiguous()
    rows = max(0, int(num_part_max) - int(num_part_min))
    cap = int(cap) if cap else max(1024, 16 * rows)
    s = _dev.stream_handle()

    def call(pairs, c, n_out):
        check(lib().mwd_linked_cell_hash(int(num_part_min), int(num_part_max), k.data_ptr(), int(numcells_x),
                                         int(numcells_y), pairs.data_ptr(), c, n_out.data_ptr(), None, s))

    return _run_pairs(call, cap)


def Linked_cell_hash(particle, numcells_x, numcells_y, num_part_min, num_part_max, pairstocheck, hashh_arr):
    """``LIBRARY_Coarse_contact_detection.py:84``.  ``particle[i].particle_id`` names row i."""
    pairs = linked_cell_pairs(hashh_arr, num_part_min, num_part_max, numcells_x, numcells_y).cpu().numpy()
    ids = None
    if particle is not None:
        ids = np.array([getattr(particle[i], "particle_id", i) if particle[i] is not None else i
                        for i in range(len(particle))], dtype=np.int64)
        if np.array_equal(ids, np.arange(len(ids))):
            ids = None
    if ids is not None:
        pairs = ids[pairs]
    pairstocheck.extend(pairs.tolist())
    return pairstocheck


def cell_keys(center_of_mass_arr, cellsize_x, cellsize_y, cellsize_z, numcells_x, numcells_y):
    """``MWDiem.py:813-816``: int64 keys of every row (truncation toward zero of the FP64 quotient)."""
    _dev.require_cuda()
    c = center_of_mass_arr if _dev.is_device(center_of_mass_arr) else torch.from_numpy(
        np.ascontiguousarray(center_of_mass_arr, dtype=np.float64)).cuda()
    c = c.to(torch.float64).contiguous()
    keys = torch.empty(c.shape[0], dtype=torch.int64, device=c.device)
    check(lib().mwd_cell_keys(int(c.shape[0]), c.data_ptr(), float(cellsize_x), float(cellsize_y),
                              float(cellsize_z), int(numcells_x), int(numcells_y), keys.data_ptr(),
                              _dev.stream_handle()))
    return keys if _dev.is_device(center_of_mass_arr) else keys.cpu().numpy()


def wall_pairs(center_of_mass_arr, wall_normals, wall_centers, num_particles_wall, num_part_lo, num_part_hi, rng,
               cap=None):
    """``MWDiem.py:808-811`` on the GPU: (P,2) int32 CUDA tensor of [particle, wall], wall-major."""
    _dev.require_cuda()

    def dev(x):
        return x.to(torch.float64).contiguous() if _dev.is_device(x) else torch.from_numpy(
            np.ascontiguousarray(x, dtype=np.float64)).cuda()

    c, wn, wc = dev(center_of_mass_arr), dev(wall_normals), dev(wall_centers)
    W, lo, hi = int(num_particles_wall), int(num_part_lo), int(num_part_hi)
    cap = int(cap) if cap else max(1024, W * max(0, hi - lo))
    s = _dev.stream_handle()

    def call(pairs, cp, n_out):
        check(lib().mwd_wall_pairs(W, lo, hi, c.data_ptr(), wn.data_ptr(), wc.data_ptr(), float(rng),
                                   pairs.data_ptr(), cp, n_out.data_ptr(), None, s))

    return _run_pairs(call, cap)


def wall_candidates(particle, center_of_mass_arr, num_particles_wall, num_particles_temp, max_particlesize,
                    pairs_to_check=None):
    """``MWDiem.py:807-811`` as a function: appends [j, k] for |n_k.(c_j - c_k)| < 6 max_particlesize."""
    W = int(num_particles_wall)
    wn = np.array([np.asarray(particle[k].normvec, dtype=np.float64) for k in range(W)]).reshape(W, 3)
    wc = np.array([np.asarray(particle[k].center_of_mass, dtype=np.float64) for k in range(W)]).reshape(W, 3)
    out = pairs_to_check if pairs_to_check is not None else []
    if W == 0:
        return out
    p = wall_pairs(center_of_mass_arr, wn, wc, W, W, num_particles_temp, 6 * max_particlesize)
    out.extend(p.cpu().numpy().tolist())
    return out
