"""Drop-in for the reference's VTK writer (LIBRARIES/LIBRARY_Vtk_creator.py:3-41).

``Vtk_creator`` has the reference's signature and effects: it applies each particle's accumulated
rotation and displacement (``quaternion_all_arr``, ``dx_all_arr``) to its vertices, resets those
rows to identity / zero, writes the particles' hull vertices and triangular faces as legacy-VTK ASCII
POLYDATA, and returns the two arrays.  For the device-resident state, ``mwdiem_gb300.writers`` writes
the same format from an asynchronous snapshot.
"""
from __future__ import annotations

import numpy as np


def Vtk_creator(particle, filename, num_part_min, num_part_max, quaternion_all_arr, dx_all_arr):
    for i in range(num_part_min, num_part_max):
        particle[i].quaternion_all = quaternion_all_arr[i].copy()
        particle[i].dx_all = dx_all_arr[i].copy()
        particle[i].Rotator_quaternion_all()
        particle[i].Translate_all()
        quaternion_all_arr[i] = np.array([1, 0, 0, 0])
        dx_all_arr[i] = np.array([0, 0, 0])
    rows = range(num_part_min, num_part_max)
    lines = ["# vtk DataFile Version 2.0\n", "# kata\n", "ASCII\n", "DATASET POLYDATA\n"]
    num_points = sum(particle[i].num_vertices for i in rows)
    lines.append("POINTS\t" + str(num_points) + "\tfloat\n")
    for i in rows:
        for j in range(particle[i].num_vertices):
            c = particle[i].vertices[j].vertex_coo
            lines.append(str(c[0]) + "\t" + str(c[1]) + "\t" + str(c[2]) + "\n")
    num_faces = sum(particle[i].num_faces for i in rows)
    lines.append("POLYGONS\t" + str(num_faces) + "\t" + str(num_faces * 4) + "\n")
    base = 0
    for i in rows:
        for j in range(particle[i].num_faces):
            f = particle[i].faces[j].face_vertices_id
            lines.append("3\t" + str(f[0] + base) + "\t" + str(f[1] + base) + "\t" + str(f[2] + base) + "\n")
        base += particle[i].num_vertices
    with open(filename, "w") as out:
        out.writelines(lines)
    return quaternion_all_arr, dx_all_arr
