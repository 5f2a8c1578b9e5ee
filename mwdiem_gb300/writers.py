"""Output of the device-resident state in the reference's formats.

``VtkSnapshot(sim)`` writes the world-frame hulls of a scene as legacy-VTK ASCII POLYDATA, the format
of LIBRARIES/LIBRARY_Vtk_creator.py: the vertex table is copied on the device, then into pinned host
memory on a side stream (the steps keep running), and a host thread formats and writes the file once
that copy is done.
Each row's triangles come from the convex hull of its body-frame vertices, computed once.
``write_particle_data(sim, prefix, step, rows)`` appends one line per particle in the format of
LIBRARIES/LIBRARY_Write_particle_data.py: the force column is the contact-force accumulator as it
stands (between ``narrow_force`` and ``integrate`` it holds the step's contact force; the integrator
consumes it), and the spring and damping parts, which the device step does not keep, are 0.
"""
from __future__ import annotations

import threading

import numpy as np
import torch
from scipy.spatial import ConvexHull


class VtkSnapshot:
    def __init__(self, sim, scene=0):
        self.sim = sim
        rows = range(sim.layout.row_begin[scene], sim.layout.row_end[scene])
        off = sim.vert_off_host
        body = sim.t["body_verts"].cpu().numpy()
        self.rows = list(rows)
        self.v0, self.v1 = int(off[self.rows[0]]), int(off[self.rows[-1] + 1])
        faces = []
        base = 0
        cache = {}
        for r in self.rows:
            pts = body[off[r]:off[r + 1], :3]
            key = pts.tobytes()
            tri = cache.get(key)
            if tri is None:
                tri = ConvexHull(pts.astype(np.float64)).simplices.astype(np.int64)
                cache[key] = tri
            faces.append(tri + base)
            base += pts.shape[0]
        self.faces = np.concatenate(faces, 0) if faces else np.zeros((0, 3), np.int64)
        self.dev = torch.empty((self.v1 - self.v0, 4), dtype=torch.float32, device=sim.device)
        self.host = torch.empty((self.v1 - self.v0, 4), dtype=torch.float32).pin_memory()
        self.stream = torch.cuda.Stream()
        self.thread = None

    def write(self, filename):
        """Snapshot now (after the work already queued on the current stream) and write in the
        background; returns the writer thread."""
        self.wait()
        # a device copy on the caller's stream (later steps may then rewrite the vertex table), then the
        # copy to pinned host memory on a side stream
        self.dev.copy_(self.sim.t["world_verts"][self.v0:self.v1])
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream())
        self.stream.wait_event(ev)
        with torch.cuda.stream(self.stream):
            self.host.copy_(self.dev, non_blocking=True)
        done = torch.cuda.Event()
        done.record(self.stream)

        def run():
            done.synchronize()
            pts = self.host.numpy()[:, :3]
            with open(filename, "w") as out:
                out.write("# vtk DataFile Version 2.0\n# kata\nASCII\nDATASET POLYDATA\n")
                out.write("POINTS\t" + str(len(pts)) + "\tfloat\n")
                out.write("".join(f"{x}\t{y}\t{z}\n" for x, y, z in pts.tolist()))
                out.write("POLYGONS\t" + str(len(self.faces)) + "\t" + str(len(self.faces) * 4) + "\n")
                out.write("".join(f"3\t{a}\t{b}\t{c}\n" for a, b, c in self.faces.tolist()))

        self.thread = threading.Thread(target=run, daemon=True)
        self.thread.start()
        return self.thread

    def wait(self):
        if self.thread is not None:
            self.thread.join()
            self.thread = None


def write_particle_data(sim, prefix, step, rows):
    """One line per row in `rows` to <prefix><row>.dat (header at step 0): centre, velocity (|vz|),
    contact force, and zeros for the spring / damping parts."""
    pos = sim.t["pos"][rows, :3].cpu().numpy()
    vel = sim.t["vel"][rows, :3].cpu().numpy()
    frc = sim.t["force"][rows, :3].cpu().numpy()
    for k, r in enumerate(rows):
        path = f"{prefix}{r}.dat"
        with open(path, "w" if step == 0 else "a") as f_out:
            if step == 0:
                f_out.write("Timestep\t Cm_x\t Cm_y\t Cm_z\t vx\t vy\t vz\t fx\t fy\t fz\t fsx\t fsy\t fsz\t fdx\t fdy\t fdz\n")
            vals = [step, *pos[k].tolist(), vel[k, 0], vel[k, 1], abs(vel[k, 2]), *frc[k].tolist(), 0.0, 0.0, 0.0,
                    0.0, 0.0, 0.0]
            f_out.write("\t".join(str(x) for x in vals) + "\n")
