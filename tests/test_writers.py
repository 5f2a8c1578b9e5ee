"""Output formats: the drop-in VTK and particle-data writers produce the reference's files byte for
byte (LIBRARIES/LIBRARY_Vtk_creator.py, LIBRARIES/LIBRARY_Write_particle_data.py, run here from the
reference checkout; skipped without it), and the device snapshot writes the same VTK layout."""
import copy
import importlib
import sys

import numpy as np
import pytest

import oracle

ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not present")


def _reference_module(name):
    import build_ref
    p = str(build_ref.REFERENCE_ROOT / "LIBRARIES")
    if p not in sys.path:
        sys.path.insert(0, p)
    # the reference's module of the same name, not this package's drop-in
    spec = importlib.util.spec_from_file_location("ref_" + name, str(build_ref.REFERENCE_ROOT / "LIBRARIES" / (name + ".py")))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _particles(seed=3):
    from mwdiem_gb300.Particle_class import Particle
    np.random.seed(seed)
    acc = np.array([0.0, 0.0, -9.81])
    ps = []
    for k in range(4):
        p = Particle(k)
        p.Spherical_convex_polygon_maker_3D(12, 24, 1.0, 0.1, 1.0, 1, acc, np.zeros(3))
        p.Translate(np.random.uniform(-5, 5, 3))
        ps.append(p)
    return ps


@ref
def test_vtk_creator_matches_reference(tmp_path):
    from mwdiem_gb300 import LIBRARY_Vtk_creator as mine
    theirs = _reference_module("LIBRARY_Vtk_creator")
    rng = np.random.default_rng(0)
    q = rng.normal(size=(4, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    dx = rng.normal(size=(4, 3))
    a, b = _particles(), _particles()
    qa, dxa = mine.Vtk_creator(a, str(tmp_path / "a.vtk"), 1, 4, q.copy(), dx.copy())
    qb, dxb = theirs.Vtk_creator(b, str(tmp_path / "b.vtk"), 1, 4, q.copy(), dx.copy())
    assert (tmp_path / "a.vtk").read_text() == (tmp_path / "b.vtk").read_text()
    assert np.array_equal(qa, qb) and np.array_equal(dxa, dxb)


@ref
def test_particle_data_writer_matches_reference(tmp_path):
    from mwdiem_gb300 import LIBRARY_Write_particle_data as mine
    theirs = _reference_module("LIBRARY_Write_particle_data")
    p = _particles()[1]
    p.velocity = np.array([0.5, -0.25, -1.5])
    p.force_normal = np.array([1.0, 2.0, 3.0])
    for step in range(3):
        mine.Particle_data_writer(p, str(tmp_path / "m_"), step)
        theirs.Particle_data_writer(p, str(tmp_path / "r_"), step)
    assert (tmp_path / "m_1.dat").read_text() == (tmp_path / "r_1.dat").read_text()


@pytest.mark.gpu
def test_device_vtk_snapshot(tmp_path):
    import torch
    from mwdiem_gb300 import scene
    from mwdiem_gb300.sim import Simulator
    from mwdiem_gb300.writers import VtkSnapshot
    sp = scene.pour_scene(n=60, box=10.0, seed=2)
    sim = Simulator(sp)
    sim.step(3)
    snap = VtkSnapshot(sim)
    snap.write(str(tmp_path / "s.vtk"))
    sim.step(2)                                  # the step may run on while the file is written
    snap.wait()
    torch.cuda.synchronize()
    text = (tmp_path / "s.vtk").read_text().split("\n")
    assert text[:4] == ["# vtk DataFile Version 2.0", "# kata", "ASCII", "DATASET POLYDATA"]
    npts = int(text[4].split("\t")[1])
    assert npts == sim.vert_off_host[-1]
    pts = np.array([[float(x) for x in ln.split("\t")] for ln in text[5:5 + npts]])
    assert pts.shape == (npts, 3)
    nf = int(text[5 + npts].split("\t")[1])
    tri = np.array([[int(x) for x in ln.split("\t")] for ln in text[6 + npts:6 + npts + nf]])
    assert np.all(tri[:, 0] == 3) and tri[:, 1:].max() < npts
