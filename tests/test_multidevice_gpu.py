"""The narrow phase on a second GPU after the first, in one process: the launch set-up (the raised
shared-memory limit of the narrow-phase kernels and their occupancy) is kept per device, so device 1
gets its own.  Needs two visible GPUs; skipped otherwise."""
import numpy as np
import pytest
import torch

import oracle
from helpers import CONTACT_PARAMS, make_pairs

pytestmark = pytest.mark.gpu


def run_on(dev, inp, N, lanes):
    from mwdiem_gb300 import gpu_fine_contact_detection as G
    p = CONTACT_PARAMS
    with torch.cuda.device(dev):
        d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda(dev) for k, v in inp.items()}
        F = torch.zeros((N, 3), dtype=torch.float32, device=f"cuda:{dev}")
        T = torch.zeros_like(F)
        F, T, _, coll = G.Contact_detection_GPU(
            d["A_com"], d["B_com"], d["A_verts"], d["B_verts"], d["A_vel"], d["B_vel"], d["A_angvel"],
            d["B_angvel"], d["A_nv"], d["B_nv"], d["A_id"], d["B_id"], d["hist"].clone(), p["Kn"], p["en"],
            p["et"], p["mu"], p["Kn_wall"], p["en_wall"], p["et_wall"], p["mu_wall"], p["num_particles_wall"],
            F, T, p["num_vertices_max"], d["qA"], d["qB"], p["timestep"], d["IsA"], d["IsB"], lanes=lanes)
        torch.cuda.synchronize(dev)
        return coll.cpu().numpy(), F.cpu().numpy()


@pytest.mark.skipif(torch.cuda.device_count() < 2, reason="needs two GPUs")
@pytest.mark.parametrize("lanes", [8, 32])
def test_narrow_phase_on_device_1_after_device_0(lanes):
    inp, N = make_pairs(800, seed=61)
    o = oracle.contact(inp, CONTACT_PARAMS, N, "f32")
    for dev in (0, 1):
        coll, F = run_on(dev, inp, N, lanes)
        assert np.array_equal(coll, o["collision"]), dev
        assert np.array_equal(F, o["force"]), dev
