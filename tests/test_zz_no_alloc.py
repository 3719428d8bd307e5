"""gaia_vbd_energy_noalloc: the energy entry point for callers that cannot allocate
device memory (hosts that own the whole device memory pool, or that forbid
cudaMalloc after start-up because it synchronizes the device).

The test calls it through the C ABI on caller-owned device arrays and checks its
result against the existing entry point, gaia_vbd_energy, on two calls in a row
(the second on a different state, so a stale scratch array would show). This file
is collected last so that a run stopping at the first failure has already run
every other test; it also passes alone in a fresh process.
"""
import ctypes as C
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_energy_noalloc_matches_energy(tmp_path, gaia_lib):
    import torch

    from gaia_gb300 import VBDPhysics, scenes
    from gaia_gb300._lib import lib
    from oracle import scene_io

    mp, pp = scenes.drop_cube(str(tmp_path), n=7, iterations=5, precision="fp64")
    model = json.load(open(mp))["Models"][0]
    _, T = scene_io.load_t(model["path"])
    dt = json.load(open(pp))["PhysicsParams"]["timeStep"]

    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    phys.initialize()
    rest = phys.positions(0)  # right after initialize the inertia targets are the rest positions
    dminv, vol, mass = phys.restShape(0)
    dev = torch.device("cuda")
    d_y = torch.tensor(rest, dtype=torch.float64, device=dev).contiguous()
    d_mass = torch.tensor(mass, dtype=torch.float64, device=dev)
    d_tets = torch.tensor(T, dtype=torch.int32, device=dev).contiguous()
    d_dminv = torch.tensor(dminv, dtype=torch.float64, device=dev).contiguous()
    d_vol = torch.tensor(vol, dtype=torch.float64, device=dev)
    d_out = torch.zeros(1, dtype=torch.float64, device=dev)

    rng = np.random.Generator(np.random.PCG64(17))
    for call in range(2):
        x = rest * (1.0 + 0.01 * (call + 1)) + rng.uniform(-4e-4, 4e-4, size=rest.shape)
        phys.setPositions(0, x)
        expected = phys.energy()
        d_x = torch.tensor(x, dtype=torch.float64, device=dev).contiguous()
        torch.cuda.synchronize()
        rc = lib().gaia_vbd_energy_noalloc(d_x.data_ptr(), d_y.data_ptr(), d_mass.data_ptr(), len(x),
                                           d_tets.data_ptr(), d_dminv.data_ptr(), d_vol.data_ptr(), len(T),
                                           model["miu"], model["lmbd"], dt, d_out.data_ptr(), None)
        assert rc == 0, lib().gaia_vbd_last_global_error()
        torch.cuda.synchronize()
        got = float(d_out.item())
        assert expected > 1e-6
        assert abs(got - expected) <= 1e-10 * abs(expected), (call, got, expected)

    # sizes beyond the fixed scratch are rejected with a message, nothing is launched
    rc = lib().gaia_vbd_energy_noalloc(d_y.data_ptr(), None, None, (1 << 24) + 1, d_tets.data_ptr(),
                                       d_dminv.data_ptr(), d_vol.data_ptr(), len(T), model["miu"], model["lmbd"],
                                       dt, d_out.data_ptr(), None)
    assert rc == 1
    assert b"at most" in lib().gaia_vbd_last_global_error()
    phys.close()
