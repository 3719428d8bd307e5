"""The CUDA path against the reference's own VBD code (through the C ABI).

Golden outputs of the reference's host/device VBD functions, compiled from its sources
(tests/golden/vbd_ref_goldens.npz, made by tests/golden/make_vbd_goldens.py; see
tests/test_ref_goldens.py for what they hold). The FP64 engine must equal the reference's
formulas evaluated in double to 1e-9; the FP32-compute engines are held to the FP32
tolerances of the other parity tests, and each check prints how far the reference's own
float arithmetic lands from the same double result.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "vbd_ref_goldens.npz"))


def _handle(mp, pp, precision):
    from gaia_gb300 import VBDPhysics, scenes

    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
    phys.initialize()
    return phys


@pytest.fixture(scope="module")
def drop6(tmp_path_factory, gaia_lib):
    from gaia_gb300 import scenes

    d = tmp_path_factory.mktemp("drop6_ref")
    return scenes.drop_cube(str(d), n=6, iterations=10, height=0.02, collision=scenes.NO_CONTACT)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 2e-5), ("fp32", 2e-5)])
def test_vertex_block_probe(drop6, precision, tol):
    """Per-vertex force and Hessian of the solve kernel (material, inertia, ground with
    friction) on the deformed cube, against the kernel composition of the reference."""
    mp, pp = drop6
    phys = _handle(mp, pp, precision)
    phys.setPositions(0, G["blk_x"])
    worst = worst32 = 0.0
    for v in range(len(G["blk_x"])):
        f, H = phys.vertexForceHessian(0, v, True)
        fr, Hr = G["blk_f64"][v], G["blk_h64"][v]
        hs = np.abs(Hr).max()
        fs = max(np.abs(fr).max(), 1e-6 * hs)
        err = max(np.abs(f - fr).max() / fs, np.abs(H - Hr).max() / hs)
        err32 = max(np.abs(G["blk_f32"][v] - fr).max() / fs, np.abs(G["blk_h32"][v] - Hr).max() / hs)
        worst, worst32 = max(worst, err), max(worst32, err32)
    print(f"{precision}: worst force/Hessian error vs the reference (double) {worst:.2e}; the reference's "
          f"float build {worst32:.2e}")
    assert worst <= tol
    phys.close()


def test_energy(drop6):
    """The FP64 energy reduction: the reference's per-tet energies summed, plus inertia."""
    mp, pp = drop6
    phys = _handle(mp, pp, "fp64")
    X = phys.positions(0)
    _, _, mass = phys.restShape(0)
    phys.setPositions(0, G["blk_x"])
    inertia = 0.5 * 300.0 ** 2 * float((mass * ((G["blk_x"] - X) ** 2).sum(axis=1)).sum())
    e_ref = float(G["blk_elastic_energy64"]) + inertia
    e = phys.energy()
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref), (e, e_ref)
    phys.close()


def test_contact_block_probe(tmp_path, gaia_lib):
    """Vertices in contact and face vertices holding relations: detection on the golden state
    gives the golden rows, and the FP64 engine's force and Hessian equal the reference's."""
    from gaia_gb300 import scenes

    mp, pp = scenes.stack_drop(str(tmp_path), spacing=0.03, gap=0.01, speed=1.0, precision="fp64")
    phys = _handle(mp, pp, "fp64")
    for m in (0, 1):
        phys.setPrevPositions(m, G[f"con_prev{m}"])
        phys.setPositions(m, G[f"con_x{m}"])
    phys.collide()
    np.testing.assert_array_equal(phys.contacts(), G["con_rows"])
    for k, (m, v) in enumerate(G["con_probe"]):
        f, H = phys.vertexForceHessian(int(m), int(v), True)
        fr, Hr = G["con_f64"][k], G["con_h64"][k]
        hs = np.abs(Hr).max()
        assert np.abs(f - fr).max() <= 1e-9 * max(np.abs(fr).max(), 1e-6 * hs), (m, v, f, fr)
        assert np.abs(H - Hr).max() <= 1e-9 * hs, (m, v)
    phys.close()


@pytest.mark.parametrize("case", ["drop", "stretch"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-5), ("fp32", 1e-5)])
def test_trajectory(case, precision, tol, tmp_path, gaia_lib):
    """Contact-free trajectories of the reference's GPU step composed from its own functions:
    the 6^3 drop (40 steps) and the released stretch (20 steps), every 10 steps."""
    from gaia_gb300 import scenes
    from tests.golden.make_vbd_goldens import stretched_cube, stretched_state

    if case == "drop":
        mp, pp = scenes.drop_cube(str(tmp_path), n=6, iterations=10, height=0.02, collision=scenes.NO_CONTACT)
    else:
        mp, pp = stretched_cube(str(tmp_path))
    phys = _handle(mp, pp, precision)
    x0 = phys.positions(0)
    if case == "stretch":
        x0 = stretched_state(x0)
        phys.setPositions(0, x0)
    ref, ref32 = G[f"traj_{case}64"], G[f"traj_{case}32"]
    for k in range(len(ref)):
        phys.runStep(10)
        x = phys.positions(0)
        den = np.linalg.norm(ref[k] - x0)
        rel = np.linalg.norm(x - ref[k]) / den
        rel32 = np.linalg.norm(ref32[k] - ref[k]) / den
        print(f"{case} {precision} step {10 * (k + 1)}: vs reference (double) {rel:.2e}; the reference's float "
              f"build {rel32:.2e}")
        assert rel <= tol, (case, precision, k, rel)
    phys.close()
