"""Mesh frames (PhysicsParams meshFrames): FP32-compute states kept relative to a per-mesh
frame offset F that follows the mesh, re-based at the start of every substep.

- on where it applies (FP32-compute precisions, no contact detection, no deformers), off
  elsewhere, and off on request;
- positions read and written through the C ABI are X + F + u: a round trip after the frame
  has moved returns what was written;
- against the FP64 oracle: the plain-drop configuration (100 steps) and a batch of uneven
  cubes, every FP32-compute precision within the parity tolerance, and the FP32 mode closer
  to the oracle with frames than without.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _handle(mp, pp, precision, **over):
    from gaia_gb300 import VBDPhysics, scenes

    tag = "_".join(f"{k}{v}" for k, v in over.items())
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, precision, out_path=pp + f".{precision}.{tag}.json",
                                                        **over))
    phys.initialize()
    return phys


def _run(mp, pp, precision, steps, **over):
    phys = _handle(mp, pp, precision, **over)
    x0 = np.concatenate([phys.positions(m) for m in range(phys.numMeshes())])
    phys.runStep(steps)
    x = np.concatenate([phys.positions(m) for m in range(phys.numMeshes())])
    st = phys.stats()
    phys.close()
    return x0, x, st


def _oracle(mp, pp, steps, oracle_lib):
    from oracle import scene_io

    sc = scene_io.load_scene(mp, pp)
    o = oracle_lib.OracleScene(sc, precision=64, nthreads=0)
    o.step(steps)
    return np.concatenate([o.positions(m) for m in range(len(sc["meshes"]))])


def _rel(x, xr, x0):
    return float(np.linalg.norm(x - xr) / np.linalg.norm(xr - x0))


@pytest.fixture(scope="module")
def plain_drop(tmp_path_factory, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes

    d = tmp_path_factory.mktemp("frames_drop")
    mp, pp = scenes.drop_cube(str(d), n=10, iterations=20, coloring="greedy", collision=scenes.NO_CONTACT)
    return mp, pp, _oracle(mp, pp, 100, oracle_lib)


def test_frames_where_they_apply(plain_drop, tmp_path):
    from gaia_gb300 import scenes

    mp, pp, _ = plain_drop
    for precision in ("fp32", "dfhi", "mixed"):
        h = _handle(mp, pp, precision)
        assert h.stats()["mesh_frames"] == 1, precision
        h.close()
    for precision, over in (("fp64", {}), ("fp32", {"meshFrames": False})):
        h = _handle(mp, pp, precision, **over)
        assert h.stats()["mesh_frames"] == 0, (precision, over)
        h.close()
    # contact detection on, and deformers: off
    mpc, ppc = scenes.drop_cube(str(tmp_path / "c"), n=5, iterations=5)
    h = _handle(mpc, ppc, "fp32")
    assert h.stats()["mesh_frames"] == 0
    h.close()
    mpt, ppt = scenes.twist_cube(str(tmp_path / "t"), n=6, iterations=5)
    h = _handle(mpt, ppt, "fp32")
    assert h.stats()["mesh_frames"] == 0
    h.close()


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_positions_round_trip_in_a_moved_frame(plain_drop, precision):
    mp, pp, _ = plain_drop
    h = _handle(mp, pp, precision)
    h.runStep(30)  # the cube has fallen: its frame offset is far from zero
    x = h.positions(0)
    rng = np.random.default_rng(3)
    xw = x + rng.uniform(-1e-4, 1e-4, size=x.shape)
    h.setPositions(0, xw)
    xr = h.positions(0)
    tol = 1e-12 if precision == "mixed" else 4e-8  # FP32 state: one rounding of the frame-relative value
    assert np.abs(xr - xw).max() <= tol
    h.close()


@pytest.mark.parametrize("precision", ["fp32", "dfhi", "mixed"])
def test_plain_drop_with_frames(plain_drop, precision):
    """The plain-drop configuration (10^3 lattice, greedy coloring, 20 iterations, 100
    steps) against the FP64 oracle, with and without frames."""
    mp, pp, ref = plain_drop
    x0, x, st = _run(mp, pp, precision, 100)
    _, xo, so = _run(mp, pp, precision, 100, meshFrames=False)
    assert st["mesh_frames"] == 1 and so["mesh_frames"] == 0
    rel, rel_off = _rel(x, ref, x0), _rel(xo, ref, x0)
    print(f"plain drop {precision}: frames {rel:.3e}, without {rel_off:.3e}")
    assert rel <= TOL
    if precision == "fp32":
        assert rel < rel_off


@pytest.mark.parametrize("precision", ["fp32", "dfhi"])
def test_batch_with_frames(tmp_path, gaia_lib, oracle_lib, precision):
    from gaia_gb300 import scenes

    mp, pp = scenes.batch_cubes(str(tmp_path), n_scenes=24, side_range=(3, 9), iterations=8)
    ref = _oracle(mp, pp, 60, oracle_lib)
    x0, x, st = _run(mp, pp, precision, 60)
    _, xo, _ = _run(mp, pp, precision, 60, meshFrames=False)
    rel, rel_off = _rel(x, ref, x0), _rel(xo, ref, x0)
    print(f"batch of 24 {precision}: frames {rel:.3e}, without {rel_off:.3e}")
    assert st["mesh_frames"] == 1
    assert rel <= TOL
