"""The persistent sweeps (sweepMode "scenes", k_sweep_scenes; sweepMode "cluster",
k_sweep_cluster; sweepMode "grid", k_sweep_grid) and the autotuned choice of color
scheduling.

In this mode one launch per substep runs every scene's iterations: each block takes whole
meshes, their colors in the merged groups' order, a block barrier between colors. Meshes
do not interact there, so per mesh the update sequence equals the merged sweep's:
- against the FP64 oracle at the parity tolerances (the plain-drop configuration, a batch
  of uneven cubes with different materials, the twist with its rotating face);
- bit-identical to the merged sweep when both use the same lanes per vertex;
- the autotuner times both schedules and keeps the faster (stats report both times);
- the mode is refused where it cannot hold: contact detection on.
The grid sweep runs the merged colors in one cooperative launch per substep with a bounded
grid barrier between colors: against the oracle, bit-identical to the per-color launches,
and its barrier made to run out (a poll limit of zero) returns a status.
"""
import numpy as np
import pytest

from gaia_gb300._lib import E_UNSUPPORTED, GaiaError

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-9, "mixed": 1e-5, "dfhi": 1e-5, "fp32": 1e-5}


def _run(mp, pp, precision, steps, **over):
    from gaia_gb300 import VBDPhysics, scenes

    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, precision, out_path=pp + f".{precision}.s.json", **over))
    phys.initialize()
    x0 = [phys.positions(m) for m in range(phys.numMeshes())]
    phys.runStep(steps)
    phys.synchronize()
    xs = [phys.positions(m) for m in range(phys.numMeshes())]
    st = phys.stats()
    phys.close()
    return np.concatenate(x0), np.concatenate(xs), st


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

    d = tmp_path_factory.mktemp("plain_drop_s")
    mp, pp = scenes.drop_cube(str(d), n=10, iterations=20, coloring="greedy", collision=scenes.NO_CONTACT)
    return mp, pp, _oracle(mp, pp, 100, oracle_lib)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp32"])
def test_plain_drop_scenes_mode(plain_drop, precision):
    mp, pp, ref = plain_drop
    x0, x, st = _run(mp, pp, precision, 100, sweepMode="scenes")
    assert st["sweep_mode"] == 1 and st["solve_variant"] == 2
    rel = _rel(x, ref, x0)
    print(f"plain drop, scenes mode, {precision}: rel {rel:.3e}, lanes {st['lanes_per_vertex']} block "
          f"{st['block_size']}, {st['kernel_launches_per_step']} launches per step")
    assert rel <= TOL[precision]
    assert st["kernel_launches_per_step"] <= 4


@pytest.fixture(scope="module")
def batch(tmp_path_factory, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes

    d = tmp_path_factory.mktemp("batch_s")
    mp, pp = scenes.batch_cubes(str(d), n_scenes=24, side_range=(3, 9), iterations=8)
    return mp, pp, _oracle(mp, pp, 30, oracle_lib)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "dfhi", "fp32"])
def test_batch_scenes_mode(batch, precision):
    mp, pp, ref = batch
    x0, x, st = _run(mp, pp, precision, 30, sweepMode="scenes")
    rel = _rel(x, ref, x0)
    print(f"batch of 24, scenes mode, {precision}: rel {rel:.3e}")
    assert st["sweep_mode"] == 1
    assert rel <= TOL[precision] * (3 if precision == "fp32" else 1)


def test_twist_scenes_mode(tmp_path, gaia_lib, oracle_lib):
    """Fixed faces and the rotator (deformed fixed vertices are neighbours of solved ones)."""
    from gaia_gb300 import scenes

    mp, pp = scenes.twist_cube(str(tmp_path), n=10, iterations=20)
    ref = _oracle(mp, pp, 20, oracle_lib)
    for precision in ("fp64", "mixed", "fp32"):
        x0, x, st = _run(mp, pp, precision, 20, sweepMode="scenes")
        assert _rel(x, ref, x0) <= TOL[precision], precision


@pytest.mark.parametrize("lanes", [4, 16])
def test_scenes_mode_equals_merged(batch, lanes):
    """Same lanes per vertex: the two schedules give bit-identical positions."""
    mp, pp, _ = batch
    common = dict(lanesPerVertex=lanes, blockSize=256, autotune=False, smallColorVertices=0, solveVariant=0)
    _, xa, sa = _run(mp, pp, "mixed", 10, sweepMode="merged", **common)
    _, xb, sb = _run(mp, pp, "mixed", 10, sweepMode="scenes", **common)
    assert sa["sweep_mode"] == 0 and sb["sweep_mode"] == 1
    np.testing.assert_array_equal(xa, xb)


def test_autotuner_picks_schedule(plain_drop, batch):
    for mp, pp, _ in (plain_drop, batch):
        _, _, st = _run(mp, pp, "mixed", 1)
        times = [st["sweep_ms_merged"], st["sweep_ms_scenes"], st["sweep_ms_cluster"], st["sweep_ms_grid"]]
        print(f"ms/iteration: merged {times[0]:.4f}, scenes {times[1]:.4f}, cluster {times[2]:.4f}, "
              f"grid {times[3]:.4f}: mode {st['sweep_mode']}")
        assert all(t > 0 for t in times)
        assert st["sweep_mode"] == int(np.argmin(times))


def test_scenes_mode_refused_with_contact(tmp_path, gaia_lib):
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp = scenes.drop_cube(str(tmp_path), n=5, iterations=5)  # contact detection on (defaults)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, "mixed", sweepMode="scenes"))
    with pytest.raises(GaiaError) as ei:
        phys.initialize()
    assert ei.value.code == E_UNSUPPORTED and "sweepMode" in str(ei.value)
    # auto falls back to the merged schedule there
    phys2 = VBDPhysics()
    phys2.loadRunningparameters(mp, scenes.set_precision(pp, "mixed", out_path=pp + ".auto.json"))
    phys2.initialize()
    assert phys2.stats()["sweep_mode"] == 0
    phys2.close()


# ---------------------------------------------------------------- the cluster sweep
@pytest.mark.parametrize("precision", ["fp64", "mixed", "dfhi", "fp32"])
def test_plain_drop_cluster_mode(plain_drop, precision):
    """The plain-drop configuration on a thread-block cluster with the scene in distributed
    shared memory (every copy of the states updated through DSMEM, a cluster barrier per
    color), against the FP64 oracle."""
    mp, pp, ref = plain_drop
    x0, x, st = _run(mp, pp, precision, 100, sweepMode="cluster")
    assert st["sweep_mode"] == 2 and st["solve_variant"] == 3 and st["cluster_size"] in (2, 4, 8, 16)
    rel = _rel(x, ref, x0)
    print(f"plain drop, cluster mode, {precision}: rel {rel:.3e}, cluster {st['cluster_size']} lanes "
          f"{st['lanes_per_vertex']} block {st['block_size']}")
    assert rel <= TOL[precision]


@pytest.mark.parametrize("precision,cluster", [("fp64", 8), ("fp64", 16), ("mixed", 4), ("mixed", 16)])
def test_batch_cluster_mode(batch, precision, cluster):
    mp, pp, ref = batch
    x0, x, st = _run(mp, pp, precision, 30, sweepMode="cluster", clusterSize=cluster)
    assert st["sweep_mode"] == 2 and st["cluster_size"] == cluster
    assert _rel(x, ref, x0) <= TOL[precision]


def test_cluster_size_that_does_not_fit_is_refused(batch):
    """The 9^3 cube's FP64 records (96 B each) split over 4 blocks need ~350 KB of shared
    memory per block: an explicit clusterSize 4 is refused, not launched."""
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp, _ = batch
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, "fp64", out_path=pp + ".c4.json", sweepMode="cluster",
                                                        clusterSize=4))
    with pytest.raises(GaiaError) as ei:
        phys.initialize()
    assert ei.value.code == E_UNSUPPORTED and "clusterSize 4" in str(ei.value)
    phys.close()


def test_twist_cluster_mode(tmp_path, gaia_lib, oracle_lib):
    """Fixed faces driven by the rotator: fixed states are staged into every copy each substep."""
    from gaia_gb300 import scenes

    mp, pp = scenes.twist_cube(str(tmp_path), n=10, iterations=20)
    ref = _oracle(mp, pp, 20, oracle_lib)
    for precision in ("fp64", "mixed"):
        x0, x, st = _run(mp, pp, precision, 20, sweepMode="cluster")
        assert _rel(x, ref, x0) <= TOL[precision], precision


@pytest.mark.parametrize("cluster", [4, 16])
def test_cluster_mode_equals_merged(batch, cluster):
    mp, pp, _ = batch
    common = dict(lanesPerVertex=8, blockSize=128, autotune=False, smallColorVertices=0, solveVariant=0)
    _, xa, _ = _run(mp, pp, "mixed", 10, sweepMode="merged", **common)
    _, xc, sc = _run(mp, pp, "mixed", 10, sweepMode="cluster", clusterSize=cluster, **common)
    assert sc["sweep_mode"] == 2
    np.testing.assert_array_equal(xa, xc)


def test_cluster_mode_refused_when_too_large(tmp_path, gaia_lib):
    """A 40^3 lattice (64k vertices) does not fit in a 16-block cluster's shared memory:
    the explicit mode is refused, and the autotuner leaves it out."""
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp = scenes.twist_cube(str(tmp_path), n=40, iterations=4)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, "mixed", sweepMode="cluster"))
    with pytest.raises(GaiaError) as ei:
        phys.initialize()
    assert ei.value.code == E_UNSUPPORTED and "does not fit" in str(ei.value)
    phys2 = VBDPhysics()
    phys2.loadRunningparameters(mp, scenes.set_precision(pp, "mixed", out_path=pp + ".auto.json"))
    phys2.initialize()
    st = phys2.stats()
    assert st["sweep_mode"] in (0, 1, 3) and st["sweep_ms_cluster"] == 0
    phys2.close()


# ---------------------------------------------------------------- the grid sweep
@pytest.mark.parametrize("precision", ["fp64", "mixed", "dfhi", "fp32"])
def test_plain_drop_grid_mode(plain_drop, precision):
    """The plain-drop configuration in one cooperative launch per substep (merged colors, a
    grid barrier between colors), against the FP64 oracle."""
    mp, pp, ref = plain_drop
    x0, x, st = _run(mp, pp, precision, 100, sweepMode="grid")
    assert st["sweep_mode"] == 3 and st["solve_variant"] == 5 and st["device_timeouts"] == 0
    rel = _rel(x, ref, x0)
    print(f"plain drop, grid mode, {precision}: rel {rel:.3e}, lanes {st['lanes_per_vertex']} block "
          f"{st['block_size']}, {st['kernel_launches_per_step']} launches per step")
    assert rel <= TOL[precision]
    assert st["kernel_launches_per_step"] <= 4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_and_twist_grid_mode(batch, precision, tmp_path, oracle_lib):
    mp, pp, ref = batch
    x0, x, st = _run(mp, pp, precision, 30, sweepMode="grid")
    assert st["sweep_mode"] == 3
    assert _rel(x, ref, x0) <= TOL[precision]
    from gaia_gb300 import scenes

    mp, pp = scenes.twist_cube(str(tmp_path), n=10, iterations=20)
    ref = _oracle(mp, pp, 20, oracle_lib)
    x0, x, st = _run(mp, pp, precision, 20, sweepMode="grid")
    assert _rel(x, ref, x0) <= TOL[precision]


@pytest.mark.parametrize("lanes,block", [(4, 128), (16, 256)])
def test_grid_mode_equals_merged(batch, lanes, block):
    """Same lanes per vertex: the grid sweep and the per-color launches give bit-identical
    positions (dfhi: own and neighbour states read through L2)."""
    mp, pp, _ = batch
    for precision in ("mixed", "dfhi"):
        common = dict(lanesPerVertex=lanes, blockSize=block, autotune=False, smallColorVertices=0, solveVariant=0)
        _, xa, sa = _run(mp, pp, precision, 10, sweepMode="merged", **common)
        _, xg, sg = _run(mp, pp, precision, 10, sweepMode="grid", **common)
        assert sa["sweep_mode"] == 0 and sg["sweep_mode"] == 3
        np.testing.assert_array_equal(xa, xg)


def test_grid_barrier_timeout_is_reported(plain_drop):
    """waitPollLimit 0: a block that is not the last to arrive at a grid barrier gives up at
    once, raises the abort flag, and every other block gives up at its next barrier; the
    kernel ends, the next synchronizing call returns GAIA_VBD_E_DEVICE_TIMEOUT once, and the
    state stays finite and readable."""
    from gaia_gb300 import VBDPhysics, scenes
    from gaia_gb300._lib import E_DEVICE_TIMEOUT

    mp, pp, _ = plain_drop
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, "mixed", out_path=pp + ".gridto.json", sweepMode="grid",
                                                        lanesPerVertex=16, blockSize=128, autotune=False,
                                                        waitPollLimit=0))
    phys.initialize()
    phys.runStep(1)
    with pytest.raises(GaiaError) as ei:
        phys.synchronize()
    assert ei.value.code == E_DEVICE_TIMEOUT, str(ei.value)
    st = phys.stats()
    assert st["device_timeouts"] > 0 and st["sweep_mode"] == 3
    phys.synchronize()  # reported once
    assert np.isfinite(phys.positions(0)).all()
    phys.close()
    # the built-in limit: no timeout
    x0, x, st = _run(mp, pp, "mixed", 2, sweepMode="grid", lanesPerVertex=16, blockSize=128, autotune=False)
    assert st["device_timeouts"] == 0 and np.isfinite(x).all()
