"""Parity of the CUDA VBD step (through the C ABI) against the FP64 CPU oracle.

Tolerances (relative position error rel = |x - x_ref|_2 / |x_ref - x_ref,0|_2
over all vertices, the metric named for this path):
  * fp64 engine  vs FP64 oracle: 1e-9 (same algorithm, different summation order)
  * mixed engine vs FP64 oracle: 1e-5 (the stated bound)
  * fp32 engine  vs FP64 oracle: 1e-5 (the stated bound), the plain-drop configuration
    included: there the FP32 states are kept relative to a per-mesh frame that follows the
    falling cube (PhysicsParams meshFrames, on by default), so the landing amplifies a
    rounding at the scale of the deformation, not of the distance fallen.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-9, "mixed": 1e-5, "dfhi": 1e-5, "fp32": 1e-5}


def _rel(x, xr, x0):
    return float(np.linalg.norm(x - xr) / max(np.linalg.norm(xr - x0), 1e-300))


def _run_gpu(mp, pp, precision, steps, **overrides):
    from gaia_gb300 import VBDPhysics, scenes

    pp2 = scenes.set_precision(pp, precision, **overrides)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp2)
    phys.initialize()
    x0 = [phys.positions(m) for m in range(phys.numMeshes())]
    phys.runStep(steps)
    phys.synchronize()
    xs = [phys.positions(m) for m in range(phys.numMeshes())]
    st = phys.stats()
    phys.close()
    return x0, xs, st


def _run_oracle(mp, pp, steps, oracle_lib):
    from oracle import scene_io

    sc = scene_io.load_scene(mp, pp)
    o = oracle_lib.OracleScene(sc, precision=64, nthreads=0)
    o.step(steps)
    return [o.positions(m) for m in range(len(sc["meshes"]))]


@pytest.fixture(scope="module")
def drop_scene(tmp_path_factory, gaia_lib):
    from gaia_gb300 import scenes

    d = tmp_path_factory.mktemp("drop")
    return scenes.drop_cube(str(d), n=8, iterations=10, height=0.02)


@pytest.fixture(scope="module")
def drop_ref(drop_scene, oracle_lib):
    mp, pp = drop_scene
    return _run_oracle(mp, pp, 40, oracle_lib)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_timed_steps_advance_like_run_step(drop_scene, precision):
    """Both forms of the timed steps (the one graph per substep that runStep launches, timed
    as a whole; the substep's three graphs with the sweeps timed apart) advance the state
    exactly as runStep does."""
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp = drop_scene
    fixed = dict(lanesPerVertex=8, blockSize=128, autotune=False, solveVariant=0, sweepMode="merged")
    _, xs, _ = _run_gpu(mp, pp, precision, 6, **fixed)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, precision, **fixed))
    phys.initialize()
    tot, sw = phys.run_steps_timed(3, sweeps=False)
    assert tot > 0 and sw is None
    tot2, sw2 = phys.run_steps_timed(3)
    assert 0 < sw2 <= tot2
    x = phys.positions(0)
    phys.close()
    np.testing.assert_array_equal(x, xs[0])


@pytest.mark.parametrize("precision", ["fp64", "mixed", "dfhi", "fp32"])
def test_drop_cube_trajectory(drop_scene, drop_ref, precision):
    """8^3 cube dropped 2 cm onto the ground, 40 steps x 10 iterations: lands, slides, settles."""
    mp, pp = drop_scene
    x0, xs, st = _run_gpu(mp, pp, precision, 40)
    rel = _rel(xs[0], drop_ref[0], x0[0])
    print(f"{precision}: rel err {rel:.3e} max {np.abs(xs[0] - drop_ref[0]).max():.3e} stats {st}")
    assert np.isfinite(rel)
    assert rel <= TOL[precision]
    assert drop_ref[0][:, 1].min() < 0.005  # it did reach the ground


@pytest.mark.parametrize("lanes", [2, 4, 8, 16, 32])
def test_lanes_per_vertex_agree(drop_scene, drop_ref, lanes):
    """Every lanes-per-vertex variant of the solve kernel gives the oracle's result."""
    mp, pp = drop_scene
    x0, xs, st = _run_gpu(mp, pp, "fp64", 40, lanesPerVertex=lanes, blockSize=128, autotune=False,
                          smallColorVertices=0)
    assert st["lanes_per_vertex"] == lanes
    assert _rel(xs[0], drop_ref[0], x0[0]) <= TOL["fp64"]


@pytest.mark.parametrize("variant", [0, 1, 4, 6, 7])
@pytest.mark.parametrize("lanes", [4, 32])
@pytest.mark.parametrize("precision", ["mixed", "dfhi", "fp32"])
def test_solve_variants_agree(drop_scene, drop_ref, variant, lanes, precision):
    """Register-pipelined (0), TMA-staged (1), two-deep register-pipelined (4),
    register-pipelined with the next wave's records prefetched into L2 (6) and double-buffered
    TMA tiles on a persistent grid (7) solve kernels, with and without programmatic dependent
    launch, give the oracle's result."""
    mp, pp = drop_scene
    for pdl in (True, False):
        x0, xs, st = _run_gpu(mp, pp, precision, 40, lanesPerVertex=lanes, blockSize=128, autotune=False,
                              solveVariant=variant, usePDL=pdl, smallColorVertices=0, sweepMode="merged")
        assert st["solve_variant"] == variant
        assert _rel(xs[0], drop_ref[0], x0[0]) <= TOL[precision], (variant, lanes, precision, pdl)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("variant,block", [(1, 128), (6, 128), (7, 64), (7, 256)])
def test_variants_are_bit_identical(drop_scene, precision, variant, block):
    """Staging records in shared memory (1, 7) or prefetching them into L2 (6) moves no
    result: the same records per lane in the same order, so variant 0 bit for bit."""
    mp, pp = drop_scene
    common = dict(lanesPerVertex=4, blockSize=block, autotune=False, smallColorVertices=0, sweepMode="merged")
    _, xa, sa = _run_gpu(mp, pp, precision, 20, solveVariant=0, **common)
    _, xb, sb = _run_gpu(mp, pp, precision, 20, solveVariant=variant, **common)
    assert sa["solve_variant"] == 0 and sb["solve_variant"] == variant
    np.testing.assert_array_equal(xa[0], xb[0])


def test_twist(tmp_path, gaia_lib, oracle_lib):
    """Twist test (both x faces Dirichlet, one rotating at 2 rad/s), 10^3 lattice, 20 steps x 20 iterations."""
    from gaia_gb300 import scenes

    mp, pp = scenes.twist_cube(str(tmp_path), n=10, iterations=20)
    ref = _run_oracle(mp, pp, 20, oracle_lib)
    for precision in ("fp64", "mixed", "dfhi", "fp32"):
        x0, xs, st = _run_gpu(mp, pp, precision, 20)
        rel = _rel(xs[0], ref[0], x0[0])
        print(f"twist {precision}: rel {rel:.3e}")
        assert rel <= TOL[precision]


@pytest.fixture(scope="module")
def plain_drop(tmp_path_factory, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes

    d = tmp_path_factory.mktemp("plain_drop")
    mp, pp = scenes.drop_cube(str(d), n=10, iterations=20, coloring="greedy", collision=scenes.NO_CONTACT)
    return mp, pp, _run_oracle(mp, pp, 100, oracle_lib)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "dfhi", "fp32"])
def test_plain_drop_configuration(precision, plain_drop):
    """The plain VBD drop exactly as configured for the CPU-runnable case: a 10^3-vertex
    lattice (3645 tets) 0.2 m above the ground plane, OrderedGreedy coloring, no contact
    detection, 20 iterations per step, 100 steps (it lands near step 60 and slides)."""
    mp, pp, ref = plain_drop
    x0, xs, st = _run_gpu(mp, pp, precision, 100)
    rel = _rel(xs[0], ref[0], x0[0])
    print(f"plain drop {precision}: rel err {rel:.3e} max {np.abs(xs[0] - ref[0]).max():.3e}")
    assert ref[0][:, 1].min() < 0.01  # it landed (the bottom started 0.2 m up)
    assert rel <= TOL[precision]


def test_batch_scenes(tmp_path, gaia_lib, oracle_lib):
    """Several independent cubes of different sizes and materials in one scene (merged colors)."""
    from gaia_gb300 import scenes

    mp, pp = scenes.batch_cubes(str(tmp_path), n_scenes=12, side_range=(3, 7), iterations=8)
    ref = _run_oracle(mp, pp, 30, oracle_lib)
    for precision in ("fp64", "mixed", "dfhi"):
        x0, xs, st = _run_gpu(mp, pp, precision, 30)
        num = sum(np.linalg.norm(a - b) ** 2 for a, b in zip(xs, ref)) ** 0.5
        den = sum(np.linalg.norm(b - a0) ** 2 for b, a0 in zip(ref, x0)) ** 0.5
        assert num / den <= TOL[precision], (precision, num / den)


def test_force_hessian_probe(drop_scene, gaia_lib, oracle_lib):
    """Per-vertex force and 3x3 Hessian of the kernel vs the oracle's 9x9 formulation, on a
    randomly deformed state (material + inertia + ground + friction)."""
    from gaia_gb300 import VBDPhysics, scenes
    from oracle import scene_io

    mp, pp = drop_scene
    sc = scene_io.load_scene(mp, pp)
    o = oracle_lib.OracleScene(sc, precision=64, nthreads=1)
    rng = np.random.Generator(np.random.PCG64(3))
    x = o.positions(0)
    x = x + rng.uniform(-1e-3, 1e-3, size=x.shape)
    x[:, 1] -= 0.021  # push the bottom layer below the ground
    o.set_positions(0, x)
    for precision, tol in (("fp64", 1e-9), ("mixed", 2e-5)):
        phys = VBDPhysics()
        phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
        phys.initialize()
        phys.setPositions(0, x)
        for v in range(0, len(x), 37):
            f, H = phys.vertexForceHessian(0, v, True)
            fr, Hr = o.vertex_force_hessian(0, v, True)
            scale_f = np.abs(fr).max() + 1e-12
            scale_h = np.abs(Hr).max()
            assert np.abs(f - fr).max() <= tol * max(scale_f, 1e-6 * scale_h), (precision, v, f, fr)
            assert np.abs(H - Hr).max() <= tol * scale_h, (precision, v, H, Hr)
        phys.close()


def test_energy_matches_oracle(drop_scene, gaia_lib, oracle_lib):
    from gaia_gb300 import VBDPhysics, scenes
    from oracle import scene_io

    mp, pp = drop_scene
    sc = scene_io.load_scene(mp, pp)
    o = oracle_lib.OracleScene(sc, precision=64, nthreads=1)
    rng = np.random.Generator(np.random.PCG64(11))
    x = o.positions(0) * 1.01 + rng.uniform(-5e-4, 5e-4, size=(sc["meshes"][0]["X"].shape))
    o.set_positions(0, x)
    er = o.energy()
    assert er > 1e-6
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-10), ("fp32", 1e-3)):
        phys = VBDPhysics()
        phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
        phys.initialize()
        phys.setPositions(0, x)
        e = phys.energy()
        phys.close()
        assert abs(e - er) <= tol * abs(er), (precision, e, er)


def test_state_roundtrip_f32(drop_scene, gaia_lib):
    """set_state_f32 / get_positions_f32 (the e2e path) round-trip host order through the slot layout."""
    from gaia_gb300 import VBDPhysics

    from gaia_gb300 import scenes

    mp, pp = drop_scene
    rng = np.random.Generator(np.random.PCG64(5))
    for precision in ("mixed", "fp64", "fp32"):
        phys = VBDPhysics()
        phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
        phys.initialize()
        n = phys.numVertices(0)
        x = rng.uniform(-1, 1, size=(n, 3)).astype(np.float32)
        v = rng.uniform(-1, 1, size=(n, 3)).astype(np.float32)
        phys.set_state_f32(x.ctypes.data, v.ctypes.data)
        out = np.empty_like(x)
        phys.get_positions_f32(out.ctypes.data)
        vo = np.empty_like(v)
        phys.get_velocities_f32(vo.ctypes.data)
        if precision == "fp32":  # positions are stored as FP32 displacements from rest
            assert np.allclose(out, x, rtol=0, atol=2e-7)
        else:
            assert np.array_equal(out, x)
        assert np.array_equal(vo, v)
        assert np.array_equal(phys.velocities(0), v.astype(np.float64))
        phys.close()
