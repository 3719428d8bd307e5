"""The FP64 convergence reduction on the GPU (evaluateConvergenceGPU, VBD/VBDPhysics.cpp:
3508-3556): energy, inertia and elastic energy and the average force norm, against the
oracle's FP64 evaluation (1e-12 relative in the FP64 engine on one state), bit-identical from call to
call and between handles (fixed-order two-pass reduction, no atomics), and the in-graph
records of evaluateConvergence at iterations -1, 0, n, 2n, ... of every substep."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("energy", "inertia", "elastic", "avg_force_norm")


def _scene(tmp_path, **extra):
    """The twist at 8^3 (fixed end faces, one driven by the rotator: fixed vertices with
    inertia energy), with damping on, so every term of the reduction is exercised."""
    from gaia_gb300 import scenes

    mp, pp = scenes.twist_cube(str(tmp_path), n=8, iterations=10, precision="fp64")
    M = json.load(open(mp))
    for m in M["Models"]:
        m["dampingHydrostatic"] = 1e-3
        m["dampingDeviatoric"] = 2e-3
    json.dump(M, open(mp, "w"))
    if extra:
        P = json.load(open(pp))
        P["PhysicsParams"].update(extra)
        json.dump(P, open(pp, "w"))
    return mp, pp


def _handle(mp, pp, precision):
    from gaia_gb300 import VBDPhysics, scenes

    h = VBDPhysics()
    h.loadRunningparameters(mp, scenes.set_precision(pp, precision))
    h.initialize()
    return h


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-11), ("fp32", 1e-5)])
def test_convergence_matches_oracle(tmp_path, precision, tol, gaia_lib, oracle_lib):
    """The reduction on one state on both sides: fresh handles (inertia targets and previous
    positions at rest), the same deformed positions set on both; the FP64 engine to 1e-12.
    The FP32-compute engines hold the positions as displacements in their state format."""
    from oracle import scene_io

    mp, pp = _scene(tmp_path)
    h = _handle(mp, pp, precision)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), precision=64, nthreads=1)
    rng = np.random.Generator(np.random.PCG64(8))
    x = h.positions(0)
    x = x * 1.002 + rng.uniform(-3e-4, 3e-4, size=x.shape)
    h.setPositions(0, x)
    o.set_positions(0, h.positions(0))  # the positions as the engine holds them
    c, co = h.evaluateConvergence(), o.convergence()
    for k in KEYS:
        assert abs(c[k] - co[k]) <= tol * abs(co[k]), (precision, k, c[k], co[k])
    assert c["inertia"] > 0 and c["elastic"] > 0 and c["avg_force_norm"] > 0
    again = h.evaluateConvergence()
    assert all(again[k] == c[k] for k in KEYS)  # bit-identical
    assert h.energy() == c["energy"]
    h.close()


def test_convergence_after_steps(tmp_path, gaia_lib, oracle_lib):
    """After 3 steps of the FP64 engine and the oracle (states equal to rounding): energies to
    1e-12; the average force norm, a residual in which the step's rounding differences are
    amplified, to 1e-9."""
    from oracle import scene_io

    mp, pp = _scene(tmp_path)
    h = _handle(mp, pp, "fp64")
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), precision=64, nthreads=1)
    h.runStep(3)
    o.step(3)
    c, co = h.evaluateConvergence(), o.convergence()
    for k in KEYS:
        assert abs(c[k] - co[k]) <= (1e-9 if k == "avg_force_norm" else 1e-12) * abs(co[k]), (k, c[k], co[k])
    h.close()


def test_convergence_bit_identical_across_handles(tmp_path, gaia_lib):
    mp, pp = _scene(tmp_path, lanesPerVertex=4, blockSize=128, autotune=False, sweepMode="merged")
    vals = []
    for _ in range(2):
        h = _handle(mp, pp, "mixed")
        h.runStep(2)
        vals.append(h.evaluateConvergence())
        h.close()
    assert all(vals[0][k] == vals[1][k] for k in KEYS)


def test_convergence_log_in_graph(tmp_path, gaia_lib, oracle_lib):
    """evaluateConvergence with evaluationSteps 3 and 10 iterations: records at iterations
    -1, 0, 3, 6, 9 of the substep; the last (after iteration 9) equals the evaluation after
    the step (the velocity update changes neither positions nor targets) and the oracle's;
    the energy at the end is below the initial guess's."""
    from oracle import scene_io

    mp, pp = _scene(tmp_path, evaluateConvergence=True, evaluationSteps=3)
    h = _handle(mp, pp, "fp64")
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), precision=64, nthreads=1)
    for step in range(3):
        h.runStep(1)
        o.step(1)
        log = h.convergenceLog()
        assert log.shape == (5, 6)
        np.testing.assert_array_equal(log[:, 0], 0)
        np.testing.assert_array_equal(log[:, 1], [-1, 0, 3, 6, 9])
        after = h.evaluateConvergence()
        np.testing.assert_array_equal(log[-1, 2:], [after[k] for k in KEYS])
        co = o.convergence()
        for j, k in enumerate(KEYS):
            tol = 1e-9 if k == "avg_force_norm" else 1e-12
            assert abs(log[-1, 2 + j] - co[k]) <= tol * abs(co[k]), (step, k)
        assert log[-1, 2] < log[0, 2]
    st = h.stats()
    h.close()
    # the records add kernels to the step, and only when asked for
    h2 = _handle(*_scene(tmp_path / "plain"), "fp64")
    assert st["kernel_launches_per_step"] == h2.stats()["kernel_launches_per_step"] + 3 * 5
    assert len(h2.convergenceLog()) == 0
    h2.close()
