"""Feature parity of the CUDA VBD step against the FP64 oracle: every optional
path of the step (Chebyshev accelerator, Rayleigh-like damping, initialization
types, Translator deformer, friction start iteration, velocity damping, initial
velocity, several meshes with different materials).

Tolerances as in test_gpu_parity.py: fp64 1e-9, mixed 1e-5 (relative position
error over all vertices after the run)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FEATURES = {
    "accelerator": ({}, {"useAccelerator": True, "acceleratorRho": 0.9}, None),
    "damping": ({"dampingHydrostatic": 2e-4, "dampingDeviatoric": 5e-4}, {}, None),
    "init1": ({"initializationType": 1}, {}, None),
    "init2": ({"initializationType": 2, "initialVelocity": [0.3, -0.2, 0.1]}, {}, None),
    "init3": ({"initializationType": 3}, {}, None),
    "init4": ({"initializationType": 4}, {}, None),
    "friction_start": ({}, {"frictionStartIter": 3}, None),
    "velocity_damping": ({"exponentialVelDamping": 0.8, "constantVelDamping": 0.01}, {}, None),
    "initial_velocity": ({"initialVelocity": [0.4, 0.0, -0.3]}, {}, None),
    "translator": ({}, {}, {"DeformerName": "Translator", "speed": [0.2, 0.0, 0.1], "selectedMeshes": [0],
                            "selectedVertices": [[0, 1, 2, 3, 4, 5]]}),
    "rotator_end_time": ({}, {}, {"DeformerName": "Rotator", "center": [0.0, 0.0, 0.0], "axis": [0.0, 1.0, 0.0],
                                  "angularVelocity": 3.0, "rotationEndTime": 0.02, "selectedMeshes": [0],
                                  "selectedVertices": [[0, 1, 2, 3, 4, 5]]}),
    "substeps": ({}, {"numSubsteps": 3, "timeStep": 0.01}, None),
}


def _scene(tmp_path, feature):
    from gaia_gb300 import scenes

    mp, pp = scenes.drop_cube(str(tmp_path), n=6, iterations=8, height=0.01)
    model_over, param_over, deformer = FEATURES[feature]
    M = json.load(open(mp))
    M["Models"][0].update(model_over)
    json.dump(M, open(mp, "w"))
    P = json.load(open(pp))
    P["PhysicsParams"].update(param_over)
    if deformer:
        P["Deformers"] = [deformer]
    json.dump(P, open(pp, "w"))
    return mp, pp


@pytest.mark.parametrize("feature", sorted(FEATURES))
def test_feature_parity(feature, tmp_path, gaia_lib, oracle_lib):
    from gaia_gb300 import VBDPhysics, scenes
    from oracle import scene_io

    mp, pp = _scene(tmp_path, feature)
    steps = 25
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 0)
    o.step(steps)
    xr, vr = o.positions(0), o.velocities(0)
    for precision, tol in (("fp64", 1e-9), ("mixed", 1e-5)):
        phys = VBDPhysics()
        phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
        phys.initialize()
        x0 = phys.positions(0)
        phys.runStep(steps)
        x, v = phys.positions(0), phys.velocities(0)
        phys.close()
        rel = np.linalg.norm(x - xr) / np.linalg.norm(xr - x0)
        assert rel <= tol, (feature, precision, rel)
        vscale = max(np.abs(vr).max(), 1e-3)
        assert np.abs(v - vr).max() <= max(tol, 1e-7) * 1e3 * vscale, (feature, precision)


def test_two_meshes_two_materials(tmp_path, gaia_lib, oracle_lib):
    """Two meshes with different Lame parameters, densities and colorings share merged colors."""
    from gaia_gb300 import VBDPhysics, scenes
    from oracle import scene_io

    Xa, Ta = scenes.lattice_cube((5, 4, 6), 0.012, (0.0, 0.02, 0.0), jitter=1e-4, seed=2)
    Xb, Tb = scenes.lattice_cube((3, 7, 4), 0.009, (0.2, 0.05, 0.0), jitter=1e-4, seed=3)
    ta, ca = scenes._write_mesh(str(tmp_path), "a", Xa, Ta)
    tb, cb = scenes._write_mesh(str(tmp_path), "b", Xb, Tb, coloring="mcs")
    models = [scenes.model_entry(ta, ca, E=3e5, nu=0.3, density=900.0),
              scenes.model_entry(tb, cb, E=2e6, nu=0.45, density=1500.0, initialVelocity=[0.0, -1.0, 0.0])]
    mp, pp = scenes._write_json(str(tmp_path), models, scenes.physics_params(1 / 300, 10, ground_y=0.0))
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 0)
    o.step(30)
    for precision, tol in (("fp64", 1e-9), ("mixed", 1e-5)):
        phys = VBDPhysics()
        phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
        phys.initialize()
        x0 = [phys.positions(m) for m in range(2)]
        phys.runStep(30)
        num = sum(np.linalg.norm(phys.positions(m) - o.positions(m)) ** 2 for m in range(2)) ** 0.5
        den = sum(np.linalg.norm(o.positions(m) - x0[m]) ** 2 for m in range(2)) ** 0.5
        phys.close()
        assert num / den <= tol, (precision, num / den)
