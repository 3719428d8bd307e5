"""PhysicsState recovery files (Framework/BasePhysicsFramework.h:127-319): the JSON the
reference's writeOutputs produces and recoverFromState reads, in its "text" form
(meshesState list of {velocities, position}) and its "binary" form (nMeshes, nVerts and
two raw FP32 files <name>.vel / <name>.pos next to the JSON).

Checks: the written files have the reference's keys and sizes; loading restores
positions and velocities to their FP32 values exactly, plus frameId; a run continued
from a text file and one continued from the binary file of the same state are
bit-identical; a state continued after loading follows the uninterrupted run; a file
whose vertex count does not match the scene is rejected."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tet(tmp_path, precision="fp64"):
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp = scenes.drop_cube(str(tmp_path), n=6, iterations=8, height=0.01)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
    phys.initialize()
    return phys, mp, pp


def _check_text(path, nv, frame):
    j = json.load(open(path))
    assert j["format"] == "text" and j["frameId"] == frame
    assert len(j["meshesState"]) == len(nv)
    for m, n in enumerate(nv):
        assert len(j["meshesState"][m]["position"]) == n
        assert len(j["meshesState"][m]["velocities"]) == n
        assert all(len(p) == 3 for p in j["meshesState"][m]["position"])
    return j


def _check_binary(path, nv, frame):
    j = json.load(open(path))
    assert j["format"] == "binary" and j["frameId"] == frame and j["nMeshes"] == len(nv)
    ms = j["meshesState"]
    assert ms["nVerts"] == list(nv)
    d = os.path.dirname(path)
    stem = os.path.splitext(os.path.basename(path))[0]
    assert ms["position_file"] == stem + ".pos" and ms["velocities_file"] == stem + ".vel"
    assert os.path.getsize(os.path.join(d, ms["position_file"])) == 12 * sum(nv)
    assert os.path.getsize(os.path.join(d, ms["velocities_file"])) == 12 * sum(nv)
    return j


def test_tet_state_round_trip(tmp_path, gaia_lib):
    from gaia_gb300 import VBDPhysics, scenes

    phys, mp, pp = _tet(tmp_path)
    phys.runStep(10)
    x10, v10 = phys.positions(0), phys.velocities(0)
    tp, bp = str(tmp_path / "A00010.json"), str(tmp_path / "B00010.json")
    phys.saveState(tp)
    phys.saveState(bp, binary=True)
    nv = [phys.numVertices(0)]
    j = _check_text(tp, nv, 10)
    _check_binary(bp, nv, 10)
    assert abs(j["curTime"] - 10 * json.load(open(pp))["PhysicsParams"]["timeStep"]) < 1e-12
    np.testing.assert_array_equal(np.array(j["meshesState"][0]["position"], np.float32), x10.astype(np.float32))

    phys.runStep(5)
    x15 = phys.positions(0)
    for path in (tp, bp):
        phys.recoverFromState(path)
        assert phys.frameId == 10
        np.testing.assert_array_equal(phys.positions(0), x10.astype(np.float32).astype(np.float64))
        np.testing.assert_array_equal(phys.velocities(0), v10.astype(np.float32).astype(np.float64))

    # continue from the text file and from the binary file in fresh handles: identical
    ends = []
    for path in (tp, bp):
        q = VBDPhysics()
        q.loadRunningparameters(mp, scenes.set_precision(pp, "fp64"))
        q.initialize()
        q.recoverFromState(path)
        q.runStep(5)
        ends.append(q.positions(0))
        q.close()
    np.testing.assert_array_equal(ends[0], ends[1])
    # and it follows the uninterrupted run up to the FP32 rounding of the saved state
    motion = np.linalg.norm(x15 - x10)
    assert np.linalg.norm(ends[0] - x15) <= 1e-3 * motion + 1e-6 * np.sqrt(x15.size)
    phys.close()


def test_tet_state_rejects_wrong_vertex_count(tmp_path, gaia_lib):
    from gaia_gb300 import GaiaError

    phys, _, _ = _tet(tmp_path)
    nv = phys.numVertices(0)
    bad = {"frameId": 3, "curTime": 0.1, "format": "text",
           "meshesState": [{"velocities": [[0.0, 0.0, 0.0]] * (nv - 1), "position": [[0.0, 0.0, 0.0]] * (nv - 1)}]}
    p = str(tmp_path / "bad.json")
    json.dump(bad, open(p, "w"))
    x = phys.positions(0)
    with pytest.raises(GaiaError):
        phys.recoverFromState(p)
    np.testing.assert_array_equal(phys.positions(0), x)
    phys.close()


def test_cloth_state_round_trip(tmp_path, gaia_lib):
    from gaia_gb300 import VBDClothSimulationFramework, scenes

    mp, pp = scenes.cloth_on_sphere(str(tmp_path), n=12, side=0.36, sphere_radius=0.12, sphere_level=2,
                                    contact_radius=0.01, iterations=6, dt=1.0 / 300.0, bending=1e-3,
                                    gap=0.004, precision="fp32")

    def engine():
        c = VBDClothSimulationFramework()
        c.loadRunningparameters(mp, pp)
        c.initialize()
        return c

    c = engine()
    c.runStep(4)
    x4, v4 = c.positions(0), c.velocities(0)
    tp, bp = str(tmp_path / "C00004.json"), str(tmp_path / "D00004.json")
    c.saveState(tp)
    c.saveState(bp, binary=True)
    nv = [c.numVertices(0)]
    _check_text(tp, nv, 4)
    _check_binary(bp, nv, 4)
    c.runStep(4)
    x8 = c.positions(0)
    c.recoverFromState(bp)
    np.testing.assert_array_equal(c.positions(0), x4.astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(c.velocities(0), v4.astype(np.float32).astype(np.float64))
    c.close()

    ends = []
    for path in (tp, bp):
        q = engine()
        q.recoverFromState(path)
        q.runStep(4)
        ends.append(q.positions(0))
        q.close()
    np.testing.assert_array_equal(ends[0], ends[1])
    motion = np.linalg.norm(x8 - x4)
    assert np.linalg.norm(ends[0] - x8) <= 1e-3 * motion, (np.linalg.norm(ends[0] - x8), motion)


def _read_ply(path):
    with open(path) as f:
        lines = f.read().splitlines()
    assert lines[0] == "ply" and lines[1] == "format ascii 1.0"
    nv = int(next(l for l in lines if l.startswith("element vertex")).split()[2])
    fl = [l for l in lines if l.startswith("element face")]
    nf = int(fl[0].split()[2]) if fl else 0
    body = lines[lines.index("end_header") + 1:]
    X = np.array([[float(t) for t in l.split()] for l in body[:nv]]).reshape(-1, 3)
    F = np.array([[int(t) for t in l.split()] for l in body[nv:nv + nf]], np.int64).reshape(-1, 4)
    assert (F[:, 0] == 3).all()
    return X, F[:, 1:]


def test_tet_output_frames(tmp_path, gaia_lib):
    """PLY (one per mesh, one for all) and raw FP32 frames of the tet surfaces."""
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp = scenes.stack_drop(str(tmp_path / "s"), spacing=0.02, precision="fp64")
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    phys.initialize()
    phys.runStep(3)
    out = tmp_path / "out"
    out.mkdir()
    phys.writePLY(str(out / "A00000003.ply"))
    phys.writePLY(str(out / "B00000003.ply"), saveAllModelsTogether=True)
    phys.writePLY(str(out / "C00000003.ply"), addModelName=True)
    phys.writeBinary(str(out / "A00000003.bin"))
    allX, allF, off = [], [], 0
    for m in range(2):
        F, V = phys.surface(m)
        x = phys.positions(m)[V]
        local = -np.ones(phys.numVertices(m), np.int64)
        local[V] = np.arange(len(V))
        Xp, Fp = _read_ply(str(out / f"A00000003_Model_{m:06d}.ply"))
        assert np.abs(Xp - x).max() <= 6e-7
        np.testing.assert_array_equal(Fp, local[F])
        name = ["lower", "upper"][m]
        assert (out / f"C00000003_Model_{m:06d}_{name}.ply").exists()
        allX.append(x)
        allF.append(local[F] + off)
        off += len(V)
    Xa, Fa = _read_ply(str(out / "B00000003.ply"))
    assert np.abs(Xa - np.concatenate(allX)).max() <= 6e-7
    np.testing.assert_array_equal(Fa, np.concatenate(allF))
    b = np.fromfile(str(out / "A00000003.bin"), np.float32).reshape(-1, 3)
    np.testing.assert_array_equal(b, np.concatenate(allX).astype(np.float32))
    phys.close()


def test_cloth_output_frames(tmp_path, gaia_lib):
    from gaia_gb300 import VBDClothSimulationFramework, scenes

    mp, pp = scenes.cloth_on_sphere(str(tmp_path / "s"), n=10, side=0.3, sphere_radius=0.1, sphere_level=2,
                                    contact_radius=0.01, iterations=4, dt=1.0 / 300.0, gap=0.004)
    c = VBDClothSimulationFramework()
    c.loadRunningparameters(mp, pp)
    c.initialize()
    c.runStep(2)
    out = tmp_path / "out"
    out.mkdir()
    c.writePLY(str(out / "A00000002.ply"))
    c.writeBinary(str(out / "A00000002.bin"))
    x = c.positions(0)
    Xp, Fp = _read_ply(str(out / "A00000002Model_0000_.ply"))
    assert np.abs(Xp - x).max() <= 6e-7
    assert Fp.shape[0] == c.numFaces(0)
    b = np.fromfile(str(out / "A00000002.bin"), np.float32).reshape(-1, 3)
    np.testing.assert_array_equal(b, x.astype(np.float32))
    c.close()
