"""Host-side logic of libgaia_vbd.so (CPU only, no GPU needed): the exported C
ABI, Models.json/Parameters.json loading with the reference's defaults, rest
shape, parallel-group merge, error codes, and the synthetic scene writer."""
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    syms = set()
    for h in ("gaia_vbd.h", "gaia_cloth.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        syms |= set(re.findall(r"\b(gaia_(?:vbd|cloth)_[a-z0-9_]+)\s*\(", text))
    return sorted(syms)


def test_library_exports_every_declared_symbol(gaia_lib):
    import ctypes

    from gaia_gb300 import _lib

    L = ctypes.CDLL(_lib.LIB_PATH)
    syms = _header_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(L, s), s
    # the Python binding declares a signature for each of them
    assert set(syms) == set(_lib.exported_symbols())


def _load(mp, pp):
    from gaia_gb300 import VBDPhysics

    p = VBDPhysics()
    p.loadRunningparameters(mp, pp)
    return p


def test_groups_and_rest_shape_match_oracle(tmp_path, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes
    from oracle import scene_io

    mp, pp = scenes.batch_cubes(str(tmp_path), n_scenes=9, side_range=(3, 6), iterations=5)
    p = _load(mp, pp)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 1)
    g1, g2 = p.parallelGroups(), o.groups()
    assert len(g1) == len(g2)
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)
    for m in range(p.numMeshes()):
        d1, v1, m1 = p.restShape(m)
        d2, v2, m2 = o.rest(m)
        assert np.array_equal(d1, d2) and np.array_equal(v1, v2) and np.array_equal(m1, m2)
    p.close()


def test_transforms_match_python_loader(tmp_path, gaia_lib, oracle_lib):
    """rotation (axis-angle), scale and translation applied in FP32 like TetMeshFEM.cpp:359-384."""
    from gaia_gb300 import scenes
    from oracle import scene_io

    X, T = scenes.lattice_cube((4, 3, 5), 0.02, jitter=1e-4, seed=2)
    tp, cp = scenes._write_mesh(str(tmp_path), "m", X, T)
    models = [scenes.model_entry(tp, cp, rotation=[0.3, -0.2, 0.5], scale=[1.5, 0.7, 1.1],
                                 translation=[0.1, 2.0, -0.3], density=700.0)]
    mp, pp = scenes._write_json(str(tmp_path), models, scenes.physics_params(0.01, 3))
    p = _load(mp, pp)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 1)
    d1, v1, m1 = p.restShape(0)
    d2, v2, m2 = o.rest(0)
    assert np.allclose(d1, d2, rtol=1e-12, atol=0) and np.allclose(v1, v2, rtol=1e-12) and np.allclose(m1, m2, rtol=1e-12)
    assert v1.min() > 0
    p.close()


def test_coloring_is_sorted_large_to_small(tmp_path, gaia_lib):
    from gaia_gb300 import scenes

    mp, pp = scenes.drop_cube(str(tmp_path), n=6)
    p = _load(mp, pp)
    col = p.coloring(0)
    sizes = np.bincount(col)
    assert np.all(np.diff(sizes) <= 0)
    groups = p.parallelGroups()
    assert [len(g) for g in groups] == list(sizes)
    p.close()


def test_missing_coloring_file_uses_greedy(tmp_path, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes

    X, T = scenes.lattice_cube((5, 4, 3), 0.01)
    tp, _ = scenes._write_mesh(str(tmp_path), "m", X, T)
    m = scenes.model_entry(tp, "")
    mp, pp = scenes._write_json(str(tmp_path), [m], scenes.physics_params(0.01, 2))
    p = _load(mp, pp)
    greedy = oracle_lib.color_greedy(len(X), T)
    cats = [np.flatnonzero(greedy == c) for c in range(greedy.max() + 1)]
    order = sorted(range(len(cats)), key=lambda c: -len(cats[c]))
    col = p.coloring(0)
    # same classes (the reference sorts them by size; equal sizes may reorder)
    for c in range(len(cats)):
        assert len(set(col[cats[c]])) == 1
    assert sorted(np.bincount(col)) == sorted(len(c) for c in cats)
    assert len(order) == col.max() + 1
    p.close()


def test_repo_root_substitution(tmp_path, gaia_lib):
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp = scenes.drop_cube(str(tmp_path / "scene"), n=4)
    M = json.load(open(mp))
    for m in M["Models"]:
        m["path"] = m["path"].replace(str(tmp_path), "${REPO_ROOT}")
        m["verticesColoringCategoriesPath"] = m["verticesColoringCategoriesPath"].replace(str(tmp_path), "${REPO_ROOT}")
    mp2 = str(tmp_path / "Models_root.json")
    json.dump(M, open(mp2, "w"))
    p = VBDPhysics()
    p.loadRunningparameters(mp2, pp, repo_root=str(tmp_path))
    assert p.numVertices(0) == 64
    p.close()


def _expect_error(mp, pp, code):
    from gaia_gb300 import GaiaError, VBDPhysics

    p = VBDPhysics()
    with pytest.raises(GaiaError) as e:
        p.loadRunningparameters(mp, pp)
    assert e.value.code == code, str(e.value)
    return str(e.value)


def test_error_codes(tmp_path, gaia_lib):
    from gaia_gb300 import _lib, scenes

    mp, pp = scenes.drop_cube(str(tmp_path), n=4)
    M = json.load(open(mp))
    # missing files
    _expect_error(str(tmp_path / "nope.json"), pp, _lib.E_INPUT)
    # malformed JSON
    bad = tmp_path / "bad.json"
    bad.write_text('{"Models": [ {"path": ')
    _expect_error(str(bad), pp, _lib.E_INPUT)
    # unsupported material
    M2 = json.loads(json.dumps(M))
    M2["Models"][0]["materialName"] = "MassSpring"
    p2 = tmp_path / "m2.json"
    json.dump(M2, open(p2, "w"))
    _expect_error(str(p2), pp, _lib.E_UNSUPPORTED)
    # fixed point out of range
    M3 = json.loads(json.dumps(M))
    M3["Models"][0]["fixedPoints"] = [1000]
    p3 = tmp_path / "m3.json"
    json.dump(M3, open(p3, "w"))
    _expect_error(str(p3), pp, _lib.E_MESH)
    # invalid coloring: two vertices of one tet in the same color
    cats = json.load(open(M["Models"][0]["verticesColoringCategoriesPath"]))
    cats[0] = cats[0] + cats[1]
    del cats[1]
    cbad = tmp_path / "cbad.json"
    json.dump(cats, open(cbad, "w"))
    M4 = json.loads(json.dumps(M))
    M4["Models"][0]["verticesColoringCategoriesPath"] = str(cbad)
    p4 = tmp_path / "m4.json"
    json.dump(M4, open(p4, "w"))
    _expect_error(str(p4), pp, _lib.E_COLORING)
    # coloring that misses a vertex
    cats = json.load(open(M["Models"][0]["verticesColoringCategoriesPath"]))
    cats[0] = cats[0][1:]
    json.dump(cats, open(cbad, "w"))
    _expect_error(str(p4), pp, _lib.E_COLORING)
    # degenerate tet (zero rest volume)
    X, T = scenes.lattice_cube((3, 3, 3), 0.01)
    X[T[0, 1]] = X[T[0, 0]]
    tp, cp = scenes._write_mesh(str(tmp_path / "deg"), "m", X, T)
    mp5, pp5 = scenes._write_json(str(tmp_path / "deg"), [scenes.model_entry(tp, cp)], scenes.physics_params(0.01, 2))
    _expect_error(mp5, pp5, _lib.E_MESH)
    # bad parameter values
    pbad = tmp_path / "pbad.json"
    for key, value in (("gpuPrecision", "fp16"), ("sweepMode", "tiles"), ("clusterSize", 3),
                       ("evaluationSteps", 0)):
        P = json.load(open(pp))
        P["PhysicsParams"][key] = value
        json.dump(P, open(pbad, "w"))
        _expect_error(mp, str(pbad), _lib.E_INPUT)
    # the engine keys beyond the reference's load on a host without a GPU
    for key, value in (("sweepMode", "grid"), ("sweepMode", "cluster"), ("meshFrames", False),
                       ("gpuPrecision", "dfhi"), ("solveVariant", 7), ("waitPollLimit", 0)):
        P = json.load(open(pp))
        P["PhysicsParams"][key] = value
        json.dump(P, open(pbad, "w"))
        _load(mp, str(pbad)).close()


def test_initialize_without_gpu_reports_no_device(tmp_path, gaia_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gaia_gb300 import GaiaError, _lib, scenes

    mp, pp = scenes.drop_cube(str(tmp_path), n=4)
    p = _load(mp, pp)
    with pytest.raises(GaiaError) as e:
        p.initialize()
    assert e.value.code == _lib.E_NO_DEVICE
    # calls that need the device state fail cleanly on a loaded-only handle
    with pytest.raises(GaiaError):
        p.runStep(1)
    p.close()


def test_lattice_is_conforming_and_positive():
    from gaia_gb300 import scenes

    X, T = scenes.lattice_cube((6, 5, 4), 0.01, jitter=1e-4, seed=1)
    assert len(T) == 5 * 5 * 4 * 3
    d = X[T[:, 1:]] - X[T[:, :1]]
    det = np.einsum("ij,ij->i", d[:, 0], np.cross(d[:, 1], d[:, 2]))
    assert det.min() > 0
    assert abs(det.sum() / 6 - 0.05 * 0.04 * 0.03) < 1e-6
    faces = np.sort(np.concatenate([T[:, [0, 1, 2]], T[:, [0, 1, 3]], T[:, [0, 2, 3]], T[:, [1, 2, 3]]]), axis=1)
    _, counts = np.unique(faces, axis=0, return_counts=True)
    assert counts.max() == 2
    boundary = 2 * (5 * 4 + 5 * 3 + 4 * 3) * 2
    assert (counts == 1).sum() == boundary


def test_lame_conversion():
    from gaia_gb300 import scenes

    mu, lm = scenes.lame(1e6, 0.4)
    assert abs(mu - 357142.857142857) < 1e-6 and abs(lm - 1428571.4285714) < 1e-4
