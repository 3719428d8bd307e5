"""The benchmark's two scene writers give the same scene: the product library's (`.t`
writer, the coloring tool's colorings) for the GPU arm, and the plain-Python writers with
the oracle's colorings for the CPU reference arm, which must not load the product library.
Same vertices, tets, coloring categories and parameters, so that both arms time the same
configuration.
"""
import json
import os

import numpy as np
import pytest


def _make(kind, d):
    from gaia_gb300 import scenes

    if kind == "drop":
        return scenes.drop_cube(d, n=6, iterations=3, coloring="greedy", collision=scenes.NO_CONTACT)
    if kind == "twist":
        return scenes.twist_cube(d, n=7, iterations=3)
    if kind == "batch":
        return scenes.batch_cubes(d, n_scenes=5, side_range=(3, 6), iterations=3)
    return scenes.collision_drop(d, n_objects=4, iterations=3, cube_sides=(4, 6), ball_radii=(0.03, 0.04),
                                 ball_tets=(300, 600))


def _read_t(path):
    X, T = [], []
    for line in open(path):
        p = line.split()
        if p and p[0] == "Vertex":
            X.append([float(v) for v in p[2:5]])
        elif p and p[0] == "Tet":
            T.append([int(v) for v in p[2:6]])
    return np.array(X), np.array(T)


def _strip(obj, root):
    """The JSON with the writer's directory taken out of every path."""
    if isinstance(obj, dict):
        return {k: _strip(v, root) for k, v in obj.items()}
    if isinstance(obj, list):
        return [_strip(v, root) for v in obj]
    if isinstance(obj, str):
        return obj.replace(root, "<dir>")
    return obj


@pytest.mark.parametrize("kind", ["drop", "twist", "batch", "collide"])
def test_oracle_writer_equals_library_writer(tmp_path, gaia_lib, oracle_lib, kind):
    from gaia_gb300 import scenes

    da, db = str(tmp_path / "library"), str(tmp_path / "oracle")
    try:
        scenes.set_writer("library")
        mpa, ppa = _make(kind, da)
        scenes.set_writer("oracle")
        mpb, ppb = _make(kind, db)
    finally:
        scenes.set_writer("library")
    ma, mb = json.load(open(mpa)), json.load(open(mpb))
    assert _strip(ma, da) == _strip(mb, db)
    assert _strip(json.load(open(ppa)), da) == _strip(json.load(open(ppb)), db)
    models = ma["Models"]
    assert models
    for m in models:
        ta, tb = m["path"], m["path"].replace(da, db)
        Xa, Ta = _read_t(ta)
        Xb, Tb = _read_t(tb)
        np.testing.assert_array_equal(Ta, Tb)
        np.testing.assert_array_equal(Xa, Xb)
        ca = m["verticesColoringCategoriesPath"]
        assert json.load(open(ca)) == json.load(open(ca.replace(da, db))), (kind, os.path.basename(ta))


def test_stored_colorings_equal_the_library_tool(gaia_lib, oracle_lib):
    """The stored colorings the reference arm reads for the two meshes too large for the
    oracle's O(V^2) coloring tool (the 100^3 twist lattice, the 512 x 512 cloth) are the
    library's tool colorings of those meshes, as the GPU arm's scene writer makes them."""
    from gaia_gb300 import physics, scenes
    from gaia_gb300.cloth import color_trimesh_tool
    from oracle import scene_colorings

    n = 100
    half = 0.5 * 0.01 * (n - 1)
    X, T = scenes.lattice_cube((n, n, n), 0.01, (0.0, -half, -half), jitter=1e-4, seed=1)
    colors, order = physics.color_tool(len(X), T)
    stored = scene_colorings.stored(len(X), T, "tet_tool")
    assert stored is not None
    np.testing.assert_array_equal(colors, stored[0])
    np.testing.assert_array_equal(order, stored[1])
    Xc, F = scenes.cloth_grid(512, 1.0, 0.3 + 0.01, 1e-3, 1)
    colors, order = color_trimesh_tool(len(Xc), F)
    stored = scene_colorings.stored(len(Xc), F, "tri_tool")
    assert stored is not None
    np.testing.assert_array_equal(colors, stored[0])
    np.testing.assert_array_equal(order, stored[1])
