"""Jones-Plassmann vertex coloring on the GPU: a proper coloring of the tet vertex graph
(no two vertices of one tet share a color), deterministic for a seed, with a color count
of the order of the library's greedy coloring; and a scene colored this way steps like
one colored by the reference's algorithm (the oracle runs it with the same coloring)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _proper(T, col):
    for i in range(4):
        for j in range(i + 1, 4):
            assert not np.any(col[T[:, i]] == col[T[:, j]])


@pytest.mark.parametrize("shape", [(7, 5, 6), (20, 20, 20)])
def test_gpu_coloring_proper(shape, gaia_lib):
    from gaia_gb300 import color_gpu, color_greedy, scenes

    X, T = scenes.lattice_cube(shape, 0.01, jitter=1e-4, seed=3)
    c1 = color_gpu(len(X), T, seed=1)
    c2 = color_gpu(len(X), T, seed=1)
    np.testing.assert_array_equal(c1, c2)
    _proper(T, c1)
    assert c1.min() == 0
    ng = int(color_greedy(len(X), T).max()) + 1
    assert int(c1.max()) + 1 <= 2 * ng + 4
    c3 = color_gpu(len(X), T, seed=7)
    _proper(T, c3)


def test_gpu_coloring_ball_and_errors(gaia_lib):
    from gaia_gb300 import color_gpu, scenes

    X, T = scenes.lattice_ball(0.05, 0.008, jitter=1e-5, seed=2)
    c = color_gpu(len(X), T, seed=3)
    _proper(T, c)
    bad = T.copy()
    bad[0, 0] = len(X) + 5
    with pytest.raises(RuntimeError):
        color_gpu(len(X), bad, seed=3)


def test_scene_with_gpu_coloring_matches_oracle(tmp_path, gaia_lib, oracle_lib):
    from gaia_gb300 import VBDPhysics, color_gpu, physics, scenes
    from oracle import scene_io

    X, T = scenes.lattice_cube((6, 6, 6), 0.01, (0.0, 0.02, 0.0), jitter=1e-4, seed=4)
    tp = str(tmp_path / "m.t")
    physics.write_t(tp, X, T)
    cp = tp + ".vertexColoring.json"
    physics.write_coloring(cp, color_gpu(len(X), T, seed=11))
    mp, pp = scenes._write_json(str(tmp_path), [scenes.model_entry(tp, cp)],
                                scenes.physics_params(1 / 300, 10, ground_y=0.0, precision="fp64"))
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 0)
    o.step(10)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    phys.initialize()
    x0 = phys.positions(0)
    phys.runStep(10)
    x = phys.positions(0)
    xr = o.positions(0)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr - x0) <= 1e-9
    phys.close()
