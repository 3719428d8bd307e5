"""The oracle itself (CPU): its per-vertex force and Hessian are the derivatives
of its energy (the reference validates its element the same way with finite
differences, VBD_NeoHookean.cpp:1536-1611), its FP64 step is deterministic and
independent of the thread count, and basic physics holds (free fall, rest)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def free_scene(tmp_path_factory, gaia_lib):
    from gaia_gb300 import scenes

    d = tmp_path_factory.mktemp("free")
    X, T = scenes.lattice_cube((4, 4, 4), 0.01, jitter=1e-4, seed=5)
    tp, cp = scenes._write_mesh(str(d), "m", X, T)
    models = [scenes.model_entry(tp, cp, E=2e5, nu=0.35, density=800.0)]
    return scenes._write_json(str(d), models, scenes.physics_params(1 / 300, 5))  # no ground


def test_force_hessian_are_energy_derivatives(free_scene, oracle_lib):
    from oracle import scene_io

    mp, pp = free_scene
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 1)
    rng = np.random.Generator(np.random.PCG64(1))
    x = o.positions(0) + rng.uniform(-1.5e-3, 1.5e-3, size=(64, 3))
    o.set_positions(0, x)
    h = 1e-7
    for v in (0, 21, 42, 63):
        f, H = o.vertex_force_hessian(0, v, False)
        g = np.zeros(3)
        Hfd = np.zeros((3, 3))
        for k in range(3):
            xp, xm = x.copy(), x.copy()
            xp[v, k] += h
            xm[v, k] -= h
            o.set_positions(0, xp)
            ep = o.energy()
            fp, _ = o.vertex_force_hessian(0, v, False)
            o.set_positions(0, xm)
            em = o.energy()
            fm, _ = o.vertex_force_hessian(0, v, False)
            g[k] = (ep - em) / (2 * h)
            Hfd[:, k] = -(fp - fm) / (2 * h)
        o.set_positions(0, x)
        assert np.allclose(f, -g, rtol=1e-5, atol=1e-6 * np.abs(H).max() * h), (v, f, -g)
        assert np.allclose(H, Hfd, rtol=1e-5, atol=1e-7 * np.abs(H).max()), (v, H, Hfd)
        assert np.allclose(H, H.T, rtol=1e-12, atol=1e-9 * np.abs(H).max())


def test_rest_state_has_no_elastic_force(free_scene, oracle_lib):
    from oracle import scene_io

    mp, pp = free_scene
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 1)
    for v in range(0, 64, 9):
        f, H = o.vertex_force_hessian(0, v, False)
        assert np.abs(f).max() < 1e-9 * np.abs(H).max()


def test_free_fall(free_scene, oracle_lib):
    """Without ground, every vertex follows x0 + g t^2/2 (implicit Euler: dt^2 g k(k+1)/2)."""
    from oracle import scene_io

    mp, pp = free_scene
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 2)
    x0 = o.positions(0)
    k = 12
    o.step(k)
    dt = 1 / 300
    expect = -9.8 * dt * dt * k * (k + 1) / 2
    dy = o.positions(0)[:, 1] - x0[:, 1]
    assert np.allclose(dy, expect, rtol=1e-7)


def test_deterministic_across_thread_counts(tmp_path, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes
    from oracle import scene_io

    mp, pp = scenes.drop_cube(str(tmp_path), n=6, iterations=6, height=0.005)
    sc = scene_io.load_scene(mp, pp)
    a = oracle_lib.OracleScene(sc, 64, 1)
    b = oracle_lib.OracleScene(sc, 64, 4)
    a.step(15)
    b.step(15)
    assert np.array_equal(a.positions(0), b.positions(0))
    assert np.array_equal(a.velocities(0), b.velocities(0))


def test_fp32_oracle_close_to_fp64(tmp_path, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes
    from oracle import scene_io

    mp, pp = scenes.twist_cube(str(tmp_path), n=6, iterations=10)
    sc = scene_io.load_scene(mp, pp)
    a = oracle_lib.OracleScene(sc, 64, 2)
    b = oracle_lib.OracleScene(sc, 32, 2)
    x0 = a.positions(0)
    a.step(10)
    b.step(10)
    rel = np.linalg.norm(b.positions(0) - a.positions(0)) / np.linalg.norm(a.positions(0) - x0)
    assert rel < 1e-3


def test_twist_deformer_moves_end_face(tmp_path, gaia_lib, oracle_lib):
    """The Rotator deformer turns the x-max face about the x axis at omega (VBDDeformer.h:75-130)."""
    from gaia_gb300 import scenes
    from oracle import scene_io

    n = 5
    mp, pp = scenes.twist_cube(str(tmp_path), n=n, iterations=4, omega=2.0)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 1)
    x0 = o.positions(0)
    o.step(30)
    x = o.positions(0)
    idx = np.arange(n ** 3)
    right = idx[idx % n == n - 1]
    left = idx[idx % n == 0]
    th = 2.0 * 30 / 300
    c, s = np.cos(th), np.sin(th)
    y0, z0 = x0[right, 1], x0[right, 2]
    assert np.allclose(x[right, 1], c * y0 - s * z0, atol=1e-6)
    assert np.allclose(x[right, 2], s * y0 + c * z0, atol=1e-6)
    assert np.allclose(x[left], x0[left])


def test_chebyshev_weights():
    """getAcceleratorOmega (VBDPhysics.cpp:3558-3574)."""
    rho = 0.93
    w = [1.0]
    w.append(2 / (2 - rho * rho))
    for _ in range(30):
        w.append(4 / (4 - rho * rho * w[-1]))
    # the recurrence converges to the fixed point of w = 4 / (4 - rho^2 w)
    w_star = 2 * (1 - np.sqrt(1 - rho * rho)) / (rho * rho)
    err = [abs(x - w_star) for x in w[1:]]
    assert all(b < a for a, b in zip(err, err[1:]))
    assert err[-1] < 1e-6 and 1.0 < w_star < 2.0
