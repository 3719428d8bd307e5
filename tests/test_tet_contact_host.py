"""Tet-mesh contact, host side: the oracle's FP32 CCD restatement against the
reference's own CCD test (golden vectors from the reference build, and the build
itself where the reference tree is present), surface extraction of the product vs the
oracle, and the oracle's contact behaviour on a stacked-cube scene."""
import ctypes as C
import json
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _ref_tree():
    from oracle.oracle import reference_root

    root = reference_root()
    return os.path.join(root, "Simulator", "Modules", "CollisionDetector", "CCDSolver.h") if root else ""


REF_TREE = _ref_tree()


def _oracle_ccd(x0, x1, p0, p1):
    from oracle import oracle as orc

    fp = C.POINTER(C.c_float)
    fn = orc.lib().oracle_ccd_tri_point
    n = len(x0)
    hit = np.zeros(n, np.int32)
    tt = np.zeros(n, np.float32)
    bary = np.zeros((n, 3), np.float32)
    t = np.zeros(1, np.float32)
    b = np.zeros(3, np.float32)
    for k in range(n):
        args = [np.ascontiguousarray(v[k], np.float32) for v in (x0, x1, p0, p1)]
        hit[k] = fn(*[v.ctypes.data_as(fp) for v in args], t.ctypes.data_as(fp), b.ctypes.data_as(fp))
        tt[k] = t[0]
        bary[k] = b
    return hit, tt, bary


def _same(a_hit, a_tt, a_bary, b_hit, b_tt, b_bary):
    assert np.array_equal(a_hit, b_hit)
    h = a_hit == 1
    assert a_tt[h].tobytes() == b_tt[h].tobytes()
    assert a_bary[h].tobytes() == b_bary[h].tobytes()


def test_ccd_matches_reference_golden_vectors():
    """tests/golden/ccd_vectors.npz holds the reference CCDSolver.h's own outputs."""
    g = np.load(os.path.join(HERE, "golden", "ccd_vectors.npz"))
    hit, tt, bary = _oracle_ccd(g["x0"], g["x1"], g["p0"], g["p1"])
    assert g["hit"].sum() > 500
    _same(hit, tt, bary, g["hit"], g["tt"], g["bary"])


@pytest.mark.skipif(not os.path.exists(REF_TREE), reason="reference tree not present")
def test_ccd_matches_reference_build_fresh_cases():
    import importlib.util

    spec = importlib.util.spec_from_file_location("mk", os.path.join(HERE, "golden", "make_ccd_vectors.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "..", "oracle"), "ref"], check=True)
    lib = C.CDLL(os.path.join(HERE, "..", "oracle", "_ref", "libccd_ref.so"))
    fn = lib.ref_ccd_tri_point
    fn.argtypes = [C.POINTER(C.c_float)] * 6
    fn.restype = C.c_int32
    x0, x1, p0, p1 = mk.cases(5000, seed=123)
    _same(*_oracle_ccd(x0, x1, p0, p1), *mk.evaluate(fn, x0, x1, p0, p1))


def _surface_invariants(X, tets, F, V):
    # closed 2-manifold: every undirected edge in two faces, used once in each direction
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    directed = {tuple(x) for x in e.tolist()}
    assert len(directed) == len(e)
    assert all((b, a) in directed for a, b in directed)
    assert len(V) - len(directed) // 2 + len(F) == 2  # Euler characteristic of a sphere
    assert np.array_equal(np.unique(F), V)
    # outward: the surface encloses the tets' total volume (divergence theorem)
    a, b, c = X[F[:, 0]], X[F[:, 1]], X[F[:, 2]]
    enclosed = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    d = X[tets[:, 1:]] - X[tets[:, :1]]
    vol = np.abs(np.einsum("ij,ij->i", d[:, 0], np.cross(d[:, 1], d[:, 2]))).sum() / 6.0
    assert enclosed == pytest.approx(vol, rel=1e-9)


def test_surface_matches_oracle(tmp_path, gaia_lib):
    from gaia_gb300 import VBDPhysics, scenes
    from oracle import oracle as orc
    from oracle import scene_io

    mp, pp = scenes.stack_drop(str(tmp_path), n_lower=5, n_upper=4, spacing=0.02)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)  # host only
    sc = scene_io.load_scene(mp, pp)
    for m, mesh in enumerate(sc["meshes"]):
        F, V = phys.surface(m)
        Fo, Vo = orc.tet_surface(mesh["X"], mesh["tets"])
        assert np.array_equal(F, Fo) and np.array_equal(V, Vo)
        _surface_invariants(mesh["X"], mesh["tets"], F, V)
    phys.close()


def test_surface_of_mirrored_mesh_is_outward(tmp_path, gaia_lib):
    """Negatively oriented tets (a mirrored mesh) still give outward faces."""
    from gaia_gb300 import VBDPhysics, scenes
    from oracle import oracle as orc

    X, T = scenes.lattice_cube((4, 3, 5), 0.02, jitter=1e-3, seed=5)
    T = T[:, [0, 2, 1, 3]]  # every tet negatively oriented
    tp, cp = scenes._write_mesh(str(tmp_path), "m", X, T)
    mp, pp = scenes._write_json(str(tmp_path), [scenes.model_entry(tp, cp)], scenes.physics_params(0.01, 2))
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    F, V = phys.surface(0)
    Xf = X.astype(np.float32).astype(np.float64)
    Fo, Vo = orc.tet_surface(Xf, T)
    assert np.array_equal(F, Fo) and np.array_equal(V, Vo)
    _surface_invariants(Xf, T, F, V)
    phys.close()


def _run_stack(tmp_path, spacing, steps):
    from gaia_gb300 import scenes
    from oracle import oracle as orc
    from oracle import scene_io

    mp, pp = scenes.stack_drop(str(tmp_path), spacing=spacing, gap=0.01, speed=1.0)
    o = orc.OracleScene(scene_io.load_scene(mp, pp), 64, 0)
    kinds = set()
    for _ in range(steps):
        o.step(1)
        kinds |= set(o.contacts()[:, 7].tolist())
    return o, kinds


def test_oracle_stack_rests_on_contact(tmp_path):
    """3 cm cells: the point-in-tet test is live (|6V| >= 1e-5), DCD holds the upper cube."""
    o, kinds = _run_stack(tmp_path, 0.03, 40)
    assert 2 in kinds
    lower, upper = o.positions(0), o.positions(1)
    assert upper[:, 1].min() > lower[:, 1].max() - 0.005


def test_oracle_stack_small_cells_ccd_only(tmp_path):
    """1 cm cells: |6V| < CMP_EPSILON = 1e-5 for every tet, so the reference's point-in-tet
    test never fires and only CCD contacts occur (penalty contact cannot hold a body that
    stays below the surface after a substep)."""
    o, kinds = _run_stack(tmp_path, 0.01, 15)
    assert kinds and kinds <= {1}


# ---- the DCD closest-point query's tetrahedral traversal (oracle) ------------------------

def _walk_case(X, T, f, t, F, max_mult=1.8, shift=0.0):
    """Ray from the centroid of surface face f toward the centroid of tet t, in FP32."""
    from oracle import oracle as orc

    o = X[F[f]].astype(np.float32).mean(0)
    tgt = X[T[t]].astype(np.float32).mean(0)
    d = (tgt - o).astype(np.float32)
    L = np.float32(np.linalg.norm(d))
    return orc.tet_walk(X, T, int(f), int(t), o, d / L, float(max_mult * L) if max_mult > 0 else -1.0)


def test_walk_reaches_every_tet_of_a_convex_mesh(oracle_lib):
    """Exact lattice (convex, with rays through edges and vertices): every walk from a
    surface face's centroid to a tet's centroid arrives, static and dynamic. On a
    jittered lattice, rays that leave through the start face itself (the target lies on
    its outer side) find no exit face and fail."""
    from gaia_gb300 import scenes
    from oracle import oracle as orc

    X, T = scenes.lattice_cube((5, 5, 5), 0.1)
    F, _ = orc.tet_surface(X, T)
    rng = np.random.default_rng(0)
    for f in rng.choice(len(F), 30, replace=False):
        for t in rng.choice(len(T), 8, replace=False):
            assert _walk_case(X, T, f, t, F) == (True, False), (f, t)
            o = X[F[f]].astype(np.float32).mean(0)
            d = X[T[t]].astype(np.float32).mean(0) - o
            ok, bound = orc.tet_walk(X, T, int(f), int(t), o, d / np.linalg.norm(d), -1.0, use_static=False)
            assert ok and not bound, (f, t)
    X, T = scenes.lattice_cube((5, 5, 5), 0.1, jitter=0.01, seed=4)
    F, _ = orc.tet_surface(X, T)
    outward = 0
    for f in rng.choice(len(F), 60, replace=False):
        a, b, c = X[F[f]]
        n = np.cross(b - a, c - a)
        for t in rng.choice(len(T), 8, replace=False):
            ok, _ = _walk_case(X, T, f, t, F)
            if np.dot(n, X[T[t]].mean(0) - (a + b + c) / 3) > 0:
                outward += 1
                assert not ok, (f, t)
    assert outward > 0


def test_walk_stops_at_the_boundary_of_a_nonconvex_mesh(oracle_lib):
    """An L-shaped block: the ray from one arm to the other crosses the notch (outside the
    mesh), so the walk reaches the boundary; within one arm it arrives."""
    from gaia_gb300 import scenes
    from oracle import oracle as orc

    X, T = scenes.lattice_cube((6, 6, 3), 0.1)
    cen = X[T].mean(1)
    T = T[~((cen[:, 0] > 0.2) & (cen[:, 1] > 0.2))]
    cen = X[T].mean(1)
    F, _ = orc.tet_surface(X, T)
    fc = X[F].mean(1)
    # start: a face on the top of arm B (y = 0.2, x > 0.35); targets in arm A (x < 0.2, y > 0.4)
    starts = np.where((np.abs(fc[:, 1] - 0.2) < 1e-9) & (fc[:, 0] > 0.35))[0]
    far = np.where((cen[:, 0] < 0.15) & (cen[:, 1] > 0.4))[0]
    near = np.where((cen[:, 0] > 0.3) & (cen[:, 1] < 0.1))[0]
    assert len(starts) and len(far) and len(near)
    for f in starts[:4]:
        for t in far[:6]:
            ok, bound = _walk_case(X, T, f, t, F, max_mult=-1)
            assert not ok and not bound, (f, t)
        for t in near[:6]:
            ok, bound = _walk_case(X, T, f, t, F)
            assert ok, (f, t)


def test_walk_pass_through_limit(oracle_lib):
    """maxSearchDistanceMultiplier: a walk that crosses an exit face farther than
    max_dis from the origin (checked every fifth tet) gives up."""
    from gaia_gb300 import scenes
    from oracle import oracle as orc

    X, T = scenes.lattice_cube((7, 7, 7), 0.1, jitter=0.005, seed=2)
    F, _ = orc.tet_surface(X, T)
    fc, cen = X[F].mean(1), X[T].mean(1)
    f = int(np.argmin(np.linalg.norm(fc - np.array([0.3, 0.3, 0.0]), axis=1)))  # bottom face, middle
    t = int(np.argmin(np.linalg.norm(cen - np.array([0.3, 0.3, 0.55]), axis=1)))  # near the top
    assert _walk_case(X, T, f, t, F, max_mult=1.8)[0]
    assert not _walk_case(X, T, f, t, F, max_mult=0.3)[0]


def _deep_state_rows(tmp_path, collision):
    """Contact rows of the oracle for the 3 cm stacked cubes with the upper cube's bottom
    layers pushed into the lower one (every point-in-tet test live)."""
    from gaia_gb300 import scenes
    from oracle import oracle as orc
    from oracle import scene_io

    mp, pp = scenes.stack_drop(str(tmp_path), spacing=0.03, gap=0.01, speed=1.0)
    P = json.load(open(pp))
    P["CollisionParams"] = collision
    json.dump(P, open(pp, "w"))
    o = orc.OracleScene(scene_io.load_scene(mp, pp), 64, 0)
    X0, X1 = o.positions(0), o.positions(1)
    deep = np.float32(np.array([0.0, -0.05, 0.0]))
    rng = np.random.default_rng(5)
    X1d = (X1 + deep + rng.normal(0, 0.002, X1.shape)).astype(np.float32).astype(np.float64)
    o.set_prev_positions(0, X0)
    o.set_prev_positions(1, X1d)
    o.set_positions(1, X1d)
    o.collide()
    return o.contacts()


def test_traversal_accepts_the_nearest_face_of_convex_meshes(tmp_path, oracle_lib):
    """For convex bodies the straight path from the nearest feasible face to an inner point
    stays inside, so the check changes nothing; a pass-through limit far below the path
    length rejects faces, which changes the rows."""
    on = _deep_state_rows(tmp_path / "a", {})
    off = _deep_state_rows(tmp_path / "b", {"checkTetTraverse": False})
    short = _deep_state_rows(tmp_path / "c", {"maxSearchDistanceMultiplier": 0.05})
    assert len(on) > 20 and (on[:, 7] == 2).sum() > 10
    np.testing.assert_array_equal(on, off)
    assert not np.array_equal(on, short)
