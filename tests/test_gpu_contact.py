"""Tet-mesh vertex-face contact on the GPU against the oracle.

- contact sets: the GPU detector (DCD point-in-tet + nearest feasible face reached by the
  tetrahedral traversal, CCD of the surface vertices' trajectories) returns exactly the
  oracle's rows on crafted states, with FP32-representable positions so that both see
  identical inputs, under the traversal's parameter variants;
- force and Hessian of vertices in contact (own contact and face-side relations) in
  the FP64 engine within 1e-9 of the oracle's;
- trajectories of a cube dropped on another (contacts appear, persist and change) in
  the FP64 engine within 1e-8 of the oracle, with the accelerator and with
  intermediate detection passes as variants; the mixed engine within 1e-4.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(tmp_path, spacing, precision="fp64", **extra):
    from gaia_gb300 import scenes

    return scenes.stack_drop(str(tmp_path), spacing=spacing, gap=0.01, speed=1.0, precision=precision, **extra)


def _pair(mp, pp):
    from gaia_gb300 import VBDPhysics
    from oracle import oracle as orc
    from oracle import scene_io

    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    phys.initialize()
    o = orc.OracleScene(scene_io.load_scene(mp, pp), 64, 0)
    return phys, o


def _f32(x):
    return np.asarray(x, np.float32).astype(np.float64)


def _states(X0, X1, spacing, seed=0):
    """(prev, current) position pairs for the two meshes, FP32-representable."""
    rng = np.random.default_rng(seed)
    out = []
    down = np.array([0.0, -0.6 * spacing, 0.0])
    deep = np.array([0.0, -1.2 * spacing, 0.0])
    # trajectories through the lower cube's top (CCD), starting from rest
    out.append(((X0, X1), (X0, X1 + down + np.array([0.0, -0.01, 0.0]))))
    # the upper cube's bottom layer already inside the lower cube (DCD), no motion
    out.append(((X0, X1 + deep), (X0, X1 + deep)))
    # both: inside at the start and moving further, with noise on every vertex
    n0 = rng.normal(0, 0.05 * spacing, X0.shape)
    n1 = rng.normal(0, 0.05 * spacing, X1.shape)
    out.append(((X0 + n0, X1 + deep + n1), (X0 + 0.5 * n0, X1 + 1.5 * deep - n1)))
    return [tuple(tuple(_f32(a) for a in pair) for pair in st) for st in out]


# CollisionParams variants of the DCD closest-point query's tetrahedral traversal: the
# reference defaults (on convex bodies it rejects nothing), a pass-through limit that
# makes walks give up (faces rejected), the dynamic walk alone, and the check off.
TRAVERSAL = {
    "default": {},
    "short": {"maxSearchDistanceMultiplier": 0.05},
    "dynamic": {"useStaticTraverse": False, "maxSearchDistanceMultiplier": 0.3},
    "off": {"checkTetTraverse": False},
}


@pytest.mark.parametrize("spacing,traversal", [(0.03, "default"), (0.01, "default"), (0.03, "short"),
                                               (0.03, "dynamic"), (0.03, "off")])
def test_contact_sets_bit_exact(spacing, traversal, tmp_path, gaia_lib, oracle_lib):
    mp, pp = _scene(tmp_path, spacing)
    if TRAVERSAL[traversal]:
        P = json.load(open(pp))
        P["CollisionParams"] = dict(TRAVERSAL[traversal])
        json.dump(P, open(pp, "w"))
    phys, o = _pair(mp, pp)
    X0, X1 = phys.positions(0), phys.positions(1)
    total = 0
    for (p0, p1), (c0, c1) in _states(X0, X1, spacing):
        for m, (prev, cur) in enumerate(((p0, c0), (p1, c1))):
            phys.setPrevPositions(m, prev)
            phys.setPositions(m, cur)
            o.set_prev_positions(m, prev)
            o.set_positions(m, cur)
        n = phys.collide()
        no = o.collide()
        rg, ro = phys.contacts(), o.contacts()
        assert n == no == len(rg)
        np.testing.assert_array_equal(rg, ro)
        total += n
    assert total > 20
    st = phys.stats()
    assert st["contact_detections"] >= 3
    assert st["contact_stack_overflow"] == 0 and st["contact_traverse_bounds"] == 0
    phys.close()


def test_contact_force_hessian(tmp_path, gaia_lib, oracle_lib):
    mp, pp = _scene(tmp_path, 0.03)
    phys, o = _pair(mp, pp)
    X0, X1 = phys.positions(0), phys.positions(1)
    (p0, p1), (c0, c1) = _states(X0, X1, 0.03)[2]
    for m, (prev, cur) in enumerate(((p0, c0), (p1, c1))):
        phys.setPrevPositions(m, prev)
        phys.setPositions(m, cur)
        o.set_prev_positions(m, prev)
        o.set_positions(m, cur)
    phys.collide()
    o.collide()
    rows = o.contacts()
    assert len(rows) > 5
    probe = set()
    for r in rows.tolist():
        probe.add((r[0], r[1]))
        probe.update((r[2], v) for v in r[3:6])
    fixed = [set(), set()]
    checked = 0
    for m, v in sorted(probe):
        if v in fixed[m]:
            continue
        f, H = phys.vertexForceHessian(m, v)
        fo, Ho = o.vertex_force_hessian(m, v)
        scale = max(np.abs(fo).max(), 1e-9)
        assert np.abs(f - fo).max() <= 1e-9 * scale + 1e-12, (m, v, f, fo)
        hs = max(np.abs(Ho).max(), 1e-9)
        assert np.abs(H - Ho).max() <= 1e-9 * hs, (m, v)
        checked += 1
    assert checked > 10
    phys.close()


VARIANTS = {
    "plain": {},
    "accelerator": {"useAccelerator": True, "acceleratorRho": 0.9},
    "intermediate": {"intermediateCollisionIterations": 3},
}


@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_stack_trajectory_fp64(variant, tmp_path, gaia_lib, oracle_lib):
    mp, pp = _scene(tmp_path, 0.03, **VARIANTS[variant])
    phys, o = _pair(mp, pp)
    x0 = np.concatenate([phys.positions(0), phys.positions(1)])
    kinds = set()
    for _ in range(4):
        phys.runStep(10)
        o.step(10)
        kinds |= set(o.contacts()[:, 7].tolist())
        x = np.concatenate([phys.positions(0), phys.positions(1)])
        xo = np.concatenate([o.positions(0), o.positions(1)])
        rel = np.linalg.norm(x - xo) / np.linalg.norm(xo - x0)
        assert rel <= 1e-8, (variant, rel)
    assert 2 in kinds  # DCD contacts occurred
    phys.close()


def test_stack_trajectory_mixed(tmp_path, gaia_lib, oracle_lib):
    from gaia_gb300 import scenes

    mp, pp = _scene(tmp_path, 0.03, precision="mixed")
    phys, o = _pair(mp, pp)
    x0 = np.concatenate([phys.positions(0), phys.positions(1)])
    phys.runStep(12)
    o.step(12)
    x = np.concatenate([phys.positions(0), phys.positions(1)])
    xo = np.concatenate([o.positions(0), o.positions(1)])
    rel = np.linalg.norm(x - xo) / np.linalg.norm(xo - x0)
    assert rel <= 1e-4, rel
    phys.close()


def test_collision_off_matches_oracle(tmp_path, gaia_lib, oracle_lib):
    """allowCCD / allowDCD false: the bodies pass through each other in both."""
    mp, pp = _scene(tmp_path, 0.03)
    P = json.load(open(pp))
    P["CollisionParams"] = {"allowCCD": False, "allowDCD": False}
    json.dump(P, open(pp, "w"))
    phys, o = _pair(mp, pp)
    phys.runStep(20)
    o.step(20)
    assert len(o.contacts()) == 0
    x, xo = phys.positions(1), o.positions(1)
    assert np.abs(x - xo).max() <= 1e-9
    phys.close()


@pytest.fixture(scope="module")
def cluster(tmp_path_factory, gaia_lib, oracle_lib):
    """The collision-heavy drop at test size (two cubes and two balls colliding in a
    column, CCD and DCD every substep), with the FP64 oracle's trajectory and its contact
    rows after every step."""
    from gaia_gb300 import scenes
    from oracle import scene_io

    d = tmp_path_factory.mktemp("cluster")
    mp, pp = scenes.contact_cluster(str(d), precision="fp64", iterations=20)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), 64, 0)
    nm = len(json.load(open(mp))["Models"])
    x0 = np.concatenate([o.positions(m) for m in range(nm)])
    rows, xs = [], []
    for _ in range(20):
        o.step(1)
        rows.append(o.contacts())
        xs.append(np.concatenate([o.positions(m) for m in range(nm)]))
    return mp, pp, nm, x0, rows, xs


def test_cluster_contact_rows_every_step_fp64(cluster):
    """FP64 engine: the contact rows of every substep's detection equal the oracle's, and the
    positions stay within 1e-8."""
    mp, pp, nm, x0, rows, xs = cluster
    phys, _ = _pair(mp, pp)
    kinds, total = set(), 0
    for k in range(20):
        phys.runStep(1)
        rg = phys.contacts()
        np.testing.assert_array_equal(rg, rows[k], err_msg=f"step {k}")
        total += len(rg)
        kinds |= set(rg[:, 7].tolist()) if len(rg) else set()
        x = np.concatenate([phys.positions(m) for m in range(nm)])
        rel = np.linalg.norm(x - xs[k]) / max(np.linalg.norm(xs[k] - x0), 1e-30)
        assert rel <= 1e-8, (k, rel)
    st = phys.stats()
    print(f"contact rows over 20 steps: {total}, kinds {sorted(kinds)}")
    assert total > 50 and {1, 2} <= kinds
    assert st["contact_stack_overflow"] == 0 and st["contact_traverse_bounds"] == 0
    phys.close()


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_cluster_trajectory_fp32_compute(cluster, precision):
    """FP32-compute engines on the colliding cluster after 20 steps against the FP64 oracle."""
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp, nm, x0, rows, xs = cluster
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, scenes.set_precision(pp, precision))
    phys.initialize()
    phys.runStep(20)
    x = np.concatenate([phys.positions(m) for m in range(nm)])
    rel = float(np.linalg.norm(x - xs[-1]) / np.linalg.norm(xs[-1] - x0))
    print(f"cluster {precision}: rel err {rel:.3e}")
    assert rel <= (1e-5 if precision == "mixed" else 1e-4), rel
    phys.close()
