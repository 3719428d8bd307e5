"""Cloth path on the CPU (no GPU needed): the library's scene loader (topology, rest
shape, colorings, merged colors) against the CPU oracle, the oracle's StVK membrane
and bending forces against finite differences of its energy, and its contact
detector's outputs against direct geometric checks."""
import json

import numpy as np
import pytest


def _scene(tmp_path, **kw):
    from gaia_gb300 import scenes

    args = dict(n=10, side=0.4, sphere_radius=0.12, sphere_level=2, contact_radius=0.01, iterations=5,
                dt=1.0 / 300.0, bending=1e-3)
    args.update(kw)
    return scenes.cloth_on_sphere(str(tmp_path), **args)


def _load(mp, pp):
    from gaia_gb300 import VBDClothSimulationFramework

    c = VBDClothSimulationFramework()
    c.loadRunningparameters(mp, pp)
    return c


def test_topology_rest_groups_match_oracle(tmp_path, gaia_lib, oracle_lib):
    from oracle import cloth as oc

    mp, pp = _scene(tmp_path)
    c = _load(mp, pp)
    o = oc.ClothOracle(oc.load_scene(mp, pp), nthreads=1)
    assert c.numMeshes() == (1, 1)
    for m in (0, 1):
        e6, fe = c.topology(m)
        oe6, ofe = o.topology(m)
        assert np.array_equal(e6, oe6) and np.array_equal(fe, ofe)
    dm, ar, ms = c.restShape(0)
    odm, oar, oms = o.rest(0)
    # different in-plane frames: areas and masses agree, DmInv up to a rotation R of the
    # frame (DmInv' = DmInv R^T), so compare the frame-invariant DmInv DmInv^T
    assert np.allclose(ar, oar, rtol=1e-12, atol=0) and np.allclose(ms, oms, rtol=1e-12, atol=0)
    for k in range(len(dm)):
        A = dm[k].reshape(2, 2).T
        B = odm[k].reshape(2, 2).T
        assert np.allclose(A @ A.T, B @ B.T, rtol=1e-9, atol=1e-9)
    g, og = c.parallelGroups(), o.groups()
    assert len(g) == len(og) and all(np.array_equal(a, b) for a, b in zip(g, og))
    c.close()


def test_edge_topology_invariants(tmp_path, gaia_lib):
    mp, pp = _scene(tmp_path, n=7)
    c = _load(mp, pp)
    F = None
    from oracle import cloth as oc

    F = oc.read_obj(json.load(open(mp))["Models"][0]["path"])[1]
    e6, fe = c.topology(0)
    assert c.numEdges(0) == len(e6)
    nv = c.numVertices(0)
    # Euler characteristic of a disc: V - E + F = 1
    assert nv - len(e6) + len(F) == 1
    for e, (v1, v2, n12, n21, f1, f2) in enumerate(e6):
        f = F[f1]
        k = list(f).index(v1)
        assert f[(k + 1) % 3] == v2 and f[(k + 2) % 3] == n12
        if f2 >= 0:
            g = F[f2]
            k = list(g).index(v2)
            assert g[(k + 1) % 3] == v1 and g[(k + 2) % 3] == n21
        else:
            assert n21 == -1
    for f in range(len(F)):
        for i in range(3):
            v1, v2 = e6[fe[f, i], 0], e6[fe[f, i], 1]
            assert {v1, v2} == {F[f][i], F[f][(i + 1) % 3]}
    c.close()


@pytest.mark.parametrize("algorithm", ["greedy", "mcs"])
@pytest.mark.parametrize("bending", [False, True])
def test_trimesh_coloring_is_proper(algorithm, bending, gaia_lib):
    from gaia_gb300 import color_trimesh, scenes

    X, F = scenes.cloth_grid(13, 1.0)
    col = color_trimesh(len(X), F, algorithm, bending)
    assert col.min() == 0
    for a, b, c in F:
        assert col[a] != col[b] and col[b] != col[c] and col[a] != col[c]
    if bending:
        # opposite vertices of each interior edge differ too
        seen = {}
        for f, t in enumerate(F):
            for i in range(3):
                key = (min(t[i], t[(i + 1) % 3]), max(t[i], t[(i + 1) % 3]))
                seen.setdefault(key, []).append(t[(i + 2) % 3])
        for opp in seen.values():
            if len(opp) == 2:
                assert col[opp[0]] != col[opp[1]]


def test_oracle_elastic_force_matches_finite_differences(tmp_path, oracle_lib):
    from oracle import cloth as oc

    mp, pp = _scene(tmp_path, n=8, side=0.3, bending=1e-2)
    o = oc.ClothOracle(oc.load_scene(mp, pp), nthreads=1)
    rng = np.random.Generator(np.random.PCG64(3))
    x = o.positions(0) + rng.uniform(-3e-3, 3e-3, size=(64, 3))
    o.set_positions(0, x)
    eps = 1e-6
    for v in (0, 9, 27, 36, 63):
        f, H = o.elastic_force_hessian(0, v)
        g = np.zeros(3)
        Hn = np.zeros((3, 3))
        for k in range(3):
            xp = x.copy()
            xp[v, k] += eps
            o.set_positions(0, xp)
            ep, (fp, _) = o.elastic_energy(0), o.elastic_force_hessian(0, v)
            xm = x.copy()
            xm[v, k] -= eps
            o.set_positions(0, xm)
            em, (fm, _) = o.elastic_energy(0), o.elastic_force_hessian(0, v)
            g[k] = (ep - em) / (2 * eps)
            Hn[:, k] = -(fp - fm) / (2 * eps)
        o.set_positions(0, x)
        assert np.abs(f + g).max() <= 1e-6 * np.abs(g).max()
        assert np.abs(H - Hn).max() <= 1e-6 * np.abs(Hn).max()


def _closest_dist32(p, a, b, c):
    """Distance from p to triangle abc in float32 (any correct method)."""
    p, a, b, c = (np.asarray(v, np.float64) for v in (p, a, b, c))
    ab, ac, ap = b - a, c - a, p - a
    n = np.cross(ab, ac)
    # project and clamp by barycentrics, else the edges
    A = np.array([[ab @ ab, ab @ ac], [ab @ ac, ac @ ac]])
    s, t = np.linalg.solve(A, [ab @ ap, ac @ ap])
    if s >= 0 and t >= 0 and s + t <= 1:
        return abs(ap @ n) / np.linalg.norm(n)

    def seg(p, u, v):
        d = v - u
        w = np.clip((p - u) @ d / (d @ d), 0, 1)
        return np.linalg.norm(p - (u + w * d))

    return min(seg(p, a, b), seg(p, b, c), seg(p, c, a))


def test_oracle_contacts_are_within_query_radius(tmp_path, oracle_lib):
    from oracle import cloth as oc

    mp, pp = _scene(tmp_path, n=9, side=0.3, gap=0.004)
    sc = oc.load_scene(mp, pp)
    o = oc.ClothOracle(sc, nthreads=2)
    o.step(6)  # the cloth reaches the sphere
    o.detect()
    r = sc["params"]["maxQueryDis"]
    vf = o.vf_contacts()
    assert len(vf) > 0
    X = [o.positions(m) for m in range(2)]
    F = [m["faces"] for m in sc["meshes"]]
    assert any(row[2] == 1 for row in vf)  # cloth-sphere contacts
    for vm, v, fm, f in vf:
        d = _closest_dist32(X[vm][v], *(X[fm][k] for k in F[fm][f]))
        assert d < r * (1 + 1e-5)
        if vm == fm:
            assert v not in F[fm][f]
    vfmin, fvmin, _ = o.min_distances(0)
    assert np.all(vfmin <= np.float32(r))
    b = o.bounds(0)
    assert np.all(b >= 0) and np.all(b <= 0.45 * r * (1 + 1e-6))
