"""The oracle against the reference's own VBD code (CPU).

tests/golden/vbd_ref_goldens.npz holds outputs of the reference's host/device VBD
functions compiled from its sources (oracle/ref_vbd.cpp, made by
tests/golden/make_vbd_goldens.py): the Neo-Hookean element, the per-vertex block as the
solve kernel composes it (material, inertia, boundary with friction, vertex-face contact),
and contact-free trajectories of its GPU step. The double build ("64") pins the oracle's
FP64 restatement to 1e-10 relative; the float build ("32") is the reference's own
arithmetic, reported for scale. Where the reference tree is present, fresh random cases
are also checked against a live build of it.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "vbd_ref_goldens.npz"))

TOL64 = 1e-10  # relative to the largest entry of the compared quantity


def _close(a, b, tol, what):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(np.asarray(a) - np.asarray(b)).max() / scale
    assert err <= tol, f"{what}: relative error {err:.3e} > {tol:.1e}"
    return err


def test_element_matches_reference(oracle_lib):
    """evaluateNeoHookeanMaterialForceAndHessian (VBD/VBDPhysicsCompute.cu:2035-2232) on 1000
    random deformed tets: the oracle's per-tet term (the CPU path's formulation,
    VBD_NeoHookean.cpp:379-581) equals it to 1e-10 of each tet's largest entry."""
    worst_f = worst_h = 0.0
    worst32 = 0.0
    for i in range(len(G["elem_A"])):
        f, h = oracle_lib.nh_element(G["elem_x"][i], G["elem_xprev"][i], G["elem_dminv"][i], G["elem_mu"][i],
                                     G["elem_lmbd"][i], G["elem_A"][i], int(G["elem_order"][i]))
        worst_f = max(worst_f, _close(f, G["elem_f64"][i], TOL64, f"force of tet {i}"))
        worst_h = max(worst_h, _close(h, G["elem_h64"][i], TOL64, f"Hessian of tet {i}"))
        worst32 = max(worst32, np.abs(G["elem_f32"][i] - G["elem_f64"][i]).max() / np.abs(G["elem_f64"][i]).max())
    print(f"element: force {worst_f:.2e}, Hessian {worst_h:.2e}; the reference's float build vs its double "
          f"build: force {worst32:.2e}")
    assert worst32 < 1e-2  # the float build is the same code (sanity of the two builds)


def test_element_energy_matches_reference():
    """evaluateNeoHookeanEnergy (:1775-1810) against an independent FP64 evaluation of the
    stable Neo-Hookean energy with the rest energy removed (the formula the GPU energy
    kernel and the oracle use)."""
    for i in range(len(G["elem_A"])):
        x, dm = G["elem_x"][i], G["elem_dminv"][i].reshape(3, 3).T  # column-major -> matrix
        Ds = (x[1:] - x[0]).T
        F = Ds @ dm
        mu, lm, A = G["elem_mu"][i], G["elem_lmbd"][i], G["elem_A"][i]
        a = 1.0 + mu / lm
        e = A * (0.5 * mu * ((F * F).sum() - 3.0) + 0.5 * lm * (np.linalg.det(F) - a) ** 2)
        e -= 0.5 * A * lm * (1.0 - a) ** 2
        assert abs(e - G["elem_e64"][i]) <= 1e-10 * max(abs(G["elem_e64"][i]), A * mu * 1e-3)


def _drop6(tmp_path):
    from gaia_gb300 import scenes

    return scenes.drop_cube(str(tmp_path), n=6, iterations=10, height=0.02, collision=scenes.NO_CONTACT)


def test_vertex_block_matches_reference(tmp_path, oracle_lib, gaia_lib):
    """Per-vertex force and Hessian as VBDSolveParallelGroup_allInOne_kernel_V2 composes them
    (material, inertia, ground penalty with friction), every vertex of the deformed 6^3
    cube partly below the ground: the oracle to 1e-10."""
    from oracle import scene_io

    mp, pp = _drop6(tmp_path)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), precision=64, nthreads=1)
    o.set_positions(0, G["blk_x"])
    wf = wh = 0.0
    for v in range(len(G["blk_x"])):
        f, h = o.vertex_force_hessian(0, v, True)
        wf = max(wf, _close(f, G["blk_f64"][v], TOL64 * np.abs(G["blk_h64"][v]).max() /
                            max(np.abs(G["blk_f64"][v]).max(), 1e-300) + TOL64, f"force of vertex {v}"))
        wh = max(wh, _close(h, G["blk_h64"][v], TOL64, f"Hessian of vertex {v}"))
    below = int((G["blk_x"][:, 1] < 0).sum())
    print(f"vertex block: force {wf:.2e}, Hessian {wh:.2e}; {below} vertices below the ground")
    assert below > 20


def test_scene_energy_matches_reference(tmp_path, oracle_lib, gaia_lib):
    """The oracle's energy of the deformed cube: elastic part = the sum of the reference's
    per-tet energies, plus the inertia energy of a fresh state (targets at rest)."""
    from oracle import scene_io

    mp, pp = _drop6(tmp_path)
    sc = scene_io.load_scene(mp, pp)
    o = oracle_lib.OracleScene(sc, precision=64, nthreads=1)
    X = o.positions(0)
    _, _, mass = o.rest(0)
    o.set_positions(0, G["blk_x"])
    dt = sc["params"]["timeStep"] / sc["params"]["numSubsteps"]
    inertia = 0.5 / dt ** 2 * float((mass * ((G["blk_x"] - X) ** 2).sum(axis=1)).sum())
    e_ref = float(G["blk_elastic_energy64"]) + inertia
    assert abs(o.energy() - e_ref) <= 1e-10 * abs(e_ref)


def _stack(tmp_path):
    from gaia_gb300 import scenes

    return scenes.stack_drop(str(tmp_path), spacing=0.03, gap=0.01, speed=1.0, precision="fp64")


def test_contact_block_matches_reference(tmp_path, oracle_lib, gaia_lib):
    """Vertices in vertex-face contact and face vertices holding relations, with
    accumulateCollisionForceAndHessian (:1731-1773) and accumlateCollisionForceAndHessianPerCollision_v2
    (:1812-1930) in the composition: the oracle's contact rows equal the ones the goldens were
    made from, and its force and Hessian equal the reference's to 1e-10."""
    from oracle import scene_io

    mp, pp = _stack(tmp_path)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), precision=64, nthreads=1)
    for m in (0, 1):
        o.set_prev_positions(m, G[f"con_prev{m}"])
        o.set_positions(m, G[f"con_x{m}"])
    o.collide()
    np.testing.assert_array_equal(o.contacts(), G["con_rows"])
    for k, (m, v) in enumerate(G["con_probe"]):
        f, h = o.vertex_force_hessian(int(m), int(v), True)
        hs = np.abs(G["con_h64"][k]).max()
        assert np.abs(f - G["con_f64"][k]).max() <= TOL64 * max(np.abs(G["con_f64"][k]).max(), 1e-6 * hs), (m, v)
        _close(h, G["con_h64"][k], TOL64, f"Hessian of ({m}, {v})")


def _stretch(tmp_path):
    from tests.golden.make_vbd_goldens import stretched_cube, stretched_state

    mp, pp = stretched_cube(str(tmp_path))
    return mp, pp, stretched_state


@pytest.mark.parametrize("case", ["drop", "stretch"])
def test_trajectories_match_reference(case, tmp_path, oracle_lib, gaia_lib):
    """runStepGPU composed from the reference's own functions (no contact detection): the
    oracle's FP64 step (VBDPhysics.cpp:1580-1632) follows it to 1e-10 every 10 steps."""
    from oracle import scene_io

    if case == "drop":
        mp, pp = _drop6(tmp_path)
        init = None
    else:
        mp, pp, init = _stretch(tmp_path)
    o = oracle_lib.OracleScene(scene_io.load_scene(mp, pp), precision=64, nthreads=1)
    x0 = o.positions(0)
    if init is not None:
        x0 = init(x0)
        o.set_positions(0, x0)
    ref = G[f"traj_{case}64"]
    for k in range(len(ref)):
        o.step(10)
        x = o.positions(0)
        rel = np.linalg.norm(x - ref[k]) / np.linalg.norm(ref[k] - x0)
        rel32 = np.linalg.norm(G[f"traj_{case}32"][k] - ref[k]) / np.linalg.norm(ref[k] - x0)
        print(f"{case} step {10 * (k + 1)}: oracle vs reference {rel:.2e}; the reference's float build {rel32:.2e}")
        assert rel <= TOL64, (case, k, rel)


@pytest.fixture(scope="module")
def live_ref():
    """The reference's VBD functions built from its tree, where that tree is present."""
    from oracle.oracle import reference_root

    if not reference_root():
        pytest.skip("reference tree not present")
    from tests.golden.make_vbd_goldens import ref_libs

    return ref_libs()


def test_live_reference_element(live_ref, oracle_lib):
    """Fresh random tets (another seed) against a build of the reference made now."""
    from tests.golden.make_vbd_goldens import random_tets

    L, ft, dt_np = live_ref[1]
    T = random_tets(np.random.Generator(np.random.PCG64(77)), 300)
    for i in range(len(T["A"])):
        x = np.ascontiguousarray(T["x"][i].reshape(-1))
        xp = np.ascontiguousarray(T["xprev"][i].reshape(-1))
        dm = np.ascontiguousarray(T["dminv"][i])
        f = np.zeros(3)
        h = np.zeros(9)
        L.ref_nh_element(x.ctypes.data, xp.ctypes.data, dm.ctypes.data, T["mu"][i], T["lmbd"][i], T["A"][i],
                         int(T["order"][i]), 0.0, 0.0, 1.0 / 300.0, f.ctypes.data, h.ctypes.data)
        fo, ho = oracle_lib.nh_element(T["x"][i], T["xprev"][i], T["dminv"][i], T["mu"][i], T["lmbd"][i], T["A"][i],
                                       int(T["order"][i]))
        _close(fo, f, TOL64, f"force of tet {i}")
        _close(ho, h.reshape(3, 3).T, TOL64, f"Hessian of tet {i}")


def test_oracle_convergence_terms(tmp_path, oracle_lib, gaia_lib):
    """The oracle's FP64 convergence evaluation (VBDPhysics.cpp:3459-3506): its energy is the
    reference's per-tet energies summed plus inertia, and its average force norm is the mean
    over all vertices of |sum of the per-tet material terms (pinned above) + inertia force|."""
    from oracle import scene_io

    mp, pp = _drop6(tmp_path)
    sc = scene_io.load_scene(mp, pp)
    o = oracle_lib.OracleScene(sc, precision=64, nthreads=1)
    X = o.positions(0)
    dminv, vol, mass = o.rest(0)
    o.set_positions(0, G["blk_x"])
    c = o.convergence()
    dt = sc["params"]["timeStep"] / sc["params"]["numSubsteps"]
    inertia = 0.5 / dt ** 2 * float((mass * ((G["blk_x"] - X) ** 2).sum(axis=1)).sum())
    assert abs(c["elastic"] - float(G["blk_elastic_energy64"])) <= 1e-10 * abs(c["elastic"])
    assert abs(c["inertia"] - inertia) <= 1e-12 * inertia
    assert c["energy"] == o.energy()
    mat = sc["meshes"][0]["material"]
    T = np.asarray(sc["meshes"][0]["tets"])
    f = mass[:, None] / dt ** 2 * (X - G["blk_x"])
    for t in range(len(T)):
        for k in range(4):
            ft, _ = oracle_lib.nh_element(G["blk_x"][T[t]], X[T[t]], dminv[t], mat["miu"], mat["lmbd"], vol[t], k)
            f[T[t, k]] += ft
    avg = float(np.linalg.norm(f, axis=1).mean())
    assert abs(c["avg_force_norm"] - avg) <= 1e-10 * avg
