"""Generate tests/golden/vbd_ref_goldens.npz from the reference's own VBD code.

Needs the reference tree (GAIA_REFERENCE_ROOT, or the oracle Makefile's REF_ROOT): it
runs ``make -C oracle ref``, which compiles the reference's host/device VBD functions
(element, inertia, boundary and friction, contact, velocity update; VBD/VBDPhysicsCompute.cu
and VBD/VBD_GeneralCompute.h) into oracle/_ref/libvbd_ref32.so (the reference's float
arithmetic) and libvbd_ref64.so (the same code in double), and records their outputs on
seeded inputs:

  elem_*   1000 random tets (rest shapes near a regular tet of 1-2 cm edges, deformation
           gradients with stretches of up to 30 % and random rotations, vertex order 0-3,
           E in [1e5, 1e7] Pa, nu in [0.3, 0.48], no damping): force (3) and Hessian (9)
           of evaluateNeoHookeanMaterialForceAndHessian, and evaluateNeoHookeanEnergy;
  blk_*    the 6^3 drop cube of the tests (scenes.drop_cube(n=6, iterations=10,
           height=0.02)), every vertex displaced by U(+-1e-3) m and the cube moved 2.1 cm
           down so that its bottom layer is below the ground: force and Hessian of every
           vertex composed as VBDSolveParallelGroup_allInOne_kernel_V2 composes them
           (material over incident tets in the kernel's slot/tree order, inertia, boundary
           with friction), at the state a freshly initialised handle has (inertia targets
           and previous positions at the rest positions);
  con_*    the stacked cubes of the contact tests (scenes.stack_drop(spacing=0.03, gap=0.01,
           speed=1.0)) at the deformed state the contact tests use, with the oracle's contact
           rows turned into the reference's CollisionDataGPU records (own contact, up to four
           relations per face vertex, VBDPhysics.cpp:1812-1894): force and Hessian of every
           vertex in contact or holding a relation, including accumulateCollisionForceAndHessian;
  traj_*   runStepGPU without contact detection (ref_step in oracle/ref_vbd.cpp): the 6^3
           drop cube for 40 steps x 10 iterations (falls, lands, slides) and a 5^3 cube
           released from a 10 % stretch in x, free of gravity and ground, for 20 steps x 10
           iterations (stretched_cube, stretched_state);
           positions every 10 steps, in the double and the float build.

The 3x3 solve inside ref_step is the LDL^T of the oracle and the kernels (CuMatrix's is not
in the reference tree). Usage: python tests/golden/make_vbd_goldens.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "vbd_ref_goldens.npz")


def ref_libs():
    """(lib32, lib64) of the reference's VBD functions, built from the reference tree."""
    from oracle.oracle import reference_root

    root = reference_root()
    if not root:
        raise SystemExit("the reference tree is not present (set GAIA_REFERENCE_ROOT)")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_ROOT={root}"], check=True)
    libs = []
    for bits in (32, 64):
        L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", f"libvbd_ref{bits}.so"))
        ft = C.c_float if bits == 32 else C.c_double
        L.ref_float_bytes.restype = C.c_int
        assert L.ref_float_bytes() == (4 if bits == 32 else 8)
        L.ref_nh_element.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, ft, ft, ft, C.c_int32, ft, ft, ft,
                                     C.c_void_p, C.c_void_p]
        L.ref_nh_energy.argtypes = [C.c_void_p, C.c_void_p, ft, ft, ft]
        L.ref_nh_energy.restype = ft
        L.ref_vertex_force_hessian.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                                               C.c_void_p]
        L.ref_step.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                               C.c_int32]
        L.ref_step.restype = C.c_int32
        libs.append((L, ft, np.float32 if bits == 32 else np.float64))
    return libs


def structs(ft):
    P = C.c_void_p

    class RefMesh(C.Structure):
        _fields_ = [("nv", C.c_int32), ("ntet", C.c_int32), ("pos", P), ("prev", P), ("inertia", P), ("vel", P),
                    ("pos_new", P), ("mass", P), ("fixed", P), ("tets", P), ("dminv", P), ("vol", P),
                    ("nbr_info", P), ("nbr_tet", P), ("nbr_order", P), ("mu", ft), ("lmbd", ft), ("kh", ft),
                    ("kd", ft), ("friction_dynamic", ft), ("friction_eps_v", ft), ("max_velocity", ft),
                    ("exp_vel_damping", ft), ("const_vel_damping", ft), ("coll", P)]

    class RefPhysics(C.Structure):
        _fields_ = [("dt", ft), ("dt_sqr_recip", ft), ("world", ft * 6), ("boundary_stiffness", ft),
                    ("boundary_friction_mu", ft), ("boundary_friction_eps_v", ft), ("collision_stiffness", ft),
                    ("step_size", ft), ("step_size_gd", ft), ("gravity", ft * 3), ("pivot_tol", ft)]

    return RefMesh, RefPhysics


class RefScene:
    """The oracle's view of a scene (rest shape, CSR, groups) in the reference's layout."""

    def __init__(self, mp, pp, lib, ft, dt_np):
        from oracle import oracle as orc
        from oracle import scene_io

        self.sc = scene_io.load_scene(mp, pp)
        self.o = orc.OracleScene(self.sc, precision=64, nthreads=1)
        self.lib, self.ft, self.dt_np = lib, ft, dt_np
        self.RefMesh, self.RefPhysics = structs(ft)
        self.keep = []
        self.meshes = (self.RefMesh * len(self.sc["meshes"]))()
        p = self.sc["params"]
        self.p = self.RefPhysics()
        dt = p["timeStep"] / p["numSubsteps"]
        self.p.dt = dt
        self.p.dt_sqr_recip = 1.0 / (dt * dt)
        for k in range(3):
            self.p.world[k] = p["worldBounds"][0][k]
            self.p.world[3 + k] = p["worldBounds"][1][k]
            self.p.gravity[k] = p["gravity"][k]
        self.p.boundary_stiffness = p["boundaryCollisionStiffness"]
        self.p.boundary_friction_mu = p["boundaryFrictionDynamic"]
        self.p.boundary_friction_eps_v = p["boundaryFrictionEpsV"]
        self.p.collision_stiffness = p.get("collisionStiffness", 1e5)
        self.p.step_size, self.p.step_size_gd = p["stepSize"], p["stepSizeGD"]
        self.p.pivot_tol = 1e-5 if dt_np == np.float32 else 1e-12
        self.arr = []
        for i, m in enumerate(self.sc["meshes"]):
            nv, T = len(m["X"]), np.asarray(m["tets"], np.int32)
            dminv, vol, mass = self.o.rest(i)
            inc = [[] for _ in range(nv)]
            for t in range(len(T)):
                for k in range(4):
                    inc[T[t, k]].append((t, k))
            info = np.zeros((nv, 2), np.int32)
            nt, no = [], []
            for v in range(nv):
                info[v] = (len(nt), len(inc[v]))
                for t, k in inc[v]:
                    nt.append(t)
                    no.append(k)
            mat = m["material"]
            a = {"pos": np.ascontiguousarray(m["X"], dt_np).reshape(-1).copy(),
                 "vel": np.ascontiguousarray(m["V0"], dt_np).reshape(-1).copy(),
                 "mass": np.ascontiguousarray(mass, dt_np), "fixed": np.ascontiguousarray(m["fixed"], np.int8),
                 "tets": np.ascontiguousarray(T.reshape(-1)), "dminv": np.ascontiguousarray(dminv, dt_np).reshape(-1),
                 "vol": np.ascontiguousarray(vol, dt_np), "nbr_info": np.ascontiguousarray(info.reshape(-1)),
                 "nbr_tet": np.ascontiguousarray(nt, np.int32), "nbr_order": np.ascontiguousarray(no, np.int32)}
            a["prev"] = a["pos"].copy()
            a["inertia"] = a["pos"].copy()
            a["pos_new"] = a["pos"].copy()
            self.arr.append(a)
            R = self.meshes[i]
            R.nv, R.ntet = nv, len(T)
            for k, v in a.items():
                setattr(R, k, v.ctypes.data)
            R.mu, R.lmbd = mat["miu"], mat["lmbd"]
            R.kh, R.kd = mat["dampingHydrostatic"], mat["dampingDeviatoric"]
            R.friction_dynamic, R.friction_eps_v = mat["frictionDynamic"], mat["frictionEpsV"]
            R.max_velocity = mat.get("maxVelocityMagnitude", -1.0)
            R.exp_vel_damping = mat["exponentialVelDamping"] ** dt
            R.const_vel_damping = mat["constantVelDamping"] * dt
            R.coll = None

    def set_positions(self, i, x):
        self.arr[i]["pos"][:] = np.asarray(x, self.dt_np).reshape(-1)

    def set_collisions(self, recs):
        self.coll = [np.ascontiguousarray(r, np.int32).reshape(-1) for r in recs]
        for i, r in enumerate(self.coll):
            self.meshes[i].coll = r.ctypes.data

    def force_hessian(self, i, v):
        f = np.zeros(3, self.dt_np)
        h = np.zeros(9, self.dt_np)
        rc = self.lib.ref_vertex_force_hessian(C.cast(self.meshes, C.c_void_p), len(self.arr), C.byref(self.p), i, v,
                                               f.ctypes.data, h.ctypes.data)
        assert rc == 0
        return f.astype(np.float64), h.reshape(3, 3).T.astype(np.float64)  # column-major -> (row, col)

    def step(self, iterations, n):
        groups = self.o.groups()
        ofs = np.zeros(len(groups) + 1, np.int32)
        ofs[1:] = np.cumsum([len(g) // 2 if g.ndim == 1 else len(g) for g in groups])
        pairs = np.ascontiguousarray(np.concatenate([np.asarray(g, np.int32).reshape(-1) for g in groups]))
        return self.lib.ref_step(C.cast(self.meshes, C.c_void_p), len(self.arr), C.byref(self.p), len(groups),
                                 ofs.ctypes.data, pairs.ctypes.data, iterations, n)

    def positions(self, i):
        return self.arr[i]["pos"].reshape(-1, 3).astype(np.float64)


def random_tets(rng, n):
    """Rest shapes near a regular tet (1-2 cm edges, random rotation and jitter), deformed
    states (random rotation times a symmetric stretch of up to 30 %, plus jitter), previous
    positions slightly away, vertex orders and materials."""
    reg = np.array([[0, 0, 0], [1, 0, 0], [0.5, np.sqrt(3) / 2, 0], [0.5, np.sqrt(3) / 6, np.sqrt(2.0 / 3.0)]])
    out = {k: [] for k in ("x", "xprev", "dminv", "A", "order", "mu", "lmbd")}
    for _ in range(n):
        Q, _r = np.linalg.qr(rng.normal(size=(3, 3)))
        X = (reg * rng.uniform(0.01, 0.02)) @ Q.T + rng.uniform(-1e-3, 1e-3, (4, 3))
        Dm = (X[1:] - X[0]).T
        if np.linalg.det(Dm) < 0:
            X[[2, 3]] = X[[3, 2]]
            Dm = (X[1:] - X[0]).T
        S = np.eye(3) + rng.uniform(-0.3, 0.3, (3, 3))
        S = 0.5 * (S + S.T)
        Q2, _r = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(Q2) < 0:
            Q2[:, 0] *= -1
        x = (X - X.mean(0)) @ (Q2 @ S).T + rng.uniform(-0.05, 0.05, 3) + rng.uniform(-2e-4, 2e-4, (4, 3))
        E, nu = rng.uniform(1e5, 1e7), rng.uniform(0.3, 0.48)
        out["x"].append(x)
        out["xprev"].append(x + rng.uniform(-1e-3, 1e-3, (4, 3)))
        out["dminv"].append(np.linalg.inv(Dm).T.reshape(-1))  # column-major
        out["A"].append(np.linalg.det(Dm) / 6.0)
        out["order"].append(int(rng.integers(0, 4)))
        out["mu"].append(E / (2 * (1 + nu)))
        out["lmbd"].append(E * nu / ((1 + nu) * (1 - 2 * nu)))
    return {k: np.asarray(v) for k, v in out.items()}


def element_goldens(libs, rng):
    T = random_tets(rng, 1000)
    g = {"elem_" + k: v for k, v in T.items()}
    for (L, ft, dt_np), tag in zip(libs, ("32", "64")):
        F = np.zeros((len(T["A"]), 3))
        H = np.zeros((len(T["A"]), 3, 3))
        Ee = np.zeros(len(T["A"]))
        for i in range(len(T["A"])):
            x = np.ascontiguousarray(T["x"][i].reshape(-1), dt_np)
            xp = np.ascontiguousarray(T["xprev"][i].reshape(-1), dt_np)
            dm = np.ascontiguousarray(T["dminv"][i], dt_np)
            f = np.zeros(3, dt_np)
            h = np.zeros(9, dt_np)
            L.ref_nh_element(x.ctypes.data, xp.ctypes.data, dm.ctypes.data, T["mu"][i], T["lmbd"][i], T["A"][i],
                             int(T["order"][i]), 0.0, 0.0, 1.0 / 300.0, f.ctypes.data, h.ctypes.data)
            F[i] = f
            H[i] = h.reshape(3, 3).T
            Ee[i] = L.ref_nh_energy(x.ctypes.data, dm.ctypes.data, T["mu"][i], T["lmbd"][i], T["A"][i])
        g[f"elem_f{tag}"], g[f"elem_h{tag}"], g[f"elem_e{tag}"] = F, H, Ee
    return g


def block_goldens(libs, d):
    from gaia_gb300 import scenes

    mp, pp = scenes.drop_cube(d, n=6, iterations=10, height=0.02, collision=scenes.NO_CONTACT)
    rng = np.random.Generator(np.random.PCG64(3))
    g = {}
    for (L, ft, dt_np), tag in zip(libs, ("32", "64")):
        rs = RefScene(mp, pp, L, ft, dt_np)
        X = rs.sc["meshes"][0]["X"]
        if tag == "32":
            x = X + np.random.Generator(np.random.PCG64(3)).uniform(-1e-3, 1e-3, size=X.shape)
            x[:, 1] -= 0.021
            x = x.astype(np.float32).astype(np.float64)  # representable in both builds
            g["blk_x"] = x
        rs.set_positions(0, g["blk_x"])
        n = len(X)
        F = np.zeros((n, 3))
        H = np.zeros((n, 3, 3))
        for v in range(n):
            F[v], H[v] = rs.force_hessian(0, v)
        g[f"blk_f{tag}"], g[f"blk_h{tag}"] = F, H
        if tag == "64":
            # elastic energy of the state from the reference's per-tet energy
            dm = rs.arr[0]["dminv"].reshape(-1, 9)
            vol = rs.arr[0]["vol"]
            T = np.asarray(rs.sc["meshes"][0]["tets"])
            mat = rs.sc["meshes"][0]["material"]
            e = 0.0
            for t in range(len(T)):
                xt = np.ascontiguousarray(g["blk_x"][T[t]].reshape(-1))
                e += L.ref_nh_energy(xt.ctypes.data, np.ascontiguousarray(dm[t]).ctypes.data, mat["miu"],
                                     mat["lmbd"], vol[t])
            g["blk_elastic_energy64"] = np.float64(e)
    del rng
    return g


def contact_records(o, nmesh, nv_of):
    """The reference's CollisionDataGPU records (VBDPhysics.cpp:1812-1894) from the oracle's
    contact rows: every contact is its vertex's own record; each face vertex takes the
    contact as a relation while it has fewer than four, in row order."""
    rows = o.contacts()
    recs = [np.zeros((nv_of[m], 23), np.int32) for m in range(nmesh)]
    for r in rows:
        m, v, fm, a, b, c, f, kind = (int(t) for t in r)
        R = recs[m][v]
        R[0], R[1], R[2], R[3], R[4], R[5] = 1, a, b, c, f, fm
        for k, fv in enumerate((a, b, c)):
            F = recs[fm][fv]
            if F[6] < 4:
                j = 7 + 4 * F[6]
                F[j], F[j + 1], F[j + 2], F[j + 3] = m, v, 0, k
                F[6] += 1
    return rows, recs


def contact_goldens(libs, d):
    from gaia_gb300 import scenes

    mp, pp = scenes.stack_drop(d, spacing=0.03, gap=0.01, speed=1.0, precision="fp64")
    g = {}
    for (L, ft, dt_np), tag in zip(libs, ("32", "64")):
        rs = RefScene(mp, pp, L, ft, dt_np)
        o = rs.o
        X0, X1 = o.positions(0), o.positions(1)
        if tag == "32":
            rng = np.random.default_rng(0)
            sp = 0.03
            deep = np.array([0.0, -1.2 * sp, 0.0])
            n0 = rng.normal(0, 0.05 * sp, X0.shape)
            n1 = rng.normal(0, 0.05 * sp, X1.shape)
            f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)  # noqa: E731
            g["con_prev0"], g["con_prev1"] = f32(X0 + n0), f32(X1 + deep + n1)
            g["con_x0"], g["con_x1"] = f32(X0 + 0.5 * n0), f32(X1 + 1.5 * deep - n1)
        for m in (0, 1):
            o.set_prev_positions(m, g[f"con_prev{m}"])
            o.set_positions(m, g[f"con_x{m}"])
        o.collide()
        rows, recs = contact_records(o, 2, [len(X0), len(X1)])
        for m in (0, 1):
            rs.set_positions(m, g[f"con_x{m}"])
            rs.arr[m]["prev"][:] = np.asarray(g[f"con_prev{m}"], dt_np).reshape(-1)
            # a fresh handle's inertia targets are its rest positions
        rs.set_collisions(recs)
        probe = sorted({(int(r[0]), int(r[1])) for r in rows} | {(int(r[2]), int(v)) for r in rows for v in r[3:6]})
        probe = [(m, v) for m, v in probe if not rs.sc["meshes"][m]["fixed"][v]]
        F = np.zeros((len(probe), 3))
        H = np.zeros((len(probe), 3, 3))
        for k, (m, v) in enumerate(probe):
            F[k], H[k] = rs.force_hessian(m, v)
        g["con_rows"] = np.asarray(rows, np.int32)
        g["con_probe"] = np.asarray(probe, np.int32)
        g[f"con_f{tag}"], g[f"con_h{tag}"] = F, H
    return g


def trajectory_goldens(libs, d):
    from gaia_gb300 import scenes

    g = {}
    mp, pp = scenes.drop_cube(os.path.join(d, "drop"), n=6, iterations=10, height=0.02, collision=scenes.NO_CONTACT)
    mp2, pp2 = stretched_cube(os.path.join(d, "stretch"))
    for (L, ft, dt_np), tag in zip(libs, ("32", "64")):
        rs = RefScene(mp, pp, L, ft, dt_np)
        xs = []
        failed = 0
        for _ in range(4):
            failed += rs.step(10, 10)
            xs.append(rs.positions(0))
        g[f"traj_drop{tag}"] = np.asarray(xs)
        g[f"traj_drop_failed{tag}"] = np.int32(failed)
        rs = RefScene(mp2, pp2, L, ft, dt_np)
        rs.set_positions(0, stretched_state(rs.sc["meshes"][0]["X"]))
        xs = []
        for _ in range(2):
            rs.step(10, 10)
            xs.append(rs.positions(0))
        g[f"traj_stretch{tag}"] = np.asarray(xs)
    return g


def stretched_cube(d):
    """A free 5^3 lattice cube (1 cm cells), no gravity, no ground; its initial state is
    the rest shape stretched by 10 % in x about the centroid (stretched_state)."""
    from gaia_gb300 import scenes

    os.makedirs(d, exist_ok=True)
    X, T = scenes.lattice_cube((5, 5, 5), 0.01, (0.0, 0.0, 0.0), jitter=1e-4, seed=9)
    tp, cp = scenes._write_mesh(d, "cube5", X, T)
    m = scenes.model_entry(tp, cp)
    params = scenes.physics_params(1.0 / 300.0, 10, gravity=(0.0, 0.0, 0.0), precision="fp64",
                                   usePlaneGround=False)
    return scenes._write_json(d, [m], params, collision=scenes.NO_CONTACT)


def stretched_state(X):
    x = np.array(X, np.float64)
    c = x.mean(axis=0)
    x[:, 0] = c[0] + 1.1 * (x[:, 0] - c[0])
    return x.astype(np.float32).astype(np.float64)


def main():
    libs = ref_libs()
    rng = np.random.Generator(np.random.PCG64(20261204))
    g = {}
    g.update(element_goldens(libs, rng))
    with tempfile.TemporaryDirectory() as d:
        g.update(block_goldens(libs, os.path.join(d, "blk")))
        g.update(contact_goldens(libs, os.path.join(d, "con")))
        g.update(trajectory_goldens(libs, os.path.join(d, "traj")))
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT}: " + ", ".join(f"{k}{list(np.shape(v))}" for k, v in g.items()))


if __name__ == "__main__":
    main()
