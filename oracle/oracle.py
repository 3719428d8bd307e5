"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py`` (its cpu_baseline and
``--impl reference`` legs) may import this module. It restates the reference's
CPU VBD path (Simulator/Modules/VBD/VBDPhysics.cpp:1580-1632, 2402-2483) and
coloring tools (GraphColoring/mcs.cpp:14-168, gready.cpp:15-117); the product
library never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")


def reference_root() -> str | None:
    """Root of the reference project's source tree, for the checker builds and the tests
    that read its files: the GAIA_REFERENCE_ROOT environment variable, else the REF_ROOT
    default of this directory's Makefile recipe. None where that tree is absent (the tests
    that need it skip)."""
    root = os.environ.get("GAIA_REFERENCE_ROOT")
    if not root:
        try:
            r = subprocess.run(["make", "-s", "-C", _HERE, "print-ref-root"], capture_output=True, text=True,
                               timeout=60)
            root = r.stdout.strip() if r.returncode == 0 else None
        except Exception:
            root = None
    return root if root and os.path.isdir(os.path.join(root, "Simulator")) else None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, no GPU needed)."""
    srcs = [os.path.join(_HERE, f) for f in ("vbd_oracle.cpp", "vbd_oracle.h", "cloth_oracle.cpp", "cloth_oracle.h",
                                              "tet_contact.cpp", "tet_contact.h")]
    if force or not os.path.exists(_LIB) or any(os.path.getmtime(_LIB) < os.path.getmtime(s) for s in srcs):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB


class OracleMesh(C.Structure):
    _fields_ = [
        ("nv", C.c_int32), ("ntet", C.c_int32),
        ("X", C.POINTER(C.c_double)), ("V0", C.POINTER(C.c_double)),
        ("tets", C.POINTER(C.c_int32)), ("fixed", C.POINTER(C.c_int8)),
        ("ncolors", C.c_int32), ("color_offsets", C.POINTER(C.c_int32)),
        ("color_verts", C.POINTER(C.c_int32)),
        ("miu", C.c_double), ("lmbd", C.c_double), ("density", C.c_double),
        ("damping_hydrostatic", C.c_double), ("damping_deviatoric", C.c_double),
        ("exp_vel_damping", C.c_double), ("const_vel_damping", C.c_double),
        ("friction_dynamic", C.c_double), ("friction_eps_v", C.c_double),
        ("init_type", C.c_int32), ("active", C.c_int32),
    ]


class OracleParams(C.Structure):
    _fields_ = [
        ("time_step", C.c_double), ("num_substeps", C.c_int32), ("iterations", C.c_int32),
        ("gravity", C.c_double * 3), ("world_lo", C.c_double * 3), ("world_hi", C.c_double * 3),
        ("use_plane_ground", C.c_int32),
        ("boundary_stiffness", C.c_double), ("boundary_friction_mu", C.c_double),
        ("boundary_friction_eps_v", C.c_double),
        ("step_size", C.c_double), ("step_size_gd", C.c_double),
        ("friction_start_iter", C.c_int32), ("associate_gravity", C.c_int32),
        ("use_accelerator", C.c_int32), ("accelerator_rho", C.c_double),
        ("allow_ccd", C.c_int32), ("allow_dcd", C.c_int32),
        ("collision_stiffness", C.c_double), ("collision_off_height", C.c_double),
        ("intermediate_collision_iterations", C.c_int32),
        ("handle_self_collision", C.c_int32), ("check_feasible_region", C.c_int32),
        ("feasible_region_eps", C.c_double),
        ("check_tet_traverse", C.c_int32), ("traverse_non_self", C.c_int32),
        ("stop_traversing_after_passing", C.c_int32), ("shift_query_to_center", C.c_int32),
        ("use_static_traverse", C.c_int32),
        ("center_shift_level", C.c_double), ("ray_tri_eps", C.c_double), ("max_search_mult", C.c_double),
    ]


class OracleDeformer(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("center", C.c_double * 3), ("axis", C.c_double * 3),
        ("angular_velocity", C.c_double), ("end_time", C.c_double), ("speed", C.c_double * 3),
        ("nsel", C.c_int32), ("sel_mesh", C.POINTER(C.c_int32)), ("sel_vert", C.POINTER(C.c_int32)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.oracle_read_t.restype = C.c_int32
        L.oracle_read_t.argtypes = [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p, C.c_void_p]
        L.oracle_color_mcs.restype = C.c_int32
        L.oracle_color_greedy.restype = C.c_int32
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_int32, C.c_int32, C.POINTER(OracleMesh), C.POINTER(OracleParams),
                                    C.c_int32, C.POINTER(OracleDeformer), C.c_int32]
        for name in ("oracle_destroy",):
            getattr(L, name).argtypes = [C.c_void_p]
        L.oracle_step.argtypes = [C.c_void_p, C.c_int32]
        L.oracle_substep_sample.argtypes = [C.c_void_p, C.c_int32]
        for name in ("oracle_get_positions", "oracle_get_velocities", "oracle_set_positions",
                     "oracle_set_velocities"):
            getattr(L, name).argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_get_rest.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_num_groups.argtypes = [C.c_void_p]
        L.oracle_group_size.argtypes = [C.c_void_p, C.c_int32]
        L.oracle_group.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_vertex_force_hessian.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                                  C.c_void_p, C.c_void_p]
        L.oracle_energy.argtypes = [C.c_void_p]
        L.oracle_energy.restype = C.c_double
        L.oracle_solve_failures.argtypes = [C.c_void_p]
        L.oracle_convergence.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_nh_element.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                        C.c_int32, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
        L.oracle_set_prev_positions.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_collide.argtypes = [C.c_void_p]
        L.oracle_collide.restype = C.c_int32
        L.oracle_get_contacts.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
        L.oracle_get_contacts.restype = C.c_int32
        L.oracle_num_surface.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_num_surface.restype = C.c_int32
        fp = C.POINTER(C.c_float)
        L.oracle_ccd_tri_point.argtypes = [fp] * 6
        L.oracle_ccd_tri_point.restype = C.c_int32
        L.oracle_tet_surface.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p]
        L.oracle_tet_walk.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, fp, fp,
                                      C.c_float, C.c_float, C.c_int32, C.POINTER(C.c_int32)]
        L.oracle_tet_walk.restype = C.c_int32
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def read_t(path: str) -> tuple[np.ndarray, np.ndarray]:
    """.t mesh (vertex ids in file order) -> positions (nv, 3) float64, tets (ntet, 4) int32."""
    L = lib()
    nv, nt = C.c_int32(), C.c_int32()
    if L.oracle_read_t(path.encode(), C.byref(nv), C.byref(nt), None, None) != 0:
        raise FileNotFoundError(path)
    X = np.empty((nv.value, 3), np.float64)
    T = np.empty((nt.value, 4), np.int32)
    L.oracle_read_t(path.encode(), C.byref(nv), C.byref(nt), X.ctypes.data, T.ctypes.data)
    return X, T


def tet_surface(X: np.ndarray, tets: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Boundary faces (nf, 3), outward, in (tet, local face) order, and the surface vertices."""
    X = np.ascontiguousarray(X, np.float64).reshape(-1)
    tets = np.ascontiguousarray(tets, np.int32).reshape(-1)
    nf, nsv = C.c_int32(), C.c_int32()
    L = lib()
    L.oracle_tet_surface(len(X) // 3, len(tets) // 4, tets.ctypes.data, X.ctypes.data, C.byref(nf), C.byref(nsv),
                         None, None)
    F = np.empty((nf.value, 3), np.int32)
    V = np.empty(nsv.value, np.int32)
    L.oracle_tet_surface(len(X) // 3, len(tets) // 4, tets.ctypes.data, X.ctypes.data, C.byref(nf), C.byref(nsv),
                         F.ctypes.data, V.ctypes.data)
    return F, V


def tet_walk(X: np.ndarray, tets: np.ndarray, face: int, target: int, origin, direction, max_dis: float = -1.0,
             ray_eps: float = 1e-10, use_static: bool = True) -> tuple[bool, int]:
    """The DCD traversal walk from surface face `face` (tet_surface order) along the ray
    origin + t * direction (FP32) -> (reached tet `target`, gave up on a size bound)."""
    X = np.ascontiguousarray(X, np.float64).reshape(-1)
    tets = np.ascontiguousarray(tets, np.int32).reshape(-1)
    fp = C.POINTER(C.c_float)
    o = np.ascontiguousarray(origin, np.float32).reshape(3)
    d = np.ascontiguousarray(direction, np.float32).reshape(3)
    st = C.c_int32()
    r = lib().oracle_tet_walk(len(X) // 3, len(tets) // 4, tets.ctypes.data, X.ctypes.data, face, target,
                              o.ctypes.data_as(fp), d.ctypes.data_as(fp), max_dis, ray_eps, int(use_static), C.byref(st))
    if r < 0:
        raise IndexError("face or target out of range")
    return bool(r), bool(st.value)


def ccd_tri_point(x0, x1, p0, p1):
    """FP32 moving point / moving triangle test -> (hit, tt, barycentrics)."""
    fp = C.POINTER(C.c_float)
    a = [np.ascontiguousarray(v, np.float32).reshape(-1) for v in (x0, x1, p0, p1)]
    tt = np.zeros(1, np.float32)
    b = np.zeros(3, np.float32)
    hit = lib().oracle_ccd_tri_point(*[v.ctypes.data_as(fp) for v in a], tt.ctypes.data_as(fp), b.ctypes.data_as(fp))
    return int(hit), float(tt[0]), b


def nh_element(x, xprev, dminv, mu: float, lmbd: float, A: float, order: int, kh: float = 0.0, kd: float = 0.0,
               dt: float = 1.0 / 300.0):
    """One tet's Neo-Hookean force (3) and 3x3 Hessian on its vertex `order` (FP64; x and
    xprev are the tet's 4 vertex positions, dminv 9 values column-major)."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    xp = np.ascontiguousarray(xprev, np.float64).reshape(-1)
    dm = np.ascontiguousarray(dminv, np.float64).reshape(-1)
    f = np.zeros(3, np.float64)
    h = np.zeros(9, np.float64)
    lib().oracle_nh_element(x.ctypes.data, xp.ctypes.data, dm.ctypes.data, mu, lmbd, A, int(order), kh, kd, dt,
                            f.ctypes.data, h.ctypes.data)
    return f, h.reshape(3, 3)


def color_mcs(nv: int, tets: np.ndarray) -> np.ndarray:
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    out = np.empty(nv, dtype=np.int32)
    n = lib().oracle_color_mcs(nv, len(tets), _ptr(tets, C.c_int32), _ptr(out, C.c_int32))
    if n < 0:
        raise RuntimeError("oracle MCS coloring failed")
    return out


def color_greedy(nv: int, tets: np.ndarray) -> np.ndarray:
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    out = np.empty(nv, dtype=np.int32)
    n = lib().oracle_color_greedy(nv, len(tets), _ptr(tets, C.c_int32), _ptr(out, C.c_int32))
    if n < 0:
        raise RuntimeError("oracle greedy coloring failed")
    return out


def color_tool(nv: int, tets: np.ndarray, algorithm: str = "mcs", balance: bool = True,
               goal_ratio: float = 1.05) -> tuple[np.ndarray, np.ndarray]:
    """The reference's GraphColoring tool (MCS or OrderedGreedy, then balancing), O(V^2) as
    the reference writes it: (colors, vertex order of the written categories)."""
    tets = np.ascontiguousarray(tets, np.int32)
    colors = np.empty(nv, np.int32)
    order = np.empty(nv, np.int32)
    L = lib()
    L.oracle_color_tool.restype = C.c_int32
    L.oracle_color_tool.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_void_p,
                                    C.c_void_p]
    n = L.oracle_color_tool(nv, len(tets), tets.ctypes.data, 0 if algorithm == "mcs" else 1, int(balance),
                            goal_ratio, colors.ctypes.data, order.ctypes.data)
    if n < 0:
        raise RuntimeError("coloring failed")
    return colors, order


def colors_to_categories(colors: np.ndarray) -> list[list[int]]:
    """GraphColoring/ColoringAlgorithms.cpp:69-80: category c lists its nodes in index order."""
    n = int(colors.max()) + 1 if len(colors) else 0
    cats: list[list[int]] = [[] for _ in range(n)]
    for v, c in enumerate(colors.tolist()):
        cats[c].append(v)
    return cats


class OracleScene:
    """A scene in the oracle. `scene` is the dict produced by
    ``gaia_gb300.scene_io.load_scene`` (meshes, params, deformers)."""

    def __init__(self, scene: dict, precision: int = 64, nthreads: int = 0):
        L = lib()
        self._keep = []
        meshes = (OracleMesh * len(scene["meshes"]))()
        for i, m in enumerate(scene["meshes"]):
            X = np.ascontiguousarray(m["X"], dtype=np.float64).reshape(-1)
            V0 = np.ascontiguousarray(m["V0"], dtype=np.float64).reshape(-1)
            tets = np.ascontiguousarray(m["tets"], dtype=np.int32).reshape(-1)
            fixed = np.ascontiguousarray(m["fixed"], dtype=np.int8)
            cats = m["colors"]
            offs = np.zeros(len(cats) + 1, dtype=np.int32)
            offs[1:] = np.cumsum([len(c) for c in cats])
            cverts = np.ascontiguousarray(np.concatenate([np.asarray(c, np.int32) for c in cats])
                                          if cats else np.zeros(0, np.int32), dtype=np.int32)
            self._keep += [X, V0, tets, fixed, offs, cverts]
            mm = meshes[i]
            mm.nv, mm.ntet = len(X) // 3, len(tets) // 4
            mm.X, mm.V0 = _ptr(X, C.c_double), _ptr(V0, C.c_double)
            mm.tets, mm.fixed = _ptr(tets, C.c_int32), _ptr(fixed, C.c_int8)
            mm.ncolors = len(cats)
            mm.color_offsets, mm.color_verts = _ptr(offs, C.c_int32), _ptr(cverts, C.c_int32)
            mat = m["material"]
            mm.miu, mm.lmbd, mm.density = mat["miu"], mat["lmbd"], mat["density"]
            mm.damping_hydrostatic = mat["dampingHydrostatic"]
            mm.damping_deviatoric = mat["dampingDeviatoric"]
            mm.exp_vel_damping = mat["exponentialVelDamping"]
            mm.const_vel_damping = mat["constantVelDamping"]
            mm.friction_dynamic = mat["frictionDynamic"]
            mm.friction_eps_v = mat["frictionEpsV"]
            mm.init_type = mat["initializationType"]
            mm.active = 1
        p = scene["params"]
        op = OracleParams()
        op.time_step, op.num_substeps, op.iterations = p["timeStep"], p["numSubsteps"], p["iterations"]
        for k in range(3):
            op.gravity[k] = p["gravity"][k]
            op.world_lo[k] = p["worldBounds"][0][k]
            op.world_hi[k] = p["worldBounds"][1][k]
        op.use_plane_ground = int(p["usePlaneGround"])
        op.boundary_stiffness = p["boundaryCollisionStiffness"]
        op.boundary_friction_mu = p["boundaryFrictionDynamic"]
        op.boundary_friction_eps_v = p["boundaryFrictionEpsV"]
        op.step_size, op.step_size_gd = p["stepSize"], p["stepSizeGD"]
        op.friction_start_iter = p["frictionStartIter"]
        op.associate_gravity = int(p["associateGravityWithInertia"])
        op.use_accelerator = int(p["useAccelerator"])
        op.accelerator_rho = p["acceleratorRho"]
        col = p.get("collision", {"allowCCD": True, "allowDCD": True})
        op.allow_ccd, op.allow_dcd = int(col["allowCCD"]), int(col["allowDCD"])
        op.collision_stiffness = p.get("collisionStiffness", 1e5)
        op.collision_off_height = p.get("collisionOffHeight", 1e7)
        op.intermediate_collision_iterations = p.get("intermediateCollisionIterations", -1)
        op.handle_self_collision = int(col.get("handleSelfCollision", True))
        op.check_feasible_region = int(col.get("checkFeasibleRegion", True))
        op.feasible_region_eps = col.get("feasibleRegionEpsilon", 1e-2)
        op.check_tet_traverse = int(col.get("checkTetTraverse", True))
        op.traverse_non_self = int(col.get("tetrahedralTraverseForNonSelfIntersection", True))
        op.stop_traversing_after_passing = int(col.get("stopTraversingAfterPassingQueryPoint", True))
        op.shift_query_to_center = int(col.get("shiftQueryPointToCenter", True))
        op.use_static_traverse = int(col.get("useStaticTraverse", True))
        op.center_shift_level = col.get("centerShiftLevel", 0.01)
        op.ray_tri_eps = col.get("rayTriIntersectionEPSILON", 1e-10)
        op.max_search_mult = col.get("maxSearchDistanceMultiplier", 1.8)
        defs = (OracleDeformer * max(1, len(scene["deformers"])))()
        for i, d in enumerate(scene["deformers"]):
            dd = defs[i]
            dd.type = 0 if d["DeformerName"] == "Rotator" else 1
            for k in range(3):
                dd.center[k] = d.get("center", [0, 0, 0])[k]
                dd.axis[k] = d.get("axis", [1, 0, 0])[k]
                dd.speed[k] = d.get("speed", [0, 0, 0])[k]
            dd.angular_velocity = d.get("angularVelocity", 0.0)
            dd.end_time = d.get("rotationEndTime", d.get("deformationEndTime", -1.0))
            sm, sv = [], []
            for mi, verts in zip(d["selectedMeshes"], d["selectedVertices"]):
                sm += [mi] * len(verts)
                sv += list(verts)
            sm = np.asarray(sm, np.int32)
            sv = np.asarray(sv, np.int32)
            self._keep += [sm, sv]
            dd.nsel = len(sm)
            dd.sel_mesh, dd.sel_vert = _ptr(sm, C.c_int32), _ptr(sv, C.c_int32)
        self._nv = [len(np.asarray(m["X"]).reshape(-1)) // 3 for m in scene["meshes"]]
        self._ntet = [len(np.asarray(m["tets"]).reshape(-1)) // 4 for m in scene["meshes"]]
        self.h = L.oracle_create(precision, len(scene["meshes"]), meshes, C.byref(op),
                                 len(scene["deformers"]), defs, nthreads)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().oracle_destroy(h)
            self.h = None

    def step(self, n: int = 1) -> None:
        lib().oracle_step(self.h, n)

    def substep_sample(self, iterations: int) -> None:
        lib().oracle_substep_sample(self.h, iterations)

    def positions(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self._nv[mesh], 3), np.float64)
        lib().oracle_get_positions(self.h, mesh, out.ctypes.data)
        return out

    def velocities(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self._nv[mesh], 3), np.float64)
        lib().oracle_get_velocities(self.h, mesh, out.ctypes.data)
        return out

    def set_positions(self, mesh: int, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64)
        lib().oracle_set_positions(self.h, mesh, x.ctypes.data)

    def set_velocities(self, mesh: int, v: np.ndarray) -> None:
        v = np.ascontiguousarray(v, np.float64)
        lib().oracle_set_velocities(self.h, mesh, v.ctypes.data)

    def rest(self, mesh: int = 0):
        nt, nv = self._ntet[mesh], self._nv[mesh]
        dminv = np.empty((nt, 9), np.float64)
        vol = np.empty(nt, np.float64)
        mass = np.empty(nv, np.float64)
        lib().oracle_get_rest(self.h, mesh, dminv.ctypes.data, vol.ctypes.data, mass.ctypes.data)
        return dminv, vol, mass

    def groups(self) -> list[np.ndarray]:
        L = lib()
        out = []
        for g in range(L.oracle_num_groups(self.h)):
            n = L.oracle_group_size(self.h, g)
            a = np.empty(2 * n, np.int32)
            L.oracle_group(self.h, g, a.ctypes.data)
            out.append(a.reshape(-1, 2))
        return out

    def vertex_force_hessian(self, mesh: int, v: int, apply_friction: bool = True):
        f = np.empty(3, np.float64)
        H = np.empty(9, np.float64)
        lib().oracle_vertex_force_hessian(self.h, mesh, v, int(apply_friction), f.ctypes.data, H.ctypes.data)
        return f, H.reshape(3, 3)

    def energy(self) -> float:
        return float(lib().oracle_energy(self.h))

    def set_prev_positions(self, mesh: int, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64)
        lib().oracle_set_prev_positions(self.h, mesh, x.ctypes.data)

    def collide(self) -> int:
        """Substep-start contact detection on the current / previous positions."""
        return int(lib().oracle_collide(self.h))

    def contacts(self) -> np.ndarray:
        """Rows (mesh, vertex, face mesh, face v0, v1, v2, surface face, kind) of the vertices in contact."""
        n = lib().oracle_get_contacts(self.h, None, 0)
        rows = np.empty((n, 8), np.int32)
        if n:
            lib().oracle_get_contacts(self.h, rows.ctypes.data, n)
        return rows

    def convergence(self) -> dict:
        """evaluateConvergence in FP64: energy, inertia, elastic, average force norm."""
        out = np.empty(4, np.float64)
        lib().oracle_convergence(self.h, out.ctypes.data)
        return {"energy": out[0], "inertia": out[1], "elastic": out[2], "avg_force_norm": out[3]}

    def solve_failures(self) -> int:
        return int(lib().oracle_solve_failures(self.h))
