"""ctypes front end of the cloth CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU baseline) may
import this module. It loads a cloth scene (Models.json / Parameters.json with
.obj meshes, ContactDetectorParams and static TriMeshSequence colliders) with the
reference loaders' defaults (VBDCloth/VBDClothPhysicsParameters.h:7-75,
TriMesh/TriMesh.h:27-50, VBDCloth/VBDBaseTriMesh.h:8-20, VBDCloth/VBDTriMeshStVK.h:12-27,
Parameters/PhysicsParameters.h:9-178) and runs the CPU restatement of the cloth
VBD step in cloth_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import json
import math

import numpy as np

from . import oracle as _orc


class ClothOracleMesh(C.Structure):
    _fields_ = [
        ("nv", C.c_int32), ("nf", C.c_int32), ("X", C.POINTER(C.c_double)), ("faces", C.POINTER(C.c_int32)),
        ("is_collider", C.c_int32), ("fixed", C.POINTER(C.c_int8)), ("ncolors", C.c_int32),
        ("color_offsets", C.POINTER(C.c_int32)), ("color_verts", C.POINTER(C.c_int32)),
        ("density", C.c_double), ("miu", C.c_double), ("lambda_", C.c_double), ("damping_stvk", C.c_double),
        ("damping_bending", C.c_double), ("bending_stiffness", C.c_double), ("friction_dynamic", C.c_double),
        ("friction_eps_v", C.c_double), ("exp_vel_damping", C.c_double), ("const_vel_damping", C.c_double),
        ("max_velocity", C.c_double), ("no_grav_threshold", C.c_double), ("has_no_grav_zone", C.c_int32),
        ("init_type", C.c_int32),
    ]


class ClothOracleParams(C.Structure):
    _fields_ = [
        ("gravity", C.c_double * 3), ("dt", C.c_double), ("num_substeps", C.c_int32), ("iterations", C.c_int32),
        ("world_lo", C.c_double * 3), ("world_hi", C.c_double * 3), ("boundary_friction_dynamic", C.c_double),
        ("boundary_contact_stiffness", C.c_double), ("boundary_friction_eps", C.c_double), ("step_size", C.c_double),
        ("associate_gravity", C.c_int32), ("handle_collision", C.c_int32), ("apply_acceleration", C.c_int32),
        ("cd_every_iteration", C.c_int32), ("contact_stiffness", C.c_double), ("contact_radius", C.c_double),
        ("thickness", C.c_double), ("relaxation", C.c_double), ("degenerate_thres", C.c_double),
        ("accelerator_rho", C.c_double), ("max_query_dis", C.c_double),
    ]


PHYSICS_DEFAULTS = {
    "gravity": [0.0, -10.0, 0.0], "timeStep": 0.01666666666666666666, "numSubsteps": 20, "iterations": 1,
    "worldBounds": [[-1e7, -1e7, -1e7], [1e7, 1e7, 1e7]], "boundaryFrictionDynamic": 0.1, "stepSize": 1.0,
    "associateGravityWithInertia": True, "handleCollision": True, "contactStiffness": 1e4, "contactRadius": 1.0,
    "thickness": 0.0, "conservativeStepRelaxation": 0.45, "boundaryFrictionEpsValue": 1e-2,
    "applyAcceleration": False, "acceleratorRho": 0.95, "contactDetectionEveryIteration": False,
}
OBJECT_DEFAULTS = {
    "scale": [1.0, 1.0, 1.0], "translation": [0.0, 0.0, 0.0], "rotation": [0.0, 0.0, 0.0], "density": 1.0,
    "maxVelocityMagnitude": -1.0, "hasNoGravZone": False, "noGravZoneThreshold": 0.0, "fixedPoints": [],
    "frictionDynamic": 0.1, "frictionEpsV": 0.1, "bendingStiffness": 0.0, "exponentialVelDamping": 1.0,
    "constantVelDamping": 0.0, "initializationType": 2, "miu": 1e4, "lambda": 1e4, "dampingStVK": 0.0,
    "dampingBending": 0.0,
}


def read_obj(path: str) -> tuple[np.ndarray, np.ndarray]:
    """TriMeshFEM::loadObj (TriMesh/TriMesh.cpp:280-407): vertices parsed as double and
    rounded to float32; the first three vertex indices of each face (1-based)."""
    X, F = [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                X.append([float(t[1]), float(t[2]), float(t[3])])
            elif t[0] == "f":
                F.append([int(t[k].split("/")[0]) - 1 for k in (1, 2, 3)])
    return np.asarray(X, np.float64).astype(np.float32), np.asarray(F, np.int32).reshape(-1, 3)


def transform(X: np.ndarray, rotation, scale, translation) -> np.ndarray:
    """applyRotationScalingTranslation (TriMesh/TriMesh.cpp:113-132): axis-angle rotation
    (FP64, rounded to float), then float32 scale and translation."""
    X = X.astype(np.float32).copy()
    r = np.asarray(rotation, np.float64)
    rot = math.sqrt(float(r @ r))
    if rot > 0:
        a = r / rot
        c, s = math.cos(rot), math.sin(rot)
        Cc = 1 - c
        R = np.array([[c + a[0] * a[0] * Cc, a[0] * a[1] * Cc - a[2] * s, a[0] * a[2] * Cc + a[1] * s],
                      [a[1] * a[0] * Cc + a[2] * s, c + a[1] * a[1] * Cc, a[1] * a[2] * Cc - a[0] * s],
                      [a[2] * a[0] * Cc - a[1] * s, a[2] * a[1] * Cc + a[0] * s, c + a[2] * a[2] * Cc]])
        Xd = X.astype(np.float64)
        X = np.stack([R[k, 0] * Xd[:, 0] + R[k, 1] * Xd[:, 1] + R[k, 2] * Xd[:, 2] for k in range(3)], 1).astype(np.float32)
    X = X * np.asarray(scale, np.float64).astype(np.float32)
    X = X + np.asarray(translation, np.float64).astype(np.float32)
    return X.astype(np.float32)


def load_scene(models_json: str, params_json: str) -> dict:
    """Cloth scene as the oracle's inputs (meshes in Models.json order, then colliders)."""
    with open(models_json) as f:
        models = json.load(f)["Models"]
    with open(params_json) as f:
        P = json.load(f)
    pp = dict(PHYSICS_DEFAULTS)
    pp.update({k: v for k, v in P.get("PhysicsParams", {}).items() if k in PHYSICS_DEFAULTS})
    pp["maxQueryDis"] = P.get("ContactDetectorParams", {}).get("maxQueryDis", 0.4)
    meshes = []
    for mj in models:
        o = dict(OBJECT_DEFAULTS)
        o.update({k: v for k, v in mj.items() if k in OBJECT_DEFAULTS})
        X, F = read_obj(mj["path"])
        X = transform(X, o["rotation"], o["scale"], o["translation"])
        with open(mj["verticesColoringCategoriesPath"]) as f:
            colors = [list(map(int, c)) for c in json.load(f)]
        fixed = np.zeros(len(X), np.int8)
        for v in o["fixedPoints"]:
            fixed[v] = 1
        meshes.append({"X": X, "faces": F, "collider": False, "fixed": fixed, "colors": colors, "params": o})
    for cj in P.get("ColliderParams", {}).get("ColliderMeshes", []):
        X, F = read_obj(cj["meshFiles"][0])
        X = transform(X, cj.get("rotation", [0, 0, 0]), cj.get("scale", [1, 1, 1]), cj.get("translation", [0, 0, 0]))
        o = {"frictionDynamic": cj.get("frictionDynamic", 0.1), "frictionEpsV": cj.get("frictionEpsV", 0.1)}
        meshes.append({"X": X, "faces": F, "collider": True, "params": o})
    return {"meshes": meshes, "params": pp}


def lib():
    L = _orc.lib()
    if not getattr(L, "_cloth_sigs", False):
        vp, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        sig = {
            "cloth_oracle_create": (vp, [i32, C.POINTER(ClothOracleMesh), C.POINTER(ClothOracleParams), i32]),
            "cloth_oracle_destroy": (None, [vp]), "cloth_oracle_error": (C.c_char_p, []),
            "cloth_oracle_step": (None, [vp, i32]),
            "cloth_oracle_get_positions": (None, [vp, i32, vp]), "cloth_oracle_set_positions": (None, [vp, i32, vp]),
            "cloth_oracle_get_velocities": (None, [vp, i32, vp]), "cloth_oracle_detect": (None, [vp]),
            "cloth_oracle_vf_contacts": (i64, [vp, vp, i64]), "cloth_oracle_ee_contacts": (i64, [vp, vp, i64]),
            "cloth_oracle_bounds": (None, [vp, i32, vp]), "cloth_oracle_min_distances": (None, [vp, i32, vp, vp, vp]),
            "cloth_oracle_num_edges": (i32, [vp, i32]), "cloth_oracle_topology": (None, [vp, i32, vp, vp]),
            "cloth_oracle_rest": (None, [vp, i32, vp, vp, vp]), "cloth_oracle_num_groups": (i32, [vp]),
            "cloth_oracle_group": (i64, [vp, i32, vp]), "cloth_oracle_elastic_energy": (d, [vp, i32]),
            "cloth_oracle_elastic_force_hessian": (None, [vp, i32, i32, vp, vp]),
            "cloth_oracle_counter": (i64, [vp, i32]),
            "cloth_oracle_vertex_force_hessian": (None, [vp, i32, i32, vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        L._cloth_sigs = True
    return L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class ClothOracle:
    """The cloth scene in the oracle (FP64 solve, FP32 contact detection)."""

    def __init__(self, scene: dict, nthreads: int = 0):
        L = lib()
        self._keep = []
        ms = scene["meshes"]
        arr = (ClothOracleMesh * len(ms))()
        for i, m in enumerate(ms):
            X = np.ascontiguousarray(m["X"], np.float64).reshape(-1)
            F = np.ascontiguousarray(m["faces"], np.int32).reshape(-1)
            self._keep += [X, F]
            a = arr[i]
            a.nv, a.nf = len(X) // 3, len(F) // 3
            a.X = X.ctypes.data_as(C.POINTER(C.c_double))
            a.faces = F.ctypes.data_as(C.POINTER(C.c_int32))
            a.is_collider = int(m["collider"])
            o = m["params"]
            a.friction_dynamic, a.friction_eps_v = o["frictionDynamic"], o["frictionEpsV"]
            if not m["collider"]:
                fixed = np.ascontiguousarray(m["fixed"], np.int8)
                offs = np.zeros(len(m["colors"]) + 1, np.int32)
                offs[1:] = np.cumsum([len(c) for c in m["colors"]])
                cv = np.ascontiguousarray(np.concatenate([np.asarray(c, np.int32) for c in m["colors"]]), np.int32)
                self._keep += [fixed, offs, cv]
                a.fixed = fixed.ctypes.data_as(C.POINTER(C.c_int8))
                a.ncolors = len(m["colors"])
                a.color_offsets = offs.ctypes.data_as(C.POINTER(C.c_int32))
                a.color_verts = cv.ctypes.data_as(C.POINTER(C.c_int32))
                a.density, a.miu, a.lambda_ = o["density"], o["miu"], o["lambda"]
                a.damping_stvk, a.damping_bending, a.bending_stiffness = o["dampingStVK"], o["dampingBending"], o["bendingStiffness"]
                a.exp_vel_damping, a.const_vel_damping = o["exponentialVelDamping"], o["constantVelDamping"]
                a.max_velocity, a.no_grav_threshold = o["maxVelocityMagnitude"], o["noGravZoneThreshold"]
                a.has_no_grav_zone, a.init_type = int(o["hasNoGravZone"]), int(o["initializationType"])
        p = scene["params"]
        q = ClothOracleParams()
        for k in range(3):
            q.gravity[k] = p["gravity"][k]
            q.world_lo[k] = p["worldBounds"][0][k]
            q.world_hi[k] = p["worldBounds"][1][k]
        q.dt = p["timeStep"] / p["numSubsteps"]
        q.num_substeps, q.iterations = p["numSubsteps"], p["iterations"]
        q.boundary_friction_dynamic, q.boundary_contact_stiffness = p["boundaryFrictionDynamic"], 1e4
        q.boundary_friction_eps, q.step_size = p["boundaryFrictionEpsValue"], p["stepSize"]
        q.associate_gravity, q.handle_collision = int(p["associateGravityWithInertia"]), int(p["handleCollision"])
        q.apply_acceleration, q.cd_every_iteration = int(p["applyAcceleration"]), int(p["contactDetectionEveryIteration"])
        q.contact_stiffness, q.contact_radius, q.thickness = p["contactStiffness"], p["contactRadius"], p["thickness"]
        q.relaxation, q.degenerate_thres = p["conservativeStepRelaxation"], 1e-6
        q.accelerator_rho, q.max_query_dis = p["acceleratorRho"], p["maxQueryDis"]
        self._nv = [len(m["X"]) for m in ms]
        self._nf = [len(m["faces"]) for m in ms]
        self.h = L.cloth_oracle_create(len(ms), arr, C.byref(q), nthreads)
        if not self.h:
            raise RuntimeError(L.cloth_oracle_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().cloth_oracle_destroy(self.h)
            self.h = None

    def step(self, n: int = 1) -> None:
        lib().cloth_oracle_step(self.h, n)

    def positions(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self._nv[mesh], 3))
        lib().cloth_oracle_get_positions(self.h, mesh, _p(out))
        return out

    def set_positions(self, mesh: int, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64)
        lib().cloth_oracle_set_positions(self.h, mesh, _p(x))

    def velocities(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self._nv[mesh], 3))
        lib().cloth_oracle_get_velocities(self.h, mesh, _p(out))
        return out

    def detect(self) -> None:
        lib().cloth_oracle_detect(self.h)

    def _rows(self, fn) -> np.ndarray:
        n = fn(self.h, None, 0)
        out = np.zeros((max(n, 1), 4), np.int32)
        fn(self.h, _p(out), n)
        return out[:n]

    def vf_contacts(self) -> np.ndarray:
        return self._rows(lib().cloth_oracle_vf_contacts)

    def ee_contacts(self) -> np.ndarray:
        return self._rows(lib().cloth_oracle_ee_contacts)

    def bounds(self, mesh: int = 0) -> np.ndarray:
        out = np.empty(self._nv[mesh])
        lib().cloth_oracle_bounds(self.h, mesh, _p(out))
        return out

    def min_distances(self, mesh: int = 0):
        ne = lib().cloth_oracle_num_edges(self.h, mesh)
        vf = np.empty(self._nv[mesh], np.float32)
        fv = np.empty(self._nf[mesh], np.float32)
        ee = np.empty(ne, np.float32)
        lib().cloth_oracle_min_distances(self.h, mesh, _p(vf), _p(fv), _p(ee))
        return vf, fv, ee

    def topology(self, mesh: int = 0):
        ne = lib().cloth_oracle_num_edges(self.h, mesh)
        e6 = np.empty((ne, 6), np.int32)
        fe = np.empty((self._nf[mesh], 3), np.int32)
        lib().cloth_oracle_topology(self.h, mesh, _p(e6), _p(fe))
        return e6, fe

    def rest(self, mesh: int = 0):
        dm = np.empty((self._nf[mesh], 4))
        ar = np.empty(self._nf[mesh])
        ms = np.empty(self._nv[mesh])
        lib().cloth_oracle_rest(self.h, mesh, _p(dm), _p(ar), _p(ms))
        return dm, ar, ms

    def groups(self) -> list[np.ndarray]:
        L = lib()
        out = []
        for g in range(L.cloth_oracle_num_groups(self.h)):
            n = L.cloth_oracle_group(self.h, g, None)
            a = np.empty((n, 2), np.int32)
            L.cloth_oracle_group(self.h, g, _p(a))
            out.append(a)
        return out

    def elastic_energy(self, mesh: int = 0) -> float:
        return lib().cloth_oracle_elastic_energy(self.h, mesh)

    def elastic_force_hessian(self, mesh: int, v: int):
        f = np.empty(3)
        h = np.empty(9)
        lib().cloth_oracle_elastic_force_hessian(self.h, mesh, v, _p(f), _p(h))
        return f, h.reshape(3, 3)

    def vertex_force_hessian(self, mesh: int, v: int):
        f = np.empty(3)
        h = np.empty(9)
        lib().cloth_oracle_vertex_force_hessian(self.h, mesh, v, _p(f), _p(h))
        return f, h.reshape(3, 3)

    def counters(self) -> dict:
        L = lib()
        return {"detections": L.cloth_oracle_counter(self.h, 0), "truncations": L.cloth_oracle_counter(self.h, 1),
                "failed_solves": L.cloth_oracle_counter(self.h, 2)}


def build() -> str:
    return _orc.build()
