"""Python restatement of the reference's VBD input handling — TEST INFRASTRUCTURE ONLY.

Reads Models.json / Parameters.json with the reference's keys and defaults
(Parameters/PhysicsParameters.h:9-178, VBD/VBDPhysicsParameters.h:5-147,
Materials/Materials.h:12-75, VBD/VBD_BaseMaterial.h:21-49,
VBD/VBD_NeoHookean.h:16-33), substitutes ${REPO_ROOT}
(Parser/InputHandler.h:128-185), loads .t meshes and coloring files, applies
rotation / scale / translation in FP32 (TetMesh/TetMeshFEM.cpp:359-384) and
marks deformer-selected vertices fixed (VBD/VBDDeformer.h:20-43). The result
feeds ``oracle.OracleScene``; the product loads the same files in C++.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

PHYSICS_DEFAULTS = {
    "gravity": [0.0, -10.0, 0.0], "timeStep": 0.01666666666666666666, "numSubsteps": 20, "iterations": 1,
    "usePlaneGround": True, "worldBounds": [[-1e7, -1e7, -1e7], [1e7, 1e7, 1e7]],
    "boundaryFrictionDynamic": 0.1, "boundaryFrictionEpsV": 1.0, "boundaryCollisionStiffness": 1e5,
    "stepSize": 1.0, "stepSizeGD": 1e-3, "frictionStartIter": 0, "associateGravityWithInertia": True,
    "useAccelerator": False, "acceleratorRho": 0.93,
    "collisionStiffness": 1e5, "collisionOffHeight": 1e7, "intermediateCollisionIterations": -1,
}
# CollisionDetector/CollisionDetertionParameters.h:41-78 (the keys the VBD step reads)
COLLISION_DEFAULTS = {"allowCCD": True, "allowDCD": True, "handleSelfCollision": True, "checkFeasibleRegion": True,
                      "feasibleRegionEpsilon": 1e-2, "checkTetTraverse": True,
                      "tetrahedralTraverseForNonSelfIntersection": True, "stopTraversingAfterPassingQueryPoint": True,
                      "shiftQueryPointToCenter": True, "useStaticTraverse": True, "loopLessTraverse": False,
                      "centerShiftLevel": 0.01, "rayTriIntersectionEPSILON": 1e-10,
                      "maxSearchDistanceMultiplier": 1.8}
MATERIAL_DEFAULTS = {
    "density": 1.0, "frictionDynamic": 0.1, "frictionEpsV": 0.01, "exponentialVelDamping": 1.0,
    "constantVelDamping": 0.0, "initializationType": 0, "miu": 1e4, "lmbd": 1e4,
    "dampingDeviatoric": 0.0, "dampingHydrostatic": 0.0,
}


def load_t(path: str) -> tuple[np.ndarray, np.ndarray]:
    """.t mesh: 'Vertex id x y z' / 'Tet id a b c d'; vertex ids map to file order."""
    if os.path.getsize(path) > (4 << 20):
        from . import oracle as _o  # C reader for large files (ids in file order)
        return _o.read_t(path)
    ids, X, T = [], [], []
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "Vertex":
                ids.append(int(p[1]))
                X.append((float(p[2]), float(p[3]), float(p[4])))
            elif p[0] == "Tet":
                T.append((int(p[2]), int(p[3]), int(p[4]), int(p[5])))
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.int64).reshape(-1, 4)
    if ids != list(range(len(ids))):
        lut = {v: i for i, v in enumerate(ids)}
        T = np.vectorize(lut.__getitem__)(T)
    return X, T.astype(np.int32)


def _subst(s: str, root: str | None) -> str:
    return s.replace("${REPO_ROOT}", root) if root else s


def transform_fp32(X: np.ndarray, rotation, scale, translation) -> np.ndarray:
    """Positions as FP32 after axis-angle rotation, scale, translation."""
    Xf = X.astype(np.float32)
    rot = math.sqrt(sum(r * r for r in rotation))
    if rot > 0:
        a = [r / rot for r in rotation]
        c, s = math.cos(rot), math.sin(rot)
        C = 1 - c
        R = [[c + a[0] * a[0] * C, a[0] * a[1] * C - a[2] * s, a[0] * a[2] * C + a[1] * s],
             [a[1] * a[0] * C + a[2] * s, c + a[1] * a[1] * C, a[1] * a[2] * C - a[0] * s],
             [a[2] * a[0] * C - a[1] * s, a[2] * a[1] * C + a[0] * s, c + a[2] * a[2] * C]]
        Xd = Xf.astype(np.float64)
        Xf = np.stack([(R[r][0] * Xd[:, 0] + R[r][1] * Xd[:, 1]) + R[r][2] * Xd[:, 2] for r in range(3)],
                      1).astype(np.float32)
    Xf = Xf * np.asarray(scale, np.float64).astype(np.float32)
    Xf = Xf + np.asarray(translation, np.float64).astype(np.float32)
    return Xf


def load_scene(models_json: str, params_json: str, repo_root: str | None = None, colorer=None) -> dict:
    """`colorer(nv, tets) -> colors` is used for models without a coloring file
    (the reference's OrderedGreedy; pass the oracle's restatement)."""
    with open(_subst(models_json, repo_root)) as f:
        models = json.load(f)
    with open(_subst(params_json, repo_root)) as f:
        params = json.load(f)
    pp = dict(PHYSICS_DEFAULTS)
    pp.update({k: v for k, v in params.get("PhysicsParams", {}).items() if k in PHYSICS_DEFAULTS or k in (
        "gpuPrecision",)})
    meshes = []
    for mj in models["Models"]:
        mat = dict(MATERIAL_DEFAULTS)
        mat.update({k: mj[k] for k in MATERIAL_DEFAULTS if k in mj})
        X, T = load_t(_subst(mj["path"], repo_root))
        Xf = transform_fp32(X, mj.get("rotation", [0, 0, 0]), mj.get("scale", [1, 1, 1]),
                            mj.get("translation", [0, 0, 0]))
        cp = mj.get("verticesColoringCategoriesPath", "")
        if cp:
            with open(_subst(cp, repo_root)) as f:
                colors = [list(map(int, c)) for c in json.load(f)]
        else:
            if colorer is None:
                raise ValueError("model has no coloring file and no colorer was given")
            col = colorer(len(Xf), T)
            colors = [np.flatnonzero(col == c).tolist() for c in range(int(col.max()) + 1)]
        fixed = np.zeros(len(Xf), np.int8)
        for v in mj.get("fixedPoints", []):
            fixed[v] = 1
        V0 = np.tile(np.asarray(mj.get("initialVelocity", [0, 0, 0]), np.float64).astype(np.float32), (len(Xf), 1))
        meshes.append({"X": Xf.astype(np.float64), "V0": V0.astype(np.float64), "tets": T, "fixed": fixed,
                       "colors": colors, "material": mat})
    deformers = params.get("Deformers", [])
    for d in deformers:
        for mi, verts in zip(d["selectedMeshes"], d["selectedVertices"]):
            meshes[mi]["fixed"][np.asarray(verts, np.int64)] = 1
    cp = dict(COLLISION_DEFAULTS)
    cp.update({k: v for k, v in params.get("CollisionParams", {}).items() if k in COLLISION_DEFAULTS})
    if cp["loopLessTraverse"]:
        raise ValueError("CollisionParams loopLessTraverse is not supported")
    pp["collision"] = cp
    return {"meshes": meshes, "params": pp, "deformers": deformers}
