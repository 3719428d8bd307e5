"""Python mirror of Gaia's VBDClothSimulationFramework over the C ABI
(include/gaia_cloth.h): loadRunningparameters / initialize / runStep / simulate,
state access and the contact detector's outputs. Everything runs in
libgaia_vbd.so; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import ClothStats, GaiaError, lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class VBDClothSimulationFramework:
    """VBDCloth/VBDClothPhysics.h:24-255 for the VBD path (runStep_CDEveryIter)."""

    def __init__(self):
        self.h = None

    def _check(self, rc: int) -> None:
        if rc != 0:
            msg = lib().gaia_cloth_last_error(self.h) if self.h else lib().gaia_vbd_last_global_error()
            raise GaiaError(rc, (msg or b"").decode())

    # ---- set-up (BasePhysicFramework::loadRunningparameters / initialize) ------------
    def loadRunningparameters(self, models_json: str, params_json: str, repo_root: str | None = None) -> None:
        h = C.c_void_p()
        rc = lib().gaia_cloth_load(models_json.encode(), params_json.encode(),
                                   repo_root.encode() if repo_root else None, C.byref(h))
        if rc != 0:
            raise GaiaError(rc, lib().gaia_vbd_last_global_error().decode())
        self.close()
        self.h = h

    def initialize(self) -> None:
        self._check(lib().gaia_cloth_initialize(self.h))

    def close(self) -> None:
        if self.h:
            lib().gaia_cloth_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # ---- stepping ----------------------------------------------------------------------
    def runStep(self, n: int = 1) -> None:
        self._check(lib().gaia_cloth_run_step(self.h, n))

    def simulate(self, num_frames: int) -> None:
        self.runStep(num_frames)
        self.synchronize()

    def synchronize(self) -> None:
        self._check(lib().gaia_cloth_synchronize(self.h))

    # ---- PhysicsState recovery files (Framework/BasePhysicsFramework.h:127-319) -------
    def saveState(self, path: str, binary: bool = False) -> None:
        self._check(lib().gaia_cloth_save_state(self.h, path.encode(), int(binary)))

    def recoverFromState(self, path: str) -> None:
        self._check(lib().gaia_cloth_load_state(self.h, path.encode()))

    def writePLY(self, path: str, saveAllModelsTogether: bool = False, addModelName: bool = False) -> None:
        self._check(lib().gaia_cloth_write_ply(self.h, path.encode(), int(saveAllModelsTogether), int(addModelName)))

    def writeBinary(self, path: str) -> None:
        self._check(lib().gaia_cloth_write_binary(self.h, path.encode()))

    def run_steps_timed(self, n: int) -> float:
        ms = C.c_float()
        self._check(lib().gaia_cloth_run_step_timed(self.h, n, C.byref(ms)))
        return float(ms.value)

    # ---- meshes and state ----------------------------------------------------------------
    def numMeshes(self) -> tuple[int, int]:
        a, b = C.c_int32(), C.c_int32()
        self._check(lib().gaia_cloth_num_meshes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def numVertices(self, mesh: int = 0) -> int:
        return int(lib().gaia_cloth_num_vertices(self.h, mesh))

    def numFaces(self, mesh: int = 0) -> int:
        return int(lib().gaia_cloth_num_faces(self.h, mesh))

    def numEdges(self, mesh: int = 0) -> int:
        return int(lib().gaia_cloth_num_edges(self.h, mesh))

    def positions(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self.numVertices(mesh), 3))
        self._check(lib().gaia_cloth_get_positions(self.h, mesh, _ptr(out)))
        return out

    def setPositions(self, mesh: int, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64)
        assert x.shape == (self.numVertices(mesh), 3)
        self._check(lib().gaia_cloth_set_positions(self.h, mesh, _ptr(x)))

    def velocities(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self.numVertices(mesh), 3))
        self._check(lib().gaia_cloth_get_velocities(self.h, mesh, _ptr(out)))
        return out

    def setVelocities(self, mesh: int, v: np.ndarray) -> None:
        v = np.ascontiguousarray(v, np.float64)
        assert v.shape == (self.numVertices(mesh), 3)
        self._check(lib().gaia_cloth_set_velocities(self.h, mesh, _ptr(v)))

    def topology(self, mesh: int = 0) -> tuple[np.ndarray, np.ndarray]:
        e6 = np.empty((self.numEdges(mesh), 6), np.int32)
        fe = np.empty((self.numFaces(mesh), 3), np.int32)
        self._check(lib().gaia_cloth_get_topology(self.h, mesh, _ptr(e6), _ptr(fe)))
        return e6, fe

    def restShape(self, mesh: int = 0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        dm = np.empty((self.numFaces(mesh), 4))
        ar = np.empty(self.numFaces(mesh))
        ms = np.empty(self.numVertices(mesh))
        self._check(lib().gaia_cloth_get_rest_shape(self.h, mesh, _ptr(dm), _ptr(ar), _ptr(ms)))
        return dm, ar, ms

    def parallelGroups(self) -> list[np.ndarray]:
        out = []
        for g in range(lib().gaia_cloth_num_groups(self.h)):
            a = np.empty((lib().gaia_cloth_group_size(self.h, g), 2), np.int32)
            self._check(lib().gaia_cloth_get_group(self.h, g, _ptr(a)))
            out.append(a)
        return out

    # ---- contact detection -----------------------------------------------------------------
    def applyCollisionDetection(self) -> None:
        self._check(lib().gaia_cloth_detect(self.h))

    def _rows(self, fn) -> np.ndarray:
        n = C.c_int64()
        self._check(fn(self.h, None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 4), np.int32)
        self._check(fn(self.h, _ptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def vfContacts(self) -> np.ndarray:
        """(vertex mesh, vertex, face mesh, face) rows of the last detection."""
        return self._rows(lib().gaia_cloth_get_vf_contacts)

    def eeContacts(self) -> np.ndarray:
        """(mesh 1, edge 1, mesh 2, edge 2) rows of the last detection."""
        return self._rows(lib().gaia_cloth_get_ee_contacts)

    def conservativeBounds(self, mesh: int = 0) -> np.ndarray:
        out = np.empty(self.numVertices(mesh))
        self._check(lib().gaia_cloth_get_bounds(self.h, mesh, _ptr(out)))
        return out

    def minDistances(self, mesh: int = 0):
        vf = np.empty(self.numVertices(mesh), np.float32)
        fv = np.empty(self.numFaces(mesh), np.float32)
        ns, _ = self.numMeshes()
        ee = np.empty(self.numEdges(mesh), np.float32) if mesh < ns else None
        self._check(lib().gaia_cloth_get_min_distances(self.h, mesh, _ptr(vf), _ptr(fv),
                                                       _ptr(ee) if ee is not None else None))
        return vf, fv, ee

    def vertexForceHessian(self, mesh: int, v: int) -> tuple[np.ndarray, np.ndarray]:
        f = np.empty(3)
        h = np.empty(9)
        self._check(lib().gaia_cloth_vertex_force_hessian(self.h, mesh, v, _ptr(f), _ptr(h)))
        return f, h.reshape(3, 3)

    def autotune(self) -> None:
        """Re-time the solve's lanes per vertex per color on the current state."""
        self._check(lib().gaia_cloth_autotune(self.h))

    def groupLanes(self) -> list[int]:
        out = np.empty(lib().gaia_cloth_num_groups(self.h), np.int32)
        self._check(lib().gaia_cloth_get_group_lanes(self.h, _ptr(out)))
        return out.tolist()

    def time_solve(self, reps: int = 5) -> float:
        """Milliseconds per sweep of the per-color solve kernels (state restored)."""
        ms = C.c_float()
        self._check(lib().gaia_cloth_time_solve(self.h, reps, C.byref(ms)))
        return float(ms.value)

    def stats(self) -> dict:
        s = ClothStats()
        self._check(lib().gaia_cloth_get_stats(self.h, C.byref(s)))
        return s.as_dict()


def color_trimesh_tool(nv: int, faces: np.ndarray, algorithm: str = "mcs", bending: bool = False, balance: bool = True,
                       goal_ratio: float = 1.05) -> tuple[np.ndarray, np.ndarray]:
    """The GraphColoring tool on a triangle mesh (defaults: MCS, balanced to 1.05):
    (colors, vertex order of the written categories)."""
    f = np.ascontiguousarray(faces, np.int32).reshape(-1)
    colors = np.empty(nv, np.int32)
    order = np.empty(nv, np.int32)
    n = lib().gaia_cloth_color_tool(nv, len(f) // 3, _ptr(f), int(bending), 0 if algorithm == "mcs" else 1,
                                    int(balance), goal_ratio, _ptr(colors), _ptr(order))
    if n < 0:
        raise GaiaError(1, lib().gaia_vbd_last_global_error().decode())
    return colors, order


def color_trimesh(nv: int, faces: np.ndarray, algorithm: str = "greedy", bending: bool = False) -> np.ndarray:
    """GraphColoring tool on a triangle mesh (vertex graph): per-vertex colors."""
    f = np.ascontiguousarray(faces, np.int32).reshape(-1)
    out = np.empty(nv, np.int32)
    fn = lib().gaia_cloth_color_greedy if algorithm == "greedy" else lib().gaia_cloth_color_mcs
    n = fn(nv, len(f) // 3, _ptr(f), int(bending), _ptr(out))
    if n < 0:
        raise GaiaError(1, lib().gaia_vbd_last_global_error().decode())
    return out
