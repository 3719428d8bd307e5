"""Python mirror of GAIA::VBDPhysics on the VBD-step path, over libgaia_vbd.so.

Method names follow the reference (Simulator/Modules/VBD/VBDPhysics.h:36-254,
Framework/BasePhysicsFramework.h:35-119): ``loadRunningparameters`` ->
``initialize`` -> ``runStep`` / ``simulate``. All compute runs in the CUDA
library; this class only marshals arguments and raises on error codes.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import GaiaError, OutputParams, Stats, lib


def _check(rc: int, handle=None) -> None:
    if rc != 0:
        L = lib()
        msg = (L.gaia_vbd_last_error(handle) if handle else L.gaia_vbd_last_global_error()) or b""
        raise GaiaError(rc, msg.decode(errors="replace"))


class VBDPhysics:
    """One VBD scene on one GPU."""

    def __init__(self):
        self._h = None
        self.models_json = None
        self.params_json = None
        self.out_folder = None
        self.repo_root = None

    # -- VBDPhysics::loadRunningparameters (VBDPhysics.cpp:90-97): host only, no GPU needed
    def loadRunningparameters(self, models_json: str, params_json: str, out_folder: str | None = None,
                              repo_root: str | None = None) -> None:
        self.close()
        self.models_json = os.fspath(models_json)
        self.params_json = os.fspath(params_json)
        self.out_folder = out_folder
        self.repo_root = repo_root
        h = C.c_void_p()
        rr = self.repo_root.encode() if self.repo_root else None
        rc = lib().gaia_vbd_load(self.models_json.encode(), self.params_json.encode(), rr, C.byref(h))
        _check(rc)
        self._h = h

    # -- VBDPhysics::initialize (VBDPhysics.cpp:208-454) + initializeGPU (:563-651)
    def initialize(self) -> None:
        if not self._h:
            raise RuntimeError("call loadRunningparameters first")
        _check(lib().gaia_vbd_initialize(self._h), self._h)

    def close(self) -> None:
        if self._h:
            lib().gaia_vbd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        if not self._h:
            raise RuntimeError("VBDPhysics is not initialized")
        return self._h

    # -- VBDPhysics::runStep (VBDPhysics.cpp:809-837)
    def runStep(self, n: int = 1) -> None:
        _check(lib().gaia_vbd_run_step(self.handle, n), self.handle)

    @property
    def frameId(self) -> int:
        """runStep calls since initialize, or the frameId of the last recovered state."""
        return int(lib().gaia_vbd_frame(self._h)) if self._h else 0

    # -- BasePhysicFramework::writeOutputs (BasePhysicsFramework.cpp:442-506)
    def writeOutputs(self, out_folder: str, frame: int) -> None:
        o = self.outputParams()
        base = os.path.join(out_folder, f"A{frame:08d}")
        together = bool(o["save_all_models_together"])
        ext = o["output_ext"]
        if ext == "bin":
            if frame == 0:
                os.makedirs(os.path.join(out_folder, "TemplateMesh"), exist_ok=True)
                self.writePLY(os.path.join(out_folder, "TemplateMesh", "TemplateMesh.ply"), False, True)
            self.writeBinary(base + ".bin")
            if frame % max(1, o["binary_mode_visualization_steps"]) == 0:
                self.writePLY(base + ".ply", together, together)
        elif ext == "ply":
            self.writePLY(base + ".ply", together, together)
        elif ext != "obj":
            print(f"[Error] Unsupported output EXT name: {ext}")
            return
        if o["output_recovery_state"] and frame % max(1, o["output_recovery_state_step"]) == 0:
            self.saveState(os.path.join(out_folder, "RecoveryStates", f"A{frame:08d}.json"),
                           binary=bool(o["output_recovery_state_binary"]))

    # -- BasePhysicFramework::simulate (BasePhysicsFramework.cpp:284-393): frame frameId, then
    # runStep and the outputs of every frame up to numFrames (num_frames overrides it). Files
    # go to the out_folder given to loadRunningparameters; without one nothing is written.
    def simulate(self, num_frames: int | None = None, save_outputs: bool | None = None) -> int:
        o = self.outputParams()
        last = o["num_frames"] if num_frames is None else num_frames
        save = bool(o["save_outputs"]) if save_outputs is None else save_outputs
        out = self.out_folder
        if out:
            os.makedirs(out, exist_ok=True)
            if o["output_recovery_state"]:
                os.makedirs(os.path.join(out, "RecoveryStates"), exist_ok=True)
            self.writeOutputs(out, self.frameId)
        steps = 0
        while self.frameId < last:
            self.runStep(1)
            steps += 1
            if out and save:
                self.writeOutputs(out, self.frameId)
        self.synchronize()
        return steps

    def synchronize(self) -> None:
        _check(lib().gaia_vbd_synchronize(self.handle), self.handle)

    def run_steps_timed(self, n: int, sweeps: bool = True) -> tuple[float, float | None]:
        """Device time (ms) of n steps and of their color sweeps. sweeps=False: the steps run
        as runStep runs them (one graph per substep) and only the total is timed."""
        tot, sw = C.c_float(), C.c_float()
        _check(lib().gaia_vbd_run_step_timed(self.handle, n, C.byref(tot), C.byref(sw) if sweeps else None),
               self.handle)
        return tot.value, (sw.value if sweeps else None)

    def reset(self) -> None:
        """Back to the initial state (rest positions, initial velocities, t = 0)."""
        _check(lib().gaia_vbd_reset(self.handle), self.handle)

    # -- tet-mesh contact (VBDPhysics::dcd / ccd / prepareCollisionDataGPU)
    def surface(self, mesh: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """Boundary faces (nf, 3), outward, and surface vertices of a mesh."""
        if not self._h:
            raise RuntimeError("call loadRunningparameters first")
        h = self._h
        nf, nsv = C.c_int32(), C.c_int32()
        _check(lib().gaia_vbd_num_surface(h, mesh, C.byref(nf), C.byref(nsv)), h)
        F = np.empty((nf.value, 3), np.int32)
        V = np.empty(nsv.value, np.int32)
        _check(lib().gaia_vbd_get_surface(h, mesh, F.ctypes.data, V.ctypes.data), h)
        return F, V

    def setPrevPositions(self, mesh: int, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64)
        _check(lib().gaia_vbd_set_prev_positions(self.handle, mesh, x.ctypes.data), self.handle)

    def collide(self) -> int:
        n = C.c_int32()
        _check(lib().gaia_vbd_collide(self.handle, C.byref(n)), self.handle)
        return n.value

    def contacts(self) -> np.ndarray:
        """Rows (mesh, vertex, face mesh, face v0, v1, v2, surface face, kind)."""
        n = C.c_int32()
        _check(lib().gaia_vbd_get_contacts(self.handle, None, 0, C.byref(n)), self.handle)
        rows = np.empty((n.value, 8), np.int32)
        if n.value:
            _check(lib().gaia_vbd_get_contacts(self.handle, rows.ctypes.data, n.value, C.byref(n)), self.handle)
        return rows

    # -- PhysicsState (Framework/BasePhysicsFramework.h:127-319): the recovery-state file
    # writeOutputs produces (BasePhysicsFramework.cpp:495-503) and recoverFromState reads
    # (BasePhysicsFramework.cpp:264-282). FP32 positions and velocities of every mesh.
    def saveState(self, path: str, binary: bool = False) -> None:
        _check(lib().gaia_vbd_save_state(self.handle, path.encode(), int(binary)), self.handle)

    def recoverFromState(self, path: str) -> None:
        _check(lib().gaia_vbd_load_state(self.handle, path.encode()), self.handle)

    # -- output frames (BasePhysicsFramework.cpp:442-489, IO/FileIO.cpp)
    def writePLY(self, path: str, saveAllModelsTogether: bool = False, addModelName: bool = False) -> None:
        _check(lib().gaia_vbd_write_ply(self.handle, path.encode(), int(saveAllModelsTogether), int(addModelName)),
               self.handle)

    def writeBinary(self, path: str) -> None:
        _check(lib().gaia_vbd_write_binary(self.handle, path.encode()), self.handle)

    def autotune(self) -> None:
        _check(lib().gaia_vbd_autotune(self.handle), self.handle)

    # -- state
    def numMeshes(self) -> int:
        return lib().gaia_vbd_num_meshes(self.handle)

    def numVertices(self, mesh: int = 0) -> int:
        return int(lib().gaia_vbd_num_vertices(self.handle, mesh))

    def numTets(self, mesh: int = 0) -> int:
        return int(lib().gaia_vbd_num_tets(self.handle, mesh))

    def positions(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self.numVertices(mesh), 3), np.float64)
        _check(lib().gaia_vbd_get_positions(self.handle, mesh, out.ctypes.data), self.handle)
        return out

    def velocities(self, mesh: int = 0) -> np.ndarray:
        out = np.empty((self.numVertices(mesh), 3), np.float64)
        _check(lib().gaia_vbd_get_velocities(self.handle, mesh, out.ctypes.data), self.handle)
        return out

    def setPositions(self, mesh: int, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64)
        if x.size != 3 * self.numVertices(mesh):
            raise ValueError("wrong size")
        _check(lib().gaia_vbd_set_positions(self.handle, mesh, x.ctypes.data), self.handle)

    def setVelocities(self, mesh: int, v: np.ndarray) -> None:
        v = np.ascontiguousarray(v, np.float64)
        if v.size != 3 * self.numVertices(mesh):
            raise ValueError("wrong size")
        _check(lib().gaia_vbd_set_velocities(self.handle, mesh, v.ctypes.data), self.handle)

    def set_state_f32(self, x_ptr: int, v_ptr: int) -> None:
        """Whole-scene FP32 state from host pointers (page-locked for full bandwidth)."""
        _check(lib().gaia_vbd_set_state_f32(self.handle, x_ptr, v_ptr), self.handle)

    def get_positions_f32(self, x_ptr: int) -> None:
        _check(lib().gaia_vbd_get_positions_f32(self.handle, x_ptr), self.handle)

    def get_velocities_f32(self, v_ptr: int) -> None:
        _check(lib().gaia_vbd_get_velocities_f32(self.handle, v_ptr), self.handle)

    # -- introspection
    def parallelGroups(self) -> list[np.ndarray]:
        L = lib()
        out = []
        for g in range(L.gaia_vbd_num_groups(self.handle)):
            n = int(L.gaia_vbd_group_size(self.handle, g))
            a = np.empty(2 * n, np.int32)
            _check(L.gaia_vbd_get_group(self.handle, g, a.ctypes.data), self.handle)
            out.append(a.reshape(-1, 2))
        return out

    def coloring(self, mesh: int = 0) -> np.ndarray:
        out = np.empty(self.numVertices(mesh), np.int32)
        _check(lib().gaia_vbd_get_coloring(self.handle, mesh, out.ctypes.data), self.handle)
        return out

    def restShape(self, mesh: int = 0):
        nt, nv = self.numTets(mesh), self.numVertices(mesh)
        dminv = np.empty((nt, 9), np.float64)
        vol = np.empty(nt, np.float64)
        mass = np.empty(nv, np.float64)
        _check(lib().gaia_vbd_get_rest_shape(self.handle, mesh, dminv.ctypes.data, vol.ctypes.data,
                                             mass.ctypes.data), self.handle)
        return dminv, vol, mass

    def energy(self) -> float:
        e = C.c_double()
        _check(lib().gaia_vbd_energy(self.handle, C.byref(e)), self.handle)
        return e.value

    def evaluateConvergence(self) -> dict:
        """evaluateConvergenceGPU on the current state, reduced in FP64 in a fixed order:
        energy, inertia and elastic energy, average force norm."""
        out = np.empty(4, np.float64)
        _check(lib().gaia_vbd_convergence(self.handle, out.ctypes.data), self.handle)
        return {"energy": out[0], "inertia": out[1], "elastic": out[2], "avg_force_norm": out[3]}

    def convergenceLog(self) -> np.ndarray:
        """The last step's in-graph records (PhysicsParams evaluateConvergence): rows of
        substep, iteration (-1 = initial guess), energy, inertia, elastic, avg force norm."""
        n = C.c_int32()
        _check(lib().gaia_vbd_get_convergence_log(self.handle, None, 0, C.byref(n)), self.handle)
        rows = np.zeros((n.value, 6), np.float64)
        if n.value:
            _check(lib().gaia_vbd_get_convergence_log(self.handle, rows.ctypes.data, n.value, C.byref(n)),
                   self.handle)
        return rows

    def vertexForceHessian(self, mesh: int, v: int, apply_friction: bool = True):
        f = np.empty(3, np.float64)
        H = np.empty(9, np.float64)
        _check(lib().gaia_vbd_vertex_force_hessian(self.handle, mesh, v, int(apply_friction), f.ctypes.data,
                                                   H.ctypes.data), self.handle)
        return f, H.reshape(3, 3)

    def colorConfigs(self) -> list[dict]:
        """Per merged color: lanes per vertex, block size, kernel variant, tuned ms per launch."""
        out = []
        for g in range(lib().gaia_vbd_num_groups(self.handle)):
            L, B, V, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_float()
            _check(lib().gaia_vbd_get_color_config(self.handle, g, C.byref(L), C.byref(B), C.byref(V), C.byref(ms)),
                   self.handle)
            out.append({"lanes": L.value, "block": B.value, "variant": V.value, "ms": ms.value})
        return out

    def outputParams(self) -> dict:
        """The frame loop's output settings from Parameters.json (host data)."""
        if not self._h:
            raise RuntimeError("call loadRunningparameters first")
        o = OutputParams()
        _check(lib().gaia_vbd_get_output_params(self._h, C.byref(o)), self._h)
        return o.as_dict()

    def stats(self) -> dict:
        s = Stats()
        _check(lib().gaia_vbd_get_stats(self.handle, C.byref(s)), self.handle)
        return s.as_dict()


def color_greedy(nv: int, tets: np.ndarray) -> np.ndarray:
    """GraphColoring tool, OrderedGreedy (gready.cpp:15-117), bit-exact."""
    tets = np.ascontiguousarray(tets, np.int32)
    out = np.empty(nv, np.int32)
    n = lib().gaia_vbd_color_greedy(nv, len(tets), tets.ctypes.data, out.ctypes.data)
    if n < 0:
        raise GaiaError(2, (lib().gaia_vbd_last_global_error() or b"").decode())
    return out


def color_tool(nv: int, tets: np.ndarray, algorithm: str = "mcs", balance: bool = True,
               goal_ratio: float = 1.05) -> tuple[np.ndarray, np.ndarray]:
    """The reference's GraphColoring tool (defaults: MCS, balanced to a 1.05 size ratio):
    (colors, vertex order of the written categories)."""
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    colors = np.empty(nv, dtype=np.int32)
    order = np.empty(nv, dtype=np.int32)
    n = lib().gaia_vbd_color_tool(nv, len(tets), tets.ctypes.data, 0 if algorithm == "mcs" else 1, int(balance),
                                  goal_ratio, colors.ctypes.data, order.ctypes.data)
    if n < 0:
        raise RuntimeError("coloring failed")
    return colors, order


def write_categories(path: str, colors: np.ndarray, order: np.ndarray) -> None:
    colors = np.ascontiguousarray(colors, np.int32)
    order = np.ascontiguousarray(order, np.int32)
    _check(lib().gaia_vbd_write_categories(os.fspath(path).encode(), len(colors), colors.ctypes.data,
                                           order.ctypes.data))


def color_gpu(nv: int, tets: np.ndarray, seed: int = 1) -> np.ndarray:
    """Jones-Plassmann vertex coloring on the GPU (not the reference's coloring)."""
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    out = np.empty(nv, dtype=np.int32)
    n = lib().gaia_vbd_color_gpu(nv, len(tets), tets.ctypes.data, out.ctypes.data, seed)
    if n < 0:
        raise RuntimeError("GPU coloring failed")
    return out


def color_mcs(nv: int, tets: np.ndarray) -> np.ndarray:
    """GraphColoring tool, MCS (mcs.cpp:14-168), bit-exact."""
    tets = np.ascontiguousarray(tets, np.int32)
    out = np.empty(nv, np.int32)
    n = lib().gaia_vbd_color_mcs(nv, len(tets), tets.ctypes.data, out.ctypes.data)
    if n < 0:
        raise GaiaError(2, (lib().gaia_vbd_last_global_error() or b"").decode())
    return out


def write_coloring(path: str, colors: np.ndarray) -> None:
    colors = np.ascontiguousarray(colors, np.int32)
    _check(lib().gaia_vbd_write_coloring(os.fspath(path).encode(), len(colors), colors.ctypes.data))


def write_t(path: str, X: np.ndarray, tets: np.ndarray) -> None:
    X = np.ascontiguousarray(X, np.float64)
    tets = np.ascontiguousarray(tets, np.int32)
    _check(lib().gaia_vbd_write_t(os.fspath(path).encode(), len(X), X.ctypes.data, len(tets), tets.ctypes.data))
