"""ctypes binding of libgaia_vbd.so (the C ABI in include/gaia_vbd.h).

The library is built in-tree by ``gaia_gb300.build.build()``. There is no CPU
fallback: if the library is missing or cannot be loaded, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgaia_vbd.so")

# status codes (include/gaia_vbd.h)
OK = 0
E_INVALID_ARG = 1
E_INPUT = 2
E_COLORING = 3
E_MESH = 4
E_CUDA = 5
E_NONFINITE = 6
E_NO_DEVICE = 7
E_UNSUPPORTED = 8
E_DEVICE_TIMEOUT = 9

STATUS_NAMES = {
    OK: "OK", E_INVALID_ARG: "INVALID_ARG", E_INPUT: "INPUT", E_COLORING: "COLORING", E_MESH: "MESH",
    E_CUDA: "CUDA", E_NONFINITE: "NONFINITE", E_NO_DEVICE: "NO_DEVICE", E_UNSUPPORTED: "UNSUPPORTED",
    E_DEVICE_TIMEOUT: "DEVICE_TIMEOUT",
}


class Stats(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("lanes_per_vertex", C.c_int32), ("block_size", C.c_int32),
        ("num_groups", C.c_int32), ("num_vertices", C.c_int64), ("num_active_vertices", C.c_int64),
        ("num_incidences", C.c_int64), ("kernel_launches_per_step", C.c_int64),
        ("fp64_fallback_solves", C.c_int64), ("failed_solves", C.c_int64), ("device_bytes", C.c_int64),
        ("autotune_ms_per_iteration", C.c_double), ("solve_variant", C.c_int32), ("mesh_frames", C.c_int32),
        ("contact_detections", C.c_int64), ("contact_stack_overflow", C.c_int64),
        ("contact_traverse_bounds", C.c_int64), ("device_timeouts", C.c_int64), ("nonfinite_solves", C.c_int64),
        ("sweep_mode", C.c_int32), ("cluster_size", C.c_int32), ("sweep_ms_merged", C.c_double),
        ("sweep_ms_scenes", C.c_double), ("sweep_ms_cluster", C.c_double), ("sweep_ms_grid", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class OutputParams(C.Structure):
    _fields_ = [
        ("num_frames", C.c_int32), ("save_outputs", C.c_int32), ("save_all_models_together", C.c_int32),
        ("binary_mode_visualization_steps", C.c_int32), ("output_recovery_state", C.c_int32),
        ("output_recovery_state_step", C.c_int32), ("output_recovery_state_binary", C.c_int32),
        ("reserved", C.c_int32), ("output_ext", C.c_char * 16),
    ]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}
        d["output_ext"] = self.output_ext.decode()
        return d


class ClothStats(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("num_groups", C.c_int32), ("num_vertices", C.c_int64),
        ("num_sim_vertices", C.c_int64), ("num_faces", C.c_int64), ("num_edges", C.c_int64),
        ("kernel_launches_per_step", C.c_int64), ("detections", C.c_int64), ("truncations", C.c_int64),
        ("vf_overflow", C.c_int64), ("ee_overflow", C.c_int64), ("fv_overflow", C.c_int64),
        ("candidate_overflow", C.c_int64), ("stack_overflow", C.c_int64), ("fp64_fallback_solves", C.c_int64),
        ("failed_solves", C.c_int64), ("device_bytes", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# Every symbol the headers (gaia_vbd.h, gaia_cloth.h) declare, with its ctypes signature.
_SIGNATURES = {
    "gaia_vbd_create": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "gaia_vbd_load": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "gaia_vbd_initialize": (C.c_int, [C.c_void_p]),
    "gaia_vbd_destroy": (None, [C.c_void_p]),
    "gaia_vbd_last_error": (C.c_char_p, [C.c_void_p]),
    "gaia_vbd_last_global_error": (C.c_char_p, []),
    "gaia_vbd_run_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "gaia_vbd_synchronize": (C.c_int, [C.c_void_p]),
    "gaia_vbd_save_state": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "gaia_vbd_num_surface": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_vbd_get_surface": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_vbd_set_prev_positions": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_collide": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gaia_vbd_get_contacts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_load_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gaia_vbd_write_ply": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32, C.c_int32]),
    "gaia_vbd_write_binary": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gaia_vbd_run_step_timed": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "gaia_vbd_autotune": (C.c_int, [C.c_void_p]),
    "gaia_vbd_reset": (C.c_int, [C.c_void_p]),
    "gaia_vbd_num_meshes": (C.c_int, [C.c_void_p]),
    "gaia_vbd_num_vertices": (C.c_int64, [C.c_void_p, C.c_int32]),
    "gaia_vbd_num_tets": (C.c_int64, [C.c_void_p, C.c_int32]),
    "gaia_vbd_get_positions": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_set_positions": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_get_velocities": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_set_velocities": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_set_state_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gaia_vbd_get_positions_f32": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gaia_vbd_get_velocities_f32": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gaia_vbd_num_groups": (C.c_int, [C.c_void_p]),
    "gaia_vbd_group_size": (C.c_int64, [C.c_void_p, C.c_int32]),
    "gaia_vbd_get_group": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_get_coloring": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_get_rest_shape": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gaia_vbd_energy": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "gaia_vbd_convergence": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gaia_vbd_get_convergence_log": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "gaia_vbd_vertex_force_hessian": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_vbd_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "gaia_vbd_get_output_params": (C.c_int, [C.c_void_p, C.POINTER(OutputParams)]),
    "gaia_vbd_frame": (C.c_int64, [C.c_void_p]),
    "gaia_vbd_get_color_config": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "gaia_vbd_energy_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_void_p,
                                          C.c_void_p]),
    "gaia_vbd_color_mcs": (C.c_int32, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_vbd_color_greedy": (C.c_int32, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_vbd_color_gpu": (C.c_int32, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_uint32]),
    "gaia_vbd_color_tool": (C.c_int32, [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_float,
                                        C.c_void_p, C.c_void_p]),
    "gaia_vbd_write_categories": (C.c_int, [C.c_char_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_vbd_write_coloring": (C.c_int, [C.c_char_p, C.c_int32, C.c_void_p]),
    "gaia_vbd_write_t": (C.c_int, [C.c_char_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]),
    # cloth (gaia_cloth.h)
    "gaia_cloth_load": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "gaia_cloth_initialize": (C.c_int, [C.c_void_p]),
    "gaia_cloth_create": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "gaia_cloth_destroy": (None, [C.c_void_p]),
    "gaia_cloth_last_error": (C.c_char_p, [C.c_void_p]),
    "gaia_cloth_run_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "gaia_cloth_run_step_timed": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "gaia_cloth_synchronize": (C.c_int, [C.c_void_p]),
    "gaia_cloth_save_state": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "gaia_cloth_load_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gaia_cloth_write_ply": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32, C.c_int32]),
    "gaia_cloth_write_binary": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gaia_cloth_num_meshes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "gaia_cloth_num_vertices": (C.c_int64, [C.c_void_p, C.c_int32]),
    "gaia_cloth_num_faces": (C.c_int64, [C.c_void_p, C.c_int32]),
    "gaia_cloth_num_edges": (C.c_int64, [C.c_void_p, C.c_int32]),
    "gaia_cloth_get_positions": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_set_positions": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_get_velocities": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_set_velocities": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_get_topology": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_cloth_get_rest_shape": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gaia_cloth_num_groups": (C.c_int, [C.c_void_p]),
    "gaia_cloth_group_size": (C.c_int64, [C.c_void_p, C.c_int32]),
    "gaia_cloth_get_group": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_detect": (C.c_int, [C.c_void_p]),
    "gaia_cloth_get_vf_contacts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "gaia_cloth_get_ee_contacts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "gaia_cloth_get_bounds": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_get_min_distances": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gaia_cloth_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ClothStats)]),
    "gaia_cloth_vertex_force_hessian": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "gaia_cloth_time_solve": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "gaia_cloth_autotune": (C.c_int, [C.c_void_p]),
    "gaia_cloth_get_group_lanes": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gaia_cloth_color_greedy": (C.c_int32, [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_color_mcs": (C.c_int32, [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]),
    "gaia_cloth_color_tool": (C.c_int32, [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                          C.c_float, C.c_void_p, C.c_void_p]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libgaia_vbd.so. Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import gaia_gb300.build as b; b.build()'` "
                "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


class GaiaError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"gaia_vbd error {STATUS_NAMES.get(code, code)}: {message}")
        self.code = code
