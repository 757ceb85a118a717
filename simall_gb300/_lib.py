"""ctypes binding of libsimall_gpu.so (the C ABI declared in include/simall_gpu.h).

Loading fails loudly: if the library has not been built (simall_gb300.build)
or cannot be loaded, importing the binding raises -- there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_P = C.c_void_p
_I = C.c_int
_I64 = C.c_int64
_D = C.c_double
_SZ = C.c_size_t

SIMALL_OK = 0
MEM_HOST = 0
MEM_DEVICE = 1

STATUS_NAMES = {
    0: "SIMALL_OK", 1: "SIMALL_ERR_INVALID_ARGUMENT", 2: "SIMALL_ERR_CUDA", 3: "SIMALL_ERR_OUT_OF_MEMORY",
    4: "SIMALL_ERR_UNSORTED_CSR", 5: "SIMALL_ERR_MISSING_DIAGONAL", 6: "SIMALL_ERR_NON_FINITE",
    7: "SIMALL_ERR_NOT_POSITIVE", 8: "SIMALL_ERR_SIZE_MISMATCH", 9: "SIMALL_ERR_BREAKDOWN",
    10: "SIMALL_ERR_TIMEOUT", 11: "SIMALL_ERR_UNSUPPORTED", 12: "SIMALL_ERR_NO_DEVICE",
    13: "SIMALL_ERR_INDEX_RANGE", 14: "SIMALL_ERR_IO", 15: "SIMALL_ERR_FORMAT",
}


class SolverConfig(C.Structure):
    _fields_ = [("preconditioner", _I), ("tolerance", _D), ("max_iterations", _I), ("precision", _I),
                ("reliable_delta", _D), ("check_interval", _I), ("engine", _I), ("kind", _I), ("restart", _I),
                ("semantics", _I), ("relative_orders", _D)]


class SolverStats(C.Structure):
    _fields_ = [("iterations", _I), ("converged", _I), ("status", _I), ("reliable_updates", _I),
                ("final_residual", _D), ("true_residual", _D), ("b_norm", _D), ("seconds", _D),
                ("engine", _I), ("preconditioner", _I), ("residual_norm", _D), ("initial_residual", _D)]


class ZoneVelocity(C.Structure):
    _fields_ = [("zone", C.c_uint32), ("u", _D * 3)]


class MomentumOptions(C.Structure):
    _fields_ = [("rho", _D), ("mu", _D), ("urfU", _D), ("dt", _D), ("bdf2", _I), ("reserved", _I)]


class SimpleOptions(C.Structure):
    _fields_ = [("urfU", _D), ("urfP", _D), ("rho", _D), ("mu", _D), ("dt", _D), ("bdf2", _I), ("simplec", _I),
                ("n_outer_correctors", _I), ("n_correctors", _I), ("n_non_orth_corr", _I),
                ("momentum_predictor", _I), ("tol_u", _D), ("tol_p", _D)]


class SimpleResiduals(C.Structure):
    _fields_ = [("mom", _D * 3), ("cont", _D), ("iterations", _I * 4), ("outer", _I), ("reserved", _I)]


class CheckpointMeta(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("time", _D), ("settings_hash", C.c_uint64)]


CHECKPOINT_MESH_ARRAYS = [("node_x", "f8"), ("node_y", "f8"), ("node_z", "f8"), ("owner", "u8"), ("neighbor", "u8"),
                          ("area_x", "f8"), ("area_y", "f8"), ("area_z", "f8"), ("centroid_x", "f8"),
                          ("centroid_y", "f8"), ("centroid_z", "f8"), ("boundary_zone", "u4"),
                          ("face_node_offsets", "i4"), ("face_node_indices", "u8"), ("volume", "f8"),
                          ("cell_centroid_x", "f8"), ("cell_centroid_y", "f8"), ("cell_centroid_z", "f8"),
                          ("cell_face_offsets", "i4"), ("cell_face_indices", "u8")]


class CheckpointMesh(C.Structure):
    _fields_ = [("n_nodes", _I64), ("n_faces", _I64), ("n_cells", _I64), ("n_face_nodes", _I64),
                ("n_cell_faces", _I64)] + [(name, _P) for name, _ in CHECKPOINT_MESH_ARRAYS]


class SimpConfig(C.Structure):
    _fields_ = [("penalty", _D), ("K_min", _D), ("K_max", _D), ("filter_radius", _D), ("volume_fraction", _D),
                ("move", _D), ("damping", _D), ("rho_min", _D)]


class MeshView(C.Structure):
    _fields_ = [("n_cells", _I64), ("n_faces", _I64), ("owner", _P), ("neighbor", _P), ("area_x", _P),
                ("area_y", _P), ("area_z", _P), ("centroid_x", _P), ("centroid_y", _P), ("centroid_z", _P),
                ("boundary_zone", _P), ("cell_centroid_x", _P), ("cell_centroid_y", _P), ("cell_centroid_z", _P),
                ("cell_face_offsets", _P), ("cell_face_indices", _P)]


class BatchSystemStats(C.Structure):
    _fields_ = [("iterations", _I), ("reliable_updates", _I), ("converged", _I), ("status", _I),
                ("true_residual", _D), ("b_norm", _D)]


class BatchStats(C.Structure):
    _fields_ = [("systems", _I), ("converged", _I), ("max_iterations", _I), ("status", _I),
                ("total_iterations", _I64), ("worst_true_residual", _D), ("block_threads", _I),
                ("ctas_per_sm", _I), ("seconds", _D), ("rows_per_pass", _I), ("autotune_source", _I),
                ("cluster_rows", _I), ("cluster_ctas", _I), ("cluster_systems", _I), ("clusters", _I)]


class Boundary(C.Structure):
    _fields_ = [("zone", C.c_uint32), ("type", _I)]


# name -> (restype, argtypes)
SIGNATURES = {
    "simall_status_string": (C.c_char_p, [_I]),
    "simall_version": (C.c_char_p, []),
    "simall_context_create": (_I, [_I, _P, C.POINTER(_P)]),
    "simall_context_destroy": (_I, [_P]),
    "simall_context_last_error": (C.c_char_p, [_P]),
    "simall_context_synchronize": (_I, [_P]),
    "simall_context_stream": (_P, [_P]),
    "simall_context_kernel_launches": (_I64, [_P]),
    "simall_diagnose_bounded_wait": (_I, [_P, C.POINTER(_I), C.POINTER(_D)]),
    "simall_diagnose_sweep_params": (_I, [_I, _I, _I]),
    "simall_diagnose_mixed_params": (_I, [_I, _I]),
    "simall_diagnose_division": (_I, [_P, _I64, _P, _P, _P, _P]),
    "simall_solver_config_default": (None, [C.POINTER(SolverConfig)]),
    "simall_solver_create": (_I, [_P, C.POINTER(SolverConfig), C.POINTER(_P)]),
    "simall_solver_destroy": (_I, [_P]),
    "simall_solver_set_matrix": (_I, [_P, _I64, _I64, _P, _P, _P, _I]),
    "simall_solver_update_values": (_I, [_P, _P, _I]),
    "simall_solver_solve": (_I, [_P, _P, _P, _I, C.POINTER(SolverStats)]),
    "simall_solver_spmv": (_I, [_P, _P, _P, _I]),
    "simall_solver_precond_apply": (_I, [_P, _P, _P, _I]),
    "simall_solver_amg_levels": (_I, [_P, _P, _P, _I]),
    "simall_amg_hierarchy_digest": (_I, [_I64, _P, _P, _P, _P, _P, _I, _P]),
    "simall_solver_last_residual": (_D, [_P]),
    "simall_solver_preconditioner": (_I, [_P, _P]),
    "simall_solver_time_kernel": (_I, [_P, _I, _I, C.POINTER(_D), C.POINTER(_D)]),
    "simall_solver_solve_csr": (_I, [_P, _I64, _I64, _P, _P, _P, _P, _P, C.POINTER(SolverStats)]),
    "simall_pressure_system_create": (_I, [_P, C.POINTER(MeshView), C.POINTER(Boundary), _I, C.POINTER(_P)]),
    "simall_pressure_system_destroy": (_I, [_P]),
    "simall_pressure_system_pattern": (_I, [_P, C.POINTER(_I64), C.POINTER(_I64), _P, _P]),
    "simall_pressure_system_periodic_twins": (_I, [_P, _P]),
    "simall_pressure_system_device_arrays": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "simall_assemble_pressure_correction": (_I, [_P, _D, _P, _P, _I, C.POINTER(_I)]),
    "simall_assemble_pressure_correction_simplec": (_I, [_P, _D, _P, _P, _P, _I, C.POINTER(_I)]),
    "simall_pressure_system_setup_field_loops": (_I, [_P, C.POINTER(MeshView), _P, _P, _I]),
    "simall_compute_face_fluxes": (_I, [_P, _D, _P, _P, _P, _P, _I]),
    "simall_lsq_gradient": (_I, [_P, _P, _P, _P, _P, _I]),
    "simall_correct_fields": (_I, [_P, _D, _D, _P, _P, _P, _P, _P, _P, _P, _I]),
    "simall_assemble_momentum": (_I, [_P, C.POINTER(MomentumOptions), _P, _P, _P, _P, _P, _I]),
    "simall_momentum_device_arrays": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "simall_momentum_download": (_I, [_P, _P, _P, _P]),
    "simall_simple_options_default": (None, [C.POINTER(SimpleOptions)]),
    "simall_simple_create": (_I, [_P, _P, _P, C.POINTER(SimpleOptions), C.POINTER(_P)]),
    "simall_simple_destroy": (_I, [_P]),
    "simall_simple_set_fields": (_I, [_P, _P, _P, _I]),
    "simall_simple_get_fields": (_I, [_P, _P, _P, _P, _I]),
    "simall_simple_device_fields": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "simall_simple_iterate": (_I, [_P, C.POINTER(SimpleResiduals)]),
    "simall_simple_advance_time_step": (_I, [_P, _I, C.POINTER(SimpleResiduals)]),
    "simall_fields_create": (_I, [_P, C.POINTER(_P)]),
    "simall_fields_destroy": (_I, [_P]),
    "simall_fields_scalar": (_I, [_P, C.c_char_p, _I64, C.POINTER(_P)]),
    "simall_fields_vector": (_I, [_P, C.c_char_p, _I64, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "simall_fields_find": (_I, [_P, C.c_char_p, _I, C.POINTER(_P), C.POINTER(_I64)]),
    "simall_fields_count": (_I, [_P, C.POINTER(_I), C.POINTER(_I)]),
    "simall_fields_name": (_I, [_P, _I, _I, C.c_char_p, _I, C.POINTER(_I64)]),
    "simall_fields_upload": (_I, [_P, C.c_char_p, _I, _P, _I64]),
    "simall_fields_download": (_I, [_P, C.c_char_p, _I, _P]),
    "simall_checkpoint_write": (_I, [C.c_char_p, C.POINTER(CheckpointMesh), _P, C.POINTER(CheckpointMeta)]),
    "simall_checkpoint_read": (_I, [C.c_char_p, _P, C.POINTER(CheckpointMeta), C.POINTER(CheckpointMesh)]),
    "simall_checkpoint_mesh_free": (None, [C.POINTER(CheckpointMesh)]),
    "simall_simple_bind_fields": (_I, [_P, _P]),
    "simall_simp_config_default": (None, [C.POINTER(SimpConfig)]),
    "simall_simp_create": (_I, [_P, _P, C.POINTER(SimpConfig), C.POINTER(_P)]),
    "simall_simp_step": (_I, [_P, C.POINTER(_D)]),
    "simall_simp_destroy": (_I, [_P]),
    "simall_pressure_system_download": (_I, [_P, _P, _P]),
    "simall_solver_use_pressure_system": (_I, [_P, _P]),
    "simall_pressure_system_solve": (_I, [_P, _P, _P, _I, C.POINTER(SolverStats)]),
    "simall_assemble_face_conductance": (_I, [_P, _D, _P, _P, _P, _I]),
    "simall_face_conductance_gradient": (_I, [_P, _D, _P, _P, _P, _P, _P, _P, _I]),
    "simall_adjoint_face_conductance": (_I, [_P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _I, C.POINTER(SolverStats)]),
    "simall_batch_create": (_I, [_P, C.POINTER(SolverConfig), C.POINTER(_P)]),
    "simall_batch_destroy": (_I, [_P]),
    "simall_batch_set_systems": (_I, [_P, _I, _P, _P, _P, _P, _P]),
    "simall_batch_solve": (_I, [_P, _P, _P, _I, _P, C.POINTER(BatchStats)]),
    "simall_batch_launch_shape": (_I, [_P, _I, _I]),
    "simall_batch_autotune_cache": (_I, [_P, C.c_char_p]),
    "simall_batch_cluster_route": (_I, [_P, _I, _I, _I]),
    "simall_autotune_cache_lookup": (_I, [C.c_char_p, C.c_char_p, C.POINTER(_I)]),
    "simall_autotune_cache_store": (_I, [C.c_char_p, C.c_char_p, C.POINTER(_I), _D]),
    "simall_gpu_axpy": (_I, [_D, _P, _P, _SZ, _P]),
    "simall_gpu_scal": (_I, [_D, _P, _SZ, _P]),
    "simall_gpu_copy": (_I, [_P, _P, _SZ, _P]),
    "simall_gpu_dot": (_I, [_P, _P, _SZ, _P, C.POINTER(_D)]),
    "simall_gpu_nrm2": (_I, [_P, _SZ, _P, C.POINTER(_D)]),
    "simall_gpu_axpby": (_I, [_D, _P, _D, _P, _SZ, _P]),
    "simall_gpu_xpby": (_I, [_P, _D, _P, _SZ, _P]),
    "simall_gpu_spmv_csr": (_I, [_SZ, _P, _P, _P, _P, _P, _P]),
    "simall_gpu_jacobi_apply": (_I, [_P, _P, _P, _SZ, _P]),
    "simall_gpu_ilu0_factor_inplace": (_I, [_SZ, _P, _P, _P, _P, C.POINTER(_I)]),
    "simall_gpu_ilu0_apply": (_I, [_SZ, _P, _P, _P, _P, _P, _P]),
    "simall_mesh_cartesian": (_I, [_I, _I, _I, _D, _D, _D] + [_P] * 18),
    "simall_mesh_rcm": (_I, [_I64, _I64] + [_P] * 9),
    "CreatePlugin": (_P, []),
    "GetPluginAbi": (_I, []),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libsimall_gpu.so (building it in-tree if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"libsimall_gpu.so not built ({path}); run simall_gb300.build.build()")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class SimallError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{name}: {msg}" if msg else name)


def check(status: int, ctx=None):
    if status != SIMALL_OK:
        msg = ""
        if ctx:
            msg = (load().simall_context_last_error(ctx) or b"").decode()
        raise SimallError(status, msg)
