"""ctypes bindings of libfempar_gpu.so (declarations in include/fempar_gpu.h).

The shared library is built in-tree by ``fempar_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback for the product path.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfempar_gpu.so")

FG_OK = 0
STATUS = {0: "FG_OK", -1: "FG_ERR_BADARG", -2: "FG_ERR_OOM", -3: "FG_ERR_CUDA", -4: "FG_ERR_NOT_CONVERGED",
          -5: "FG_ERR_NUMERIC", -6: "FG_ERR_TIMEOUT", -7: "FG_ERR_UNSUPPORTED", -8: "FG_ERR_NO_DEVICE"}
FG_ERR_NOT_CONVERGED = -4

FG_POISSON, FG_ELASTICITY = 0, 1
FG_FN_ZERO, FG_FN_CONST, FG_FN_SHARP_WAVE, FG_FN_LINEAR, FG_FN_QP_VALUES = 0, 1, 2, 3, 4
FG_INPUTS_ON_DEVICE, FG_LEAN_SYSTEM, FG_FAST_INTEGRATION = 1, 2, 4
FG_PREC_NONE, FG_PREC_JACOBI, FG_PREC_BDDC = 0, 1, 2
FG_BDDC_WEIGHT_MULTIPLICITY, FG_BDDC_WEIGHT_STIFFNESS, FG_BDDC_WEIGHT_SUBPART = 0, 1, 2
FG_BDDC_HANDLER_STANDARD, FG_BDDC_HANDLER_ELASTICITY = 0, 1
FG_FP64, FG_MIXED = 0, 1
FG_DENSE_LOWER = 1
FG_RES_RES, FG_RES_RHS, FG_DELTA_RHS, FG_DELTA_DELTA, FG_RES_NRMGIVEN_RHS_NRMGIVEN, FG_RES_NRMGIVEN_RES_NRMGIVEN = range(6)

# every symbol include/fempar_gpu.h declares
EXPORTS = [
    "fg_status_string", "fg_last_error", "fg_version",
    "fg_ctx_create", "fg_ctx_destroy", "fg_ctx_memory", "fg_ctx_get_stream", "fg_ctx_kernel_launches",
    "fg_mesh_create_structured", "fg_mesh_destroy", "fg_mesh_create_unstructured", "fg_mesh_read_gid",
    "fg_mesh_get_info", "fg_mesh_get_vefs",
    "fg_space_create", "fg_space_create_dg", "fg_space_destroy", "fg_space_release_pattern", "fg_space_get_info", "fg_space_get_dof_map",
    "fg_space_get_dirichlet_coords", "fg_space_get_qp_coords",
    "fg_assemble", "fg_system_reassemble", "fg_system_destroy",
    "fg_system_export_csr", "fg_system_export_rhs", "fg_system_export_dirichlet_values",
    "fg_system_spmv_device", "fg_system_spmv_device_noalloc", "fg_system_spmv_solver_layout_device",
    "fg_solve", "fg_solve_device", "fg_system_error_norms",
    "fg_solver_params_default", "fg_integrand_default",
    "fg_bddc_params_default", "fg_bddc_create", "fg_bddc_numerical_setup", "fg_bddc_get_info",
    "fg_bddc_apply_device", "fg_bddc_solve", "fg_bddc_solve_device", "fg_bddc_destroy",
    "fg_batch_create", "fg_batch_run", "fg_batch_get_info", "fg_batch_destroy",
    "fg_partition_create", "fg_partition_destroy", "fg_partition_get_info", "fg_partition_get_dof_import_sizes",
    "fg_partition_get_dof_import", "fg_partition_assemble", "fg_partition_comm_device", "fg_partition_solve",
    "fg_request_footprint", "fg_server_create", "fg_server_submit", "fg_server_wait", "fg_server_take_solution",
    "fg_server_stats", "fg_server_destroy", "fg_dense_gemm_nt",
]


class Integrand(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("cell_coef", C.c_void_p),
        ("coef_const", C.c_double),
        ("nu", C.c_double),
        ("source_fn", C.c_int),
        ("fn_param", C.c_double * 8),
        ("qp_source", C.c_void_p),
        ("boundary_fn", C.c_int),
        ("dirichlet_values", C.c_void_p),
        ("flags", C.c_int),
    ]


class MeshInfo(C.Structure):
    _fields_ = [
        ("num_cells", C.c_int64), ("num_vertices", C.c_int64), ("num_edges", C.c_int64),
        ("num_faces", C.c_int64), ("num_vefs", C.c_int64),
        ("unstructured", C.c_int32), ("max_cells_around_vertex", C.c_int32),
    ]


class PartitionInfo(C.Structure):
    _fields_ = [("num_parts", C.c_int32), ("num_local_dofs", C.c_int64), ("max_part_dofs", C.c_int64),
                ("num_couplings", C.c_int64), ("nnz_full", C.c_int64), ("nnz_upper", C.c_int64),
                ("num_dirichlet", C.c_int64)]


class DofImportSizes(C.Structure):
    _fields_ = [("num_dofs", C.c_int32), ("num_interior_dofs", C.c_int32), ("num_interface_dofs", C.c_int32),
                ("num_rcv", C.c_int32), ("num_snd", C.c_int32), ("num_unpack", C.c_int32), ("num_pack", C.c_int32),
                ("num_cells", C.c_int64), ("first_local_dof", C.c_int64)]


class SolverParams(C.Structure):
    _fields_ = [
        ("precond", C.c_int),
        ("precision", C.c_int),
        ("criterion", C.c_int),
        ("rtol", C.c_double),
        ("atol", C.c_double),
        ("max_iters", C.c_int),
        ("inner_rtol", C.c_double),
        ("inner_max_iters", C.c_int),
        ("check_every", C.c_int),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_int),
        ("outer_iterations", C.c_int),
        ("converged", C.c_int),
        ("error_estimate", C.c_double),
        ("tolerance", C.c_double),
        ("solve_ms", C.c_double),
        ("kernel_launches", C.c_int64),
    ]


class SpaceInfo(C.Structure):
    _fields_ = [
        ("num_dims", C.c_int), ("order", C.c_int), ("ncomp", C.c_int),
        ("dofs_per_cell", C.c_int), ("qp_per_cell", C.c_int),
        ("num_cells", C.c_int64), ("num_free", C.c_int64), ("num_dirichlet", C.c_int64),
        ("nnz_full", C.c_int64), ("nnz_upper", C.c_int64), ("solver_vec_len", C.c_int64),
        ("solver_entries", C.c_int64), ("solver_layout", C.c_int32),
    ]


class ErrorNorms(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("mean_norm", "l1_norm", "l2_norm", "linfty_norm", "h1_seminorm",
                                          "h1_norm", "w1infty_seminorm", "w1infty_norm", "energy_norm")]


class BddcParams(C.Structure):
    _fields_ = [
        ("nsub", C.c_int32 * 3),
        ("cuts", C.c_void_p),
        ("use_vertices", C.c_int32),
        ("use_edges", C.c_int32),
        ("use_faces", C.c_int32),
        ("weighting", C.c_int32),
        ("coarse_handler", C.c_int32),
        ("use_subparts", C.c_int32),
    ]


class BddcInfo(C.Structure):
    _fields_ = [
        ("num_subdomains", C.c_int32),
        ("max_local_dofs", C.c_int32),
        ("num_interface_dofs", C.c_int64),
        ("num_coarse_dofs", C.c_int64),
        ("symbolic_ms", C.c_double),
        ("numeric_ms", C.c_double),
        ("device_bytes", C.c_uint64),
        ("factor_flops", C.c_double),
        ("factor_ms", C.c_double),
        ("coarse_ms", C.c_double),
    ]


class BatchProblem(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("order", C.c_int32),
        ("coef", C.c_double),
        ("qp_source", C.c_void_p),
        ("x", C.c_void_p),
    ]


class BatchResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("iterations", C.c_int32),
        ("refinements", C.c_int32),
        ("team", C.c_int32),
        ("rel_residual", C.c_double),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("threads", C.c_int32), ("ctas", C.c_int32), ("max_team", C.c_int32), ("teams_gt1", C.c_int32),
        ("graph", C.c_int32),
        ("total_dofs", C.c_int64),
        ("predicted_balance", C.c_double),
        ("run_ms", C.c_double),
        ("autotune_ms", C.c_double),
        ("team_share", C.c_double),
    ]


class Request(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("n", C.c_int32 * 3),
        ("order", C.c_int),
        ("cell_coef", C.c_void_p),
        ("coef_const", C.c_double),
        ("nu", C.c_double),
        ("source_fn", C.c_int),
        ("fn_param", C.c_double * 8),
        ("dirichlet_ids", C.c_void_p),
        ("n_ids", C.c_int),
        ("solver", SolverParams),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("iterations", C.c_int),
        ("outer_iterations", C.c_int),
        ("num_free", C.c_int64),
        ("t_queue_ms", C.c_double),
        ("t_run_ms", C.c_double),
        ("t_total_ms", C.c_double),
        ("solve_ms", C.c_double),
        ("footprint_bytes", C.c_uint64),
    ]


class FGError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = f"{where}: {STATUS.get(status, status)}"
        try:
            err = lib().fg_last_error().decode()
            if err:
                msg += f" ({err})"
        except Exception:
            pass
        super().__init__(msg)


_lib = None


def lib():
    """Load libfempar_gpu.so; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m fempar_gb300.build` "
                          "(the GB300 path has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
    pp = C.POINTER(C.c_void_p)
    sig = {
        "fg_status_string": (C.c_char_p, [i32]),
        "fg_last_error": (C.c_char_p, []),
        "fg_version": (C.c_char_p, []),
        "fg_ctx_create": (i32, [i32, C.c_uint64, pp]),
        "fg_ctx_destroy": (i32, [vp]),
        "fg_ctx_memory": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "fg_ctx_get_stream": (i32, [vp, pp]),
        "fg_ctx_kernel_launches": (i32, [vp, C.POINTER(C.c_int64)]),
        "fg_mesh_create_structured": (i32, [vp, i32, vp, vp, vp, pp]),
        "fg_mesh_destroy": (i32, [vp]),
        "fg_partition_create": (i32, [vp, vp, pp]),
        "fg_partition_destroy": (i32, [vp]),
        "fg_partition_get_info": (i32, [vp, C.POINTER(PartitionInfo)]),
        "fg_partition_get_dof_import_sizes": (i32, [vp, i32, C.POINTER(DofImportSizes)]),
        "fg_partition_get_dof_import": (i32, [vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "fg_partition_assemble": (i32, [vp, vp, pp]),
        "fg_partition_comm_device": (i32, [vp, vp]),
        "fg_partition_solve": (i32, [vp, vp, vp, vp, vp]),
        "fg_mesh_create_unstructured": (i32, [vp, C.c_int64, vp, C.c_int64, vp, C.c_int64, vp, vp, vp, pp]),
        "fg_mesh_read_gid": (i32, [vp, C.c_char_p, C.c_char_p, pp]),
        "fg_mesh_get_info": (i32, [vp, C.POINTER(MeshInfo)]),
        "fg_mesh_get_vefs": (i32, [vp, vp, vp]),
        "fg_space_create": (i32, [vp, i32, i32, vp, i32, pp]),
        "fg_space_destroy": (i32, [vp]),
        "fg_space_create_dg": (i32, [vp, i32, pp]),
        "fg_space_release_pattern": (i32, [vp]),
        "fg_space_get_info": (i32, [vp, C.POINTER(SpaceInfo)]),
        "fg_space_get_dof_map": (i32, [vp, vp]),
        "fg_space_get_dirichlet_coords": (i32, [vp, vp]),
        "fg_space_get_qp_coords": (i32, [vp, vp, i32]),
        "fg_assemble": (i32, [vp, C.POINTER(Integrand), pp]),
        "fg_system_reassemble": (i32, [vp, C.POINTER(Integrand)]),
        "fg_system_destroy": (i32, [vp]),
        "fg_system_export_csr": (i32, [vp, i32, i32, vp, vp, vp]),
        "fg_system_export_rhs": (i32, [vp, vp]),
        "fg_system_export_dirichlet_values": (i32, [vp, vp]),
        "fg_system_spmv_device": (i32, [vp, i32, vp, vp]),
        "fg_dense_gemm_nt": (i32, [vp, C.c_int64, C.c_int64, C.c_int64, C.c_double, vp, C.c_int64, C.c_int64, vp,
                                   C.c_int64, C.c_int64, C.c_double, vp, C.c_int64, C.c_int64, i32]),
        "fg_system_spmv_solver_layout_device": (i32, [vp, i32, vp, vp, i32]),
        "fg_system_spmv_device_noalloc": (i32, [vp, i32, vp, vp]),
        "fg_solve": (i32, [vp, C.POINTER(SolverParams), vp, vp, vp, C.POINTER(SolveInfo)]),
        "fg_solve_device": (i32, [vp, C.POINTER(SolverParams), vp, vp, vp, C.POINTER(SolveInfo)]),
        "fg_solver_params_default": (None, [C.POINTER(SolverParams)]),
        "fg_request_footprint": (i32, [C.POINTER(Request), C.POINTER(C.c_uint64), C.POINTER(C.c_int64)]),
        "fg_server_create": (i32, [i32, C.c_uint64, i32, pp]),
        "fg_server_submit": (i32, [vp, C.POINTER(Request), C.POINTER(C.c_uint64)]),
        "fg_server_wait": (i32, [vp, C.c_uint64, i32, C.POINTER(Result)]),
        "fg_server_take_solution": (i32, [vp, C.c_uint64, vp]),
        "fg_server_stats": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_int64)]),
        "fg_server_destroy": (i32, [vp]),
        "fg_integrand_default": (None, [C.POINTER(Integrand)]),
        "fg_system_error_norms": (i32, [vp, vp, i32, i32, vp, vp, C.POINTER(ErrorNorms)]),
        "fg_bddc_params_default": (None, [C.POINTER(BddcParams)]),
        "fg_bddc_create": (i32, [vp, C.POINTER(BddcParams), pp]),
        "fg_bddc_numerical_setup": (i32, [vp]),
        "fg_bddc_get_info": (i32, [vp, C.POINTER(BddcInfo)]),
        "fg_bddc_apply_device": (i32, [vp, i32, vp, vp]),
        "fg_bddc_solve": (i32, [vp, C.POINTER(SolverParams), vp, vp, vp, C.POINTER(SolveInfo)]),
        "fg_bddc_solve_device": (i32, [vp, C.POINTER(SolverParams), vp, vp, vp, C.POINTER(SolveInfo)]),
        "fg_bddc_destroy": (i32, [vp]),
        "fg_batch_create": (i32, [vp, i32, C.POINTER(BatchProblem), i32, C.POINTER(SolverParams), i32, pp]),
        "fg_batch_run": (i32, [vp, C.POINTER(BatchResult)]),
        "fg_batch_get_info": (i32, [vp, C.POINTER(BatchInfo)]),
        "fg_batch_destroy": (i32, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status, where):
    if status != FG_OK:
        raise FGError(status, where)
    return status
