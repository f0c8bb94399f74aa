"""ctypes binding of the C ABI declared in include/feng_cuda.h.

The shared library is the in-tree ``feng_gb300/_feng_cuda.so`` built by
``feng_gb300.build``.  Loading fails loudly when it is missing: there is no
CPU fallback for the backend.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_feng_cuda.so"

OK = 0
STATUS_NAMES = {
    0: "OK", -1: "ERROR", -2: "READ_ERROR", -3: "INVALID_ARG", -4: "DEVICE_FAIL",
    -5: "NOT_CONVERGED", -6: "PC_FAILED", -7: "NONFINITE", -8: "BAD_COLORING",
}


class FeError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class FormDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("coeff", C.c_double), ("coeff2", C.c_double),
                ("source", C.c_int32), ("params", C.c_double * 4)]


class SpaceDesc(C.Structure):
    _fields_ = [("field", C.c_int32), ("degree", C.c_int32), ("ncomp", C.c_int32),
                ("cnc", C.c_int32), ("essential", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("krylov", C.c_int32), ("restart", C.c_int32), ("max_iter", C.c_int32),
                ("rel_tol", C.c_double), ("abs_tol", C.c_double), ("div_tol", C.c_double),
                ("precond", C.c_int32), ("pc_block_rows", C.c_int32), ("precision", C.c_int32),
                ("quad_degree", C.c_int32), ("mg_inner", C.c_int32), ("mg_smooth", C.c_int32),
                ("gs_passes", C.c_int32)]


class NewtonOptions(C.Structure):
    _fields_ = [("tol_residual", C.c_double), ("tol_correction", C.c_double),
                ("tol_divergence", C.c_double), ("max_iter", C.c_int32),
                ("recompute_every", C.c_int32), ("residual_decrease", C.c_double),
                ("stationary", C.c_int32), ("rel_residual", C.c_double),
                ("linear_rtol_min", C.c_double), ("residual_scale", C.c_double)]


class TransientOptions(C.Structure):
    _fields_ = [("dt", C.c_double), ("t0", C.c_double), ("guess", C.c_int32), ("train_from", C.c_int32),
                ("use_from", C.c_int32), ("train_iters", C.c_int32), ("batch", C.c_int64),
                ("lr", C.c_double), ("seed", C.c_uint64)]


class StepStats(C.Structure):
    _fields_ = [("step", C.c_int32), ("newton_iterations", C.c_int32), ("krylov_iterations", C.c_int32),
                ("status", C.c_int32), ("guess_used", C.c_int32), ("t", C.c_double),
                ("residual_ref", C.c_double), ("residual_guess", C.c_double),
                ("residual_extrap", C.c_double), ("residual", C.c_double), ("step_ms", C.c_double),
                ("guess_ms", C.c_double), ("train_ms", C.c_double), ("train_loss", C.c_double),
                ("guess_scale", C.c_double)]


class NewtonStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("krylov_iterations", C.c_int32),
                ("matrix_assemblies", C.c_int32), ("status", C.c_int32),
                ("residual0", C.c_double), ("residual", C.c_double), ("correction", C.c_double),
                ("residual_ms", C.c_double), ("matrix_ms", C.c_double),
                ("factor_ms", C.c_double), ("solve_ms", C.c_double)]


P = C.c_void_p
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

# name -> (restype, argtypes); pointer arguments that may be NULL use c_void_p.
SIGNATURES = {
    "fe_cuda_last_error": (C.c_char_p, []),
    "fe_cuda_version": (C.c_int, []),
    "fe_cuda_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "fe_mesh_generate_square": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_uint64, C.POINTER(P)]),
    "fe_mesh_read_msh": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "fe_export_vtk": (C.c_int, [P, P, P, C.POINTER(C.c_char_p), C.c_int, C.POINTER(C.c_char_p), C.c_int,
                                C.c_int, C.c_char_p]),
    "fe_tet_quadrature_rule": (C.c_int, [C.c_int, C.POINTER(C.c_int), P, P, P, P]),
    "fe_setup3d_create": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.POINTER(P)]),
    "fe_setup_get_dof_z": (C.c_int, [P, P]),
    "fe_mesh3d_generate_cube": (C.c_int, [C.c_int, P, C.c_double, C.c_uint64, C.POINTER(P)]),
    "fe_mesh3d_write_msh": (C.c_int, [P, C.c_char_p]),
    "fe_mesh3d_read_msh": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "fe_mesh3d_from_arrays": (C.c_int, [C.c_int64, P, P, P, C.c_int64, P, C.c_int64, P, C.POINTER(P)]),
    "fe_mesh3d_sizes": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "fe_mesh3d_arrays": (C.c_int, [P, P, P, P, P, P]),
    "fe_mesh3d_destroy": (None, [P]),
    "fe_export_vtk3d": (C.c_int, [P, P, P, C.POINTER(C.c_char_p), C.c_int, C.POINTER(C.c_char_p), C.c_int,
                                  C.c_int, C.c_char_p]),
    "fe_mesh_read_msh_groups": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_int,
                                          C.c_char_p, C.POINTER(P)]),
    "fe_mesh_write_msh": (C.c_int, [P, C.c_char_p]),
    "fe_mesh_from_arrays": (C.c_int, [C.c_int64, P, P, C.c_int64, P, C.c_int64, P, C.c_int32, C.POINTER(P)]),
    "fe_mesh_sizes": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "fe_mesh_arrays": (C.c_int, [P, P, P, P, P, P, P]),
    "fe_mesh_destroy": (None, [P]),
    "fe_setup_create": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(P)]),
    "fe_setup_destroy": (None, [P]),
    "fe_setup_sizes": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int64), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "fe_setup_get_pattern": (C.c_int, [P, P, P]),
    "fe_setup_get_coloring": (C.c_int, [P, P, P]),
    "fe_setup_get_element_dofs": (C.c_int, [P, P]),
    "fe_setup_get_dof_info": (C.c_int, [P, P, P, P, P, P]),
    "fe_setup_get_blocks": (C.c_int, [P, P]),
    "fe_quadrature_rule": (C.c_int, [C.c_int, C.POINTER(C.c_int), P, P, P]),
    "fe_cuda_system_create": (C.c_int, [P, P, C.c_int, P, C.POINTER(P)]),
    "fe_cuda_system_create_from_tables": (C.c_int, [C.c_int, C.c_int64, P, P, C.c_int64, C.c_int64,
                                                    C.c_int, P, P, P, P, P, P, C.c_int, P,
                                                    C.POINTER(P)]),
    "fe_cuda_system_destroy": (None, [P]),
    "fe_cuda_system_sizes": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int)]),
    "fe_cuda_get_pattern": (C.c_int, [P, P, P]),
    "fe_cuda_get_coloring": (C.c_int, [P, P, P]),
    "fe_cuda_validate_coloring": (C.c_int, [P]),
    "fe_cuda_set_solution": (C.c_int, [P, P, P]),
    "fe_cuda_get_solution": (C.c_int, [P, P]),
    "fe_cuda_set_time": (C.c_int, [P, C.c_double, C.c_double]),
    "fe_cuda_norm_points": (C.c_int, [P, P, P, P]),
    "fe_cuda_l2_error": (C.c_int, [P, C.c_int, P, P]),
    "fe_cuda_set_bdf": (C.c_int, [P, C.c_int, P, P, P]),
    "fe_cuda_compute_soldot": (C.c_int, [P]),
    "fe_cuda_set_to_zero": (C.c_int, [P]),
    "fe_cuda_set_matrix_to_zero": (C.c_int, [P]),
    "fe_cuda_set_residual_to_zero": (C.c_int, [P]),
    "fe_cuda_assemble_residuals": (C.c_int, [P]),
    "fe_cuda_assemble_matrices": (C.c_int, [P]),
    "fe_cuda_get_rhs_max_norm": (C.c_int, [P, C.POINTER(C.c_double)]),
    "fe_cuda_set_tolerances": (C.c_int, [P, C.c_double, C.c_double, C.c_int]),
    "fe_cuda_solve": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "fe_cuda_correct_solution": (C.c_int, [P]),
    "fe_cuda_get_matrix": (C.c_int, [P, P]),
    "fe_cuda_get_rhs": (C.c_int, [P, P]),
    "fe_cuda_get_du": (C.c_int, [P, P]),
    "fe_cuda_get_du_max_norm": (C.c_int, [P, C.POINTER(C.c_double)]),
    "fe_cuda_jacobian_route": (C.c_int, [P, C.POINTER(C.c_int)]),
    "fe_setup_set_pattern_mode": (C.c_int, [C.c_int]),
    "fe_setup_pattern_on_device": (C.c_int, [P, C.POINTER(C.c_int)]),
    "fe_cuda_newton": (C.c_int, [P, C.POINTER(NewtonOptions), C.POINTER(NewtonStats)]),
    "fe_cuda_get_times": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fe_cuda_reset_times": (C.c_int, [P]),
    "fe_cuda_synchronize": (C.c_int, [P]),
    "fe_cuda_bench_phase": (C.c_int, [P, C.c_int, C.c_int, C.c_int64, C.POINTER(C.c_double)]),
    "fe_cuda_launch_count": (C.c_int, [C.POINTER(C.c_int64)]),
    "fe_cuda_smoother_bytes": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "fe_cuda_phase_bytes": (C.c_int, [P, C.c_int, C.POINTER(C.c_int64)]),
    "fe_cuda_save_solution": (C.c_int, [P]),
    "fe_cuda_restore_solution": (C.c_int, [P]),
    "fe_cuda_event_record": (C.c_int, [P, C.c_int]),
    "fe_cuda_event_elapsed": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "fe_cuda_set_device": (C.c_int, [C.c_int]),
    "fe_cuda_max_norm_noalloc": (C.c_int, [P, C.c_int64, P, C.POINTER(C.c_double)]),
    "fe_cuda_set_constrained_rows": (C.c_int, [P, P, C.c_int64]),
    "fe_cuda_constrain_essential_components": (C.c_int, [P]),
    "fe_cuda_set_periodic_pairs": (C.c_int, [P, P, P, C.c_int64]),
    "fe_cuda_apply_periodicity": (C.c_int, [P]),
    "fe_cuda_transient_create": (C.c_int, [P, C.POINTER(TransientOptions), C.POINTER(NewtonOptions),
                                           C.POINTER(P)]),
    "fe_cuda_transient_steps": (C.c_int, [P, C.c_int, P]),
    "fe_cuda_apply_preconditioner": (C.c_int, [P, P, P]),
    "fe_setup_set_quadrature": (C.c_int, [P, C.c_int, P]),
    "fe_cuda_system_create_from_tables_rule": (C.c_int, [C.c_int, C.c_int64, P, P, C.c_int64, C.c_int64, C.c_int, P, P,
                                                          P, P, P, P, C.c_int, P, C.c_int, P, P]),
    "fe_cuda_transient_get_network": (C.c_int, [P, P]),
    "fe_cuda_transient_set_network": (C.c_int, [P, P]),
    "fe_cuda_transient_destroy": (None, [P]),
    "fe_mlp_sizes": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                               C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
    "fe_mlp_create": (C.c_int, [C.c_uint64, C.c_int64, C.POINTER(P)]),
    "fe_mlp_destroy": (None, [P]),
    "fe_mlp_set_params": (C.c_int, [P, P]),
    "fe_mlp_get_params": (C.c_int, [P, P]),
    "fe_mlp_forward": (C.c_int, [P, P, C.c_int64, P]),
    "fe_mlp_train_step": (C.c_int, [P, P, P, P, C.c_int64, C.c_double, P, C.POINTER(C.c_double)]),
}

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads the backend library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"CUDA backend library {p} is missing: run feng_gb300.build.build() "
            "(there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> int:
    if status != OK:
        msg = load().fe_cuda_last_error()
        raise FeError(status, msg.decode() if msg else "")
    return status


def ptr(a: np.ndarray | None):
    """Raw pointer of a C-contiguous array (or NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)
