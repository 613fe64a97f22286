"""ctypes binding of libsimp_gb300.so (the C ABI of include/simp_gpu.h).

The library is built in-tree by :mod:`sparlab_gb300.build`.  There is no CPU
fallback: if the shared library is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

SIMP_OK = 0
SIMP_BAD_INPUT = 1
SIMP_BREAKDOWN = 2
SIMP_UNDERCONSTRAINED = 3
SIMP_MAXITER = 4
SIMP_NONFINITE = 5
SIMP_CUDA_ERROR = 6
PRECISION_FP64 = 0
PRECISION_MIXED = 1

EXPORTS = [
    "simp_default_options", "simp_ctx_create", "simp_ctx_destroy", "simp_last_error",
    "simp_set_layout", "simp_factorize", "simp_set_pattern", "simp_set_values",
    "simp_set_values_device", "simp_setup", "simp_solve", "simp_apply_preconditioner",
    "simp_stats", "simp_level_aggregates", "simp_level_matrix", "simp_level_prolongator",
    "simp_problem_create", "simp_problem_destroy", "simp_problem_last_error",
    "simp_problem_sizes", "simp_set_design", "simp_get_design", "simp_evaluate",
    "simp_oc_update", "simp_mma_update", "simp_iterate", "simp_problem_stats", "simp_filter_forward",
    "simp_filter_adjoint", "simp_problem_kff", "simp_element_stiffness",
    "simp_problem_apply_operator", "simp_problem_time_operator", "simp_filter_volume_noalloc",
    "simp_kernel_launches", "simp_default_modal_options", "simp_modal", "simp_modal_warning",
    "simp_element_mass", "simp_default_buckling_options", "simp_buckling", "simp_buckling_warning",
    "simp_projection_variants", "simp_surrogate_last_error", "simp_surrogate_create",
    "simp_surrogate_destroy", "simp_surrogate_num_params", "simp_surrogate_get_params",
    "simp_surrogate_set_params", "simp_surrogate_add_sample", "simp_surrogate_num_samples",
    "simp_surrogate_train", "simp_surrogate_predict", "simp_surrogate_forward",
    "simp_problem_set_surrogate", "simp_problem_learned_seconds", "simp_conv3d_bf16",
    "simp_surrogate_loss_gradient", "simp_autotune_enable", "simp_autotune_report",
    "simp_autotune_set", "simp_iterate_batch",
    "simp_conv3d_wgrad", "simp_problem_apply_level0",
]


class SolverOptions(C.Structure):
    _fields_ = [("strength_threshold", C.c_double), ("max_levels", C.c_int32),
                ("coarse_size", C.c_int32), ("smoother_degree", C.c_int32),
                ("chebyshev_ratio", C.c_double), ("prolongator_damping", C.c_double),
                ("lanczos_steps", C.c_int32), ("coarse_pivot_tolerance", C.c_double),
                ("reuse_aggregates", C.c_int32), ("iterative_tolerance", C.c_double),
                ("max_iterations", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32),
                ("cuda_graphs", C.c_int32), ("matrix_free_transfer", C.c_int32),
                ("matrix_free", C.c_int32), ("tensor_cores", C.c_int32)]


class AmgStats(C.Structure):
    _fields_ = [("num_levels", C.c_int32), ("reused_aggregates", C.c_int32),
                ("operator_complexity", C.c_double), ("grid_complexity", C.c_double),
                ("coarse_pivot_ratio", C.c_double), ("setup_seconds", C.c_double),
                ("storage_nonzeros", C.c_int64), ("level_rows", C.c_int64 * 16),
                ("level_nnz", C.c_int64 * 16), ("level_aggregates", C.c_int64 * 16),
                ("level_lambda", C.c_double * 16)]

    def as_dict(self):
        n = self.num_levels
        return {
            "num_levels": n, "reused_aggregates": bool(self.reused_aggregates),
            "operator_complexity": self.operator_complexity,
            "grid_complexity": self.grid_complexity,
            "coarse_pivot_ratio": self.coarse_pivot_ratio,
            "setup_seconds": self.setup_seconds, "storage_nonzeros": self.storage_nonzeros,
            "levels": [{"unknowns": self.level_rows[k], "nonzeros": self.level_nnz[k],
                        "aggregates": self.level_aggregates[k],
                        "lambda_max": self.level_lambda[k]} for k in range(n)],
        }


class ProblemDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("thickness", C.c_double), ("element_matrix", C.POINTER(C.c_double)),
                ("fixed", C.POINTER(C.c_uint8)), ("num_loads", C.c_int32),
                ("loads", C.POINTER(C.c_double)), ("weights", C.POINTER(C.c_double)),
                ("filter_radius", C.c_double), ("volume_fraction", C.c_double),
                ("initial_density", C.c_double), ("penalty", C.c_double),
                ("emin_ratio", C.c_double), ("move_limit", C.c_double), ("damping", C.c_double),
                ("warm_start", C.c_int32), ("block_pcg", C.c_int32), ("optimizer", C.c_int32),
                ("projection", C.c_int32), ("eta", C.c_double), ("beta_start", C.c_double),
                ("beta_max", C.c_double), ("beta_factor", C.c_double), ("beta_interval", C.c_int32),
                ("advance_on_convergence", C.c_int32), ("change_tolerance", C.c_double),
                ("robust", C.c_int32), ("robust_delta", C.c_double),
                ("robust_volume_interval", C.c_int32), ("warm_history", C.c_int32)]


class Evaluation(C.Structure):
    _fields_ = [("compliance", C.c_double), ("volume", C.c_double),
                ("volume_fraction", C.c_double), ("linear_iterations", C.c_int32),
                ("relres_max", C.c_double)]


class OcStep(C.Structure):
    _fields_ = [("lam", C.c_double), ("achieved_volume", C.c_double), ("max_change", C.c_double),
                ("bisections", C.c_int32), ("volume_converged", C.c_int32)]


class IterationRecord(C.Structure):
    _fields_ = [("compliance", C.c_double), ("volume_fraction", C.c_double),
                ("max_change", C.c_double), ("lam", C.c_double), ("gray_level", C.c_double),
                ("linear_iterations", C.c_int32), ("bisections", C.c_int32),
                ("seconds", C.c_double), ("volume_converged", C.c_int32), ("final_stage", C.c_int32),
                ("beta", C.c_double), ("eroded_volume_fraction", C.c_double),
                ("dilated_volume_fraction", C.c_double), ("dilated_target_fraction", C.c_double)]


class ModalOptions(C.Structure):
    _fields_ = [("num_modes", C.c_int32), ("mass_type", C.c_int32), ("max_iterations", C.c_int32),
                ("tolerance", C.c_double), ("shift_factor", C.c_double),
                ("rigid_body_ratio", C.c_double), ("residual_tolerance", C.c_double),
                ("warm_start", C.c_int32), ("density", C.c_double),
                ("element_mass", C.POINTER(C.c_double)), ("concurrent_solves", C.c_int32)]


class ModalInfo(C.Structure):
    _fields_ = [("num_modes", C.c_int32), ("iterations", C.c_int32), ("subspace_size", C.c_int32),
                ("converged", C.c_int32), ("linear_iterations", C.c_int64),
                ("final_change", C.c_double), ("total_mass", C.c_double),
                ("num_warnings", C.c_int32)]


class RobustRecord(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "eta_eroded", "eta_intermediate", "eta_dilated", "compliance_eroded",
        "compliance_intermediate", "compliance_dilated", "volume_fraction_eroded",
        "volume_fraction_intermediate", "volume_fraction_dilated", "dilated_target_fraction")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BucklingOptions(C.Structure):
    _fields_ = [("num_modes", C.c_int32), ("max_iterations", C.c_int32), ("tolerance", C.c_double),
                ("residual_tolerance", C.c_double), ("young", C.c_double), ("poisson", C.c_double),
                ("transform", C.c_int32), ("concurrent_solves", C.c_int32), ("shift_hint", C.c_double)]


class BucklingInfo(C.Structure):
    _fields_ = [("num_modes", C.c_int32), ("iterations", C.c_int32), ("subspace_size", C.c_int32),
                ("converged", C.c_int32), ("no_positive_load_factor", C.c_int32),
                ("subspace_cols", C.c_int32), ("linear_iterations", C.c_int64),
                ("final_change", C.c_double), ("num_warnings", C.c_int32), ("transformed", C.c_int32),
                ("sigma", C.c_double), ("factorizations", C.c_int32)]


_lock = threading.Lock()
_lib = None


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it first when its sources are newer)."""
    global _lib
    with _lock:
        if _lib is None:
            if build_if_missing and not _build.up_to_date():
                _build.build()
            if not os.path.exists(_build.LIB):
                raise RuntimeError("libsimp_gb300.so is not built; run sparlab_gb300.build.build()")
            lib = C.CDLL(_build.LIB)
            lib.simp_last_error.restype = C.c_char_p
            lib.simp_problem_last_error.restype = C.c_char_p
            lib.simp_kernel_launches.restype = C.c_int64
            lib.simp_modal_warning.restype = C.c_char_p
            lib.simp_buckling_warning.restype = C.c_char_p
            lib.simp_surrogate_last_error.restype = C.c_char_p
            _lib = lib
    return _lib


class SolverError(RuntimeError):
    """Bad input, breakdown, under-constrained or non-finite (sparlab::SolverError)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class ConvergenceError(SolverError):
    """Iteration budget spent (sparlab::ConvergenceError)."""


def raise_for(code: int, msg: str):
    if code == SIMP_OK:
        return
    if code == SIMP_MAXITER:
        raise ConvergenceError(code, msg)
    raise SolverError(code, msg)


def default_options(**kw) -> SolverOptions:
    o = SolverOptions()
    load().simp_default_options(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown solver option {k!r}")
        setattr(o, k, v)
    return o


def autotune_report():
    """The launch-shape tuner's choices: {key: (chosen variant, [ms per variant])}."""
    lib = load()
    need = C.c_int64()
    lib.simp_autotune_report(None, C.c_int64(0), C.byref(need))
    buf = C.create_string_buffer(max(1, need.value))
    lib.simp_autotune_report(buf, C.c_int64(len(buf)), C.byref(need))
    out = {}
    for line in buf.value.decode().splitlines():
        parts = line.split()
        if len(parts) >= 2:
            out[parts[0]] = (int(parts[1]), [float(v) for v in parts[2:]])
    return out


def ptr(a, ctype=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(ctype))
