"""ctypes declarations of the solver entry points of include/m3d_gb300.h."""
from __future__ import annotations

import ctypes as C

from ._abi import Leaves, _fn, c_double_p, c_int_p


class Params(C.Structure):
    """struct m3d_params."""
    _fields_ = [
        ("bicgstab_tol", C.c_double),
        ("bicgstab_maxiter", C.c_int),
        ("scattered_field", C.c_int),
        ("air_z_threshold", C.c_double),
        ("div_correction", C.c_int),
        ("div_corr_iters", C.c_int),
        ("div_corr_tol", C.c_double),
        ("divcorr_outer_max", C.c_int),
        ("divcorr_iter_per_dc", C.c_int),
        ("sigma_bg", C.c_double),
        ("precision", C.c_int),
        ("true_residual_check", C.c_int),
        ("max_refinements", C.c_int),
        ("print_level", C.c_int),
        ("forward_interleaved", C.c_int),
        ("row_kernels", C.c_int),
        ("divcorr_precond", C.c_int),
        ("ssor_form", C.c_int),
        ("gradcorr", C.c_int),
        ("gradcorr_fmax", C.c_double),
        ("gradcorr_presmooth", C.c_int),
        ("divcorr_mixed", C.c_int),
        ("inner_tol_floor", C.c_double),
        ("residual_replacement", C.c_int),
        ("gradcorr_overlap", C.c_int),
        ("krylov", C.c_int),
        ("fgmres_m", C.c_int),
        ("learned_period", C.c_int),
        ("sweep_rows", C.c_int),
        ("coop_sweep", C.c_int),
        ("cuda_graphs", C.c_int),
        ("ssor_relax", C.c_double),
    ]


class Stats(C.Structure):
    """struct m3d_stats."""
    _fields_ = [
        ("n_rhs", C.c_int),
        ("iterations", C.c_int * 64),
        ("status", C.c_int * 64),
        ("true_residual", C.c_double * 64),
        ("total_iterations", C.c_int),
        ("refinements", C.c_int),
        ("seconds", C.c_double),
        ("kernel_launches", C.c_longlong),
        ("divcorr_calls", C.c_int),
        ("divcorr_outer", C.c_int),
        ("divcorr_cg_iterations", C.c_longlong),
        ("forward_iterations", C.c_longlong),
        ("adjoint_iterations", C.c_longlong),
        ("divcorr_cg_sweeps", C.c_longlong),
        ("divcorr_setup_ms", C.c_double),
        ("replacements", C.c_int),
        ("graphs_failed", C.c_int),
        ("graph_replays", C.c_longlong),
    ]


class KernelTimes(C.Structure):
    """struct m3d_kernel_times."""
    _fields_ = [
        ("launches", C.c_longlong * 6),
        ("ms", C.c_double * 6),
        ("bytes", C.c_double * 6),
        ("launches_k", (C.c_longlong * 5) * 6),
        ("ms_k", (C.c_double * 5) * 6),
        ("bytes_k", (C.c_double * 5) * 6),
    ]


class TuneEntry(C.Structure):
    """struct m3d_tune_entry."""
    _fields_ = [("row_kernels", C.c_int), ("K", C.c_int), ("ms_per_iter", C.c_double),
                ("ms_per_rhs_iter", C.c_double)]


class RegParams(C.Structure):
    """struct m3d_reg_params."""
    _fields_ = [
        ("alpha_s", C.c_double), ("alpha_x", C.c_double), ("alpha_y", C.c_double), ("alpha_z", C.c_double),
        ("n_smooth", C.c_int),
    ]


KERNEL_CLASSES = ("spmv", "ssor", "vector", "divcorr", "gradcorr", "sensitivity")

SOLVER_SYMBOLS = [
    "m3d_params_default", "m3d_solver_create", "m3d_solver_destroy", "m3d_last_error",
    "m3d_solver_setup", "m3d_solver_sizes", "m3d_set_sigma", "m3d_set_stations",
    "m3d_set_tolerance_override", "m3d_current_omega", "m3d_compute_single_frequency",
    "m3d_factorize_frequency", "m3d_release_factorization", "m3d_background_E",
    "m3d_set_background_fields", "m3d_build_adjoint_rhs", "m3d_adjoint_solve", "m3d_solve_rhs",
    "m3d_compute_sensitivity", "m3d_build_perturbation_rhs", "m3d_extract_delta_impedance",
    "m3d_forward_batch", "m3d_gradient_batch", "m3d_jtjv_batch", "m3d_solve_rhs_batch", "m3d_station_gradients",
    "m3d_group_station_gradients", "m3d_reg_setup", "m3d_reg_num_active", "m3d_reg_active_to_global",
    "m3d_reg_apply_wtw", "m3d_reg_apply_cmcmt", "m3d_reg_diagonal_wtw", "m3d_reg_evaluate", "m3d_dot_batched", "m3d_dot_batched_noalloc", "m3d_get_stats",
    "m3d_timer_start", "m3d_timer_stop", "m3d_set_kernel_timing", "m3d_get_kernel_times",
    "m3d_test_set_consume_no_wait", "m3d_autotune",
    "m3d_cnn_create", "m3d_cnn_destroy", "m3d_cnn_last_error", "m3d_cnn_get_weights", "m3d_cnn_set_weights",
    "m3d_cnn_forward", "m3d_cnn_backward", "m3d_cnn_train_step",
    "m3d_learn_setup", "m3d_learn_collect", "m3d_learn_train", "m3d_set_krylov",
]


def declare(lib) -> None:
    vp = C.c_void_p
    _fn(lib, "m3d_params_default", None, [C.POINTER(Params)])
    _fn(lib, "m3d_solver_create", C.c_int, [C.c_int, C.POINTER(vp)])
    _fn(lib, "m3d_solver_destroy", None, [vp])
    _fn(lib, "m3d_last_error", C.c_char_p, [vp])
    _fn(lib, "m3d_solver_setup", C.c_int, [vp, C.POINTER(Leaves), C.POINTER(Params)])
    _fn(lib, "m3d_solver_sizes", C.c_int, [vp, c_int_p, c_int_p, c_int_p, c_int_p])
    _fn(lib, "m3d_set_sigma", C.c_int, [vp, c_double_p, C.c_int])
    _fn(lib, "m3d_set_stations", C.c_int, [vp, c_double_p, C.c_int])
    _fn(lib, "m3d_set_tolerance_override", C.c_int, [vp, C.c_double])
    _fn(lib, "m3d_current_omega", C.c_int, [vp, c_double_p])
    _fn(lib, "m3d_compute_single_frequency", C.c_int, [vp, C.c_double, c_double_p])
    _fn(lib, "m3d_factorize_frequency", C.c_int, [vp, C.c_double])
    _fn(lib, "m3d_release_factorization", C.c_int, [vp])
    _fn(lib, "m3d_background_E", C.c_int, [vp, C.c_int, c_double_p])
    _fn(lib, "m3d_set_background_fields", C.c_int, [vp, c_double_p, c_double_p])
    _fn(lib, "m3d_build_adjoint_rhs", C.c_int, [vp, c_double_p, c_double_p, c_double_p])
    _fn(lib, "m3d_adjoint_solve", C.c_int, [vp, c_double_p, c_double_p])
    _fn(lib, "m3d_solve_rhs", C.c_int, [vp, c_double_p, c_double_p])
    _fn(lib, "m3d_solve_rhs_batch", C.c_int, [vp, c_double_p, C.c_int, c_double_p])
    _fn(lib, "m3d_station_gradients", C.c_int, [vp, c_double_p, C.c_int, c_double_p])
    _fn(lib, "m3d_group_station_gradients", C.c_int,
        [C.POINTER(vp), C.c_int, c_double_p, C.POINTER(c_double_p), C.POINTER(C.c_int),
         C.POINTER(c_double_p), C.POINTER(c_double_p), C.c_int, C.POINTER(C.c_int)])
    _fn(lib, "m3d_compute_sensitivity", C.c_int, [vp, c_double_p, c_double_p, c_double_p])
    _fn(lib, "m3d_build_perturbation_rhs", C.c_int, [vp, C.c_int, c_double_p, c_double_p])
    _fn(lib, "m3d_extract_delta_impedance", C.c_int, [vp, c_double_p, C.c_int, c_double_p])
    _fn(lib, "m3d_forward_batch", C.c_int, [vp, c_double_p, C.c_int, c_double_p, c_double_p])
    _fn(lib, "m3d_gradient_batch", C.c_int,
        [vp, c_double_p, C.c_int, c_double_p, c_double_p, c_double_p, c_double_p])
    _fn(lib, "m3d_jtjv_batch", C.c_int, [vp, c_double_p, C.c_int, c_double_p, c_double_p, C.c_double, c_double_p])
    _fn(lib, "m3d_reg_setup", C.c_int, [vp, C.POINTER(RegParams)])
    _fn(lib, "m3d_reg_num_active", C.c_int, [vp, c_int_p])
    _fn(lib, "m3d_reg_active_to_global", C.c_int, [vp, c_int_p])
    _fn(lib, "m3d_reg_apply_wtw", C.c_int, [vp, c_double_p, c_double_p])
    _fn(lib, "m3d_reg_apply_cmcmt", C.c_int, [vp, c_double_p, c_double_p])
    _fn(lib, "m3d_reg_diagonal_wtw", C.c_int, [vp, c_double_p])
    _fn(lib, "m3d_reg_evaluate", C.c_int, [vp, c_double_p, c_double_p, c_double_p, c_double_p])
    _fn(lib, "m3d_dot_batched", C.c_int, [vp, vp, vp, C.c_longlong, C.c_int, vp])
    _fn(lib, "m3d_dot_batched_noalloc", C.c_int, [vp, vp, C.c_longlong, C.c_int, vp, vp])
    _fn(lib, "m3d_get_stats", C.c_int, [vp, C.POINTER(Stats)])
    _fn(lib, "m3d_timer_start", C.c_int, [vp])
    _fn(lib, "m3d_timer_stop", C.c_int, [vp, c_double_p])
    _fn(lib, "m3d_set_kernel_timing", C.c_int, [vp, C.c_int])
    _fn(lib, "m3d_get_kernel_times", C.c_int, [vp, C.POINTER(KernelTimes)])
    _fn(lib, "m3d_test_set_consume_no_wait", C.c_int, [vp, C.c_int])
    fp = C.POINTER(C.c_float)
    _fn(lib, "m3d_cnn_create", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint, C.POINTER(vp)])
    _fn(lib, "m3d_cnn_destroy", None, [vp])
    _fn(lib, "m3d_cnn_last_error", C.c_char_p, [vp])
    _fn(lib, "m3d_cnn_get_weights", C.c_int, [vp, fp, fp])
    _fn(lib, "m3d_cnn_set_weights", C.c_int, [vp, fp, fp])
    _fn(lib, "m3d_cnn_forward", C.c_int, [vp, fp, C.c_int, C.c_int, C.c_int, C.c_int, fp])
    _fn(lib, "m3d_cnn_backward", C.c_int, [vp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp, fp])
    _fn(lib, "m3d_cnn_train_step", C.c_int, [vp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                             C.POINTER(C.c_double)])
    _fn(lib, "m3d_set_krylov", C.c_int, [vp, C.c_int, C.c_int, C.c_int])
    _fn(lib, "m3d_learn_setup", C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_uint, C.c_longlong])
    _fn(lib, "m3d_learn_collect", C.c_int, [vp, c_double_p, C.c_int, C.POINTER(C.c_longlong)])
    _fn(lib, "m3d_learn_train", C.c_int, [vp, C.c_int, C.c_float, C.c_int, C.c_uint, C.c_double, c_double_p,
                                          c_double_p])
    _fn(lib, "m3d_autotune", C.c_int, [vp, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(TuneEntry), c_int_p,
                                       c_int_p, c_int_p, c_int_p])
