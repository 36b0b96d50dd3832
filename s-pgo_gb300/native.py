"""ctypes binding of the C ABI declared in ``include/spgo.h``.

Loads the in-tree ``_build/libspgo.so``.  There is no fallback: if the library
is missing or fails to load, importing this module raises, so nothing can run
the solver on anything but the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libspgo.so")

SPGO_OK = 0
SPGO_ERR_INVALID_ARG, SPGO_ERR_UNSUPPORTED, SPGO_ERR_BUFFER_SMALL, SPGO_ERR_CUDA, SPGO_ERR_NOT_SPD = -1, -2, -3, -4, -5
PREC_MIXED, PREC_FP64 = 0, 1
LOSS_L2, LOSS_CAUCHY, LOSS_HUBER = 0, 1, 2
STATUS_RUNNING, STATUS_CONVERGED, STATUS_MAX_ITERS, STATUS_STALLED = 0, 1, 2, 3
MAX_WINDOW = 96

# symbols include/spgo.h declares (checked by the tests)
EXPORTED = [
    "spgo_version", "spgo_last_error", "spgo_default_params", "spgo_plan_create", "spgo_plan_create_opts",
    "spgo_plan_sizes_get",
    "spgo_plan_destroy", "spgo_plan_offsets", "spgo_solver_create", "spgo_solver_destroy", "spgo_set_params",
    "spgo_gn_step", "spgo_lm_reset", "spgo_lm_iterate", "spgo_lm_status", "spgo_lm_solve",
    "spgo_export_system", "spgo_launch_count", "spgo_profile_enable", "spgo_profile_read",
    "spgo_cost_noalloc", "spgo_export_reduced", "spgo_mlp_forward", "spgo_mlp_grad", "spgo_mlp_adam",
    "spgo_lm_set_controller", "spgo_lm_features", "spgo_lm_probe", "spgo_autotune", "spgo_lm_trace",
]
TRACE_MAX = 128
MLP_PARAMS, MLP_INPUTS, MLP_CACHE_PER_SAMPLE = 5378, 16, 386
PROFILE_KINDS = ["chain", "linearize", "cost", "pair_reduce", "schur", "assemble", "factor_solve", "backsub",
                 "update", "bookkeeping", "refine", "resid_pass"]


class HostProblem(C.Structure):
    """``spgo_host_problem``; the array fields are addresses (``ndarray.ctypes.data``):
    intrinsics float32[8], T_r_to_l float64[16], host int32[L], anchor_uv float32[2L],
    obs_ptr int64[L+1], obs_frame int32[O], obs_uv float32[4O], and the optional
    FP64 pixel arrays anchor_uv_f64 float64[2L], obs_uv_f64 float64[4O]."""
    _fields_ = [("n_poses", C.c_int32), ("n_landmarks", C.c_int32), ("n_obs", C.c_int64),
                ("intrinsics", C.c_void_p), ("T_r_to_l", C.c_void_p),
                ("host", C.c_void_p), ("anchor_uv", C.c_void_p),
                ("obs_ptr", C.c_void_p), ("obs_frame", C.c_void_p),
                ("obs_uv", C.c_void_p), ("anchor_uv_f64", C.c_void_p), ("obs_uv_f64", C.c_void_p)]


class PlanSizes(C.Structure):
    _fields_ = [("n_problems", C.c_int32), ("total_poses", C.c_int32), ("total_landmarks", C.c_int32),
                ("total_obs", C.c_int64), ("n_chunks", C.c_int32), ("n_schur_items", C.c_int32),
                ("max_params", C.c_int32), ("schur_chunk_tiles", C.c_int32), ("static_bytes", C.c_size_t),
                ("workspace_bytes", C.c_size_t), ("slab_elems", C.c_int64), ("pair_records", C.c_int64),
                ("schur_flops", C.c_int64), ("n_tc_items", C.c_int32), ("tc_chunk_tiles", C.c_int32),
                ("schur_flops_landmark", C.c_int64), ("tc_split", C.c_int32), ("simt_split", C.c_int32)]


class PlanOptions(C.Structure):
    """``spgo_plan_options``: Schur work shapes chosen when the batch is planned."""
    _fields_ = [("tc_split", C.c_int32), ("simt_split", C.c_int32), ("reserved", C.c_int32 * 6)]


class Params(C.Structure):
    _fields_ = [("loss", C.c_int32), ("near_boost", C.c_int32), ("loss_scale", C.c_float), ("eps", C.c_float),
                ("alpha_min", C.c_float), ("alpha_max", C.c_float), ("lambda0", C.c_double),
                ("lambda_max", C.c_double), ("tol", C.c_double), ("max_iters", C.c_int32),
                ("refine_steps", C.c_int32), ("use_graph", C.c_int32), ("use_tc", C.c_int32),
                ("cost_block", C.c_int32), ("lin_block", C.c_int32), ("outer_steps", C.c_int32),
                ("wait_us", C.c_int32), ("ctl_min_log10", C.c_float), ("outer_tol", C.c_float),
                ("stop_rho", C.c_float)]


class ProblemStatus(C.Structure):
    _fields_ = [("cost0", C.c_double), ("cost", C.c_double), ("lambda_", C.c_double), ("iterations", C.c_int32),
                ("accepted", C.c_int32), ("status", C.c_int32), ("factor_failures", C.c_int32),
                ("wait_timeouts", C.c_int32), ("pad", C.c_int32)]


class DeviceProblem(C.Structure):
    """spgo_device_problem: HostProblem's fields, device pointers."""
    _fields_ = [(n, t) for n, t in HostProblem._fields_ if not n.endswith("_f64")]


class SpgoError(RuntimeError):
    pass


_lib = None


def lib() -> C.CDLL:
    """Load (once) and return the CUDA library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SpgoError(f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
    L.spgo_version.restype = C.c_int
    L.spgo_last_error.restype = C.c_char_p
    L.spgo_default_params.argtypes = [C.POINTER(Params)]
    L.spgo_default_params.restype = None
    L.spgo_plan_create.argtypes = [C.POINTER(HostProblem), i32, i32, C.POINTER(vp)]
    L.spgo_plan_create_opts.argtypes = [C.POINTER(HostProblem), i32, i32, C.POINTER(PlanOptions), C.POINTER(vp)]
    L.spgo_plan_sizes_get.argtypes = [vp, C.POINTER(PlanSizes)]
    L.spgo_plan_destroy.argtypes = [vp]
    L.spgo_plan_offsets.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.spgo_solver_create.argtypes = [vp, vp, sz, vp, sz, vp, vp, vp, C.POINTER(vp)]
    L.spgo_solver_destroy.argtypes = [vp]
    L.spgo_set_params.argtypes = [vp, C.POINTER(Params)]
    L.spgo_gn_step.argtypes = [vp, i32, C.c_float, vp]
    L.spgo_lm_reset.argtypes = [vp, vp]
    L.spgo_lm_iterate.argtypes = [vp, i32, vp]
    L.spgo_lm_status.argtypes = [vp, C.POINTER(ProblemStatus), vp]
    L.spgo_lm_solve.argtypes = [vp, i32, C.POINTER(C.c_int32), vp]
    L.spgo_export_system.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, vp]
    L.spgo_mlp_forward.argtypes = [vp, vp, i32, vp, vp, vp]
    L.spgo_mlp_grad.argtypes = [vp, vp, vp, i32, vp, vp, vp, vp, vp]
    L.spgo_mlp_adam.argtypes = [vp, vp, vp, vp, i32, C.c_float, vp]
    L.spgo_lm_set_controller.argtypes = [vp, vp, vp]
    L.spgo_lm_features.argtypes = [vp, vp, vp]
    L.spgo_lm_probe.argtypes = [vp, i32, C.POINTER(C.c_double), C.POINTER(C.c_double), vp]
    L.spgo_lm_trace.argtypes = [vp, i32, vp, vp, vp, vp, vp]
    L.spgo_lm_trace.restype = C.c_int
    L.spgo_autotune.argtypes = [vp, C.POINTER(Params), vp]
    L.spgo_autotune.restype = C.c_int
    for name in ("spgo_mlp_forward", "spgo_mlp_grad", "spgo_mlp_adam", "spgo_lm_set_controller",
                 "spgo_lm_features", "spgo_lm_probe"):
        getattr(L, name).restype = C.c_int
    L.spgo_export_reduced.argtypes = [vp, i32, C.c_double, vp, vp, vp]
    L.spgo_export_reduced.restype = C.c_int
    L.spgo_profile_enable.argtypes = [vp, i32]
    L.spgo_profile_read.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int64), i32, vp]
    L.spgo_cost_noalloc.argtypes = [C.POINTER(DeviceProblem), vp, vp, C.POINTER(Params), vp, vp]
    L.spgo_cost_noalloc.restype = C.c_int
    L.spgo_launch_count.argtypes = [vp]
    L.spgo_launch_count.restype = i64
    for name in ("spgo_plan_create", "spgo_plan_create_opts", "spgo_plan_sizes_get", "spgo_plan_destroy",
                 "spgo_plan_offsets",
                 "spgo_solver_create", "spgo_solver_destroy", "spgo_set_params", "spgo_gn_step", "spgo_lm_reset",
                 "spgo_lm_iterate", "spgo_lm_status", "spgo_lm_solve", "spgo_export_system", "spgo_profile_enable",
                 "spgo_profile_read"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(rc: int, what: str = "") -> None:
    if rc != SPGO_OK:
        msg = lib().spgo_last_error().decode(errors="replace")
        raise SpgoError(f"{what} failed ({rc}): {msg}")


def default_params() -> Params:
    p = Params()
    lib().spgo_default_params(C.byref(p))
    return p
