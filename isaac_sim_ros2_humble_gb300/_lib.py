"""ctypes binding of libgbmp.so (the C-ABI declared in include/gbmp.h).

The shared library is required: if it is missing or fails to load, every call
raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgbmp.so")

OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "CUDA error",
          4: "code generation failed", 5: "capacity exceeded", 6: "timed out", 7: "not solved",
          8: "unsupported"}
CHECK_VERDICT, CHECK_COST = 0, 1
STEP_L2, STEP_LINF, STEP_COUNT = 0, 1, 2
BALANCE_DEFAULT, BALANCE_SIZE, BALANCE_SWAP, BALANCE_NONE = 0, 1, 2, 3
ROBOT_GENERIC, ROBOT_CODEGEN = 0, 1


class Projection(C.Structure):
    _fields_ = [("task_link", C.c_int32), ("offset", C.c_float * 16), ("reference", C.c_float * 6),
                ("tolerance", C.c_float * 6), ("use_boundary", C.c_int32), ("iterations", C.c_int32)]


class CheckRequest(C.Structure):
    _fields_ = [("robot", C.c_void_p), ("env", C.c_void_p), ("d_q", C.c_void_p), ("n", C.c_int64),
                ("d_verdict", C.c_void_p), ("d_costs", C.c_void_p), ("d_total", C.c_void_p),
                ("d_poses", C.c_void_p), ("d_centers", C.c_void_p)]


class GbmpError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"gbmp status {status} ({STATUS.get(status, '?')}): {message}")
        self.status = status


class RobotDesc(C.Structure):
    _fields_ = [("num_links", C.c_int32), ("joint_types", C.c_void_p), ("joint_poses", C.c_void_p),
                ("joint_axes", C.c_void_p), ("parent", C.c_void_p), ("num_spheres", C.c_int32),
                ("sphere_link", C.c_void_p), ("sphere_pos", C.c_void_p), ("sphere_radius", C.c_void_p),
                ("active_joints", C.c_void_p), ("lower", C.c_void_p), ("upper", C.c_void_p),
                ("default_values", C.c_void_p), ("self_enables", C.c_void_p), ("resolution", C.c_float)]


class RrtcSettings(C.Structure):
    _fields_ = [("lanes", C.c_int32), ("max_iters", C.c_int32), ("range", C.c_float), ("resolution", C.c_float),
                ("step_rule", C.c_int32), ("seed", C.c_uint64), ("time_limit_s", C.c_double),
                ("dynamic_domain", C.c_int32), ("dd_alpha", C.c_float), ("dd_radius", C.c_float),
                ("dd_min_radius", C.c_float), ("balance", C.c_int32), ("tree_ratio", C.c_float)]


class RrtcResult(C.Structure):
    _fields_ = [("solved", C.c_int32), ("status", C.c_int32), ("path_len", C.c_int32), ("cost", C.c_float),
                ("start_tree_size", C.c_int32), ("goal_tree_size", C.c_int32), ("iterations", C.c_int32),
                ("kernel_ms", C.c_double)]


class RrtcProblem(C.Structure):
    _fields_ = [("robot", C.c_void_p), ("env", C.c_void_p), ("start", C.c_void_p), ("goal", C.c_void_p),
                ("seed", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("num_streams", C.c_int32), ("hbm_budget_bytes", C.c_int64), ("max_batch_states", C.c_int64),
                ("plan_workers", C.c_int32), ("plan_batch", C.c_int32), ("plan_lanes", C.c_int32),
                ("planner_max_nodes", C.c_int32), ("plan_path_cap", C.c_int32), ("plan_max_iters", C.c_int32),
                ("plan_range", C.c_float), ("plan_resolution", C.c_float), ("step_rule", C.c_int32),
                ("plan_time_limit_s", C.c_double), ("plan_max_blocks", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("solved", C.c_int32), ("path_len", C.c_int32), ("cost", C.c_float),
                ("latency_ms", C.c_double), ("queue_ms", C.c_double)]


class ServerMetrics(C.Structure):
    _fields_ = [("completed", C.c_int64), ("batches", C.c_int64), ("plan_batches", C.c_int64),
                ("states_checked", C.c_int64), ("budget_in_use", C.c_int64), ("check_p50_ms", C.c_double),
                ("check_p95_ms", C.c_double), ("check_p99_ms", C.c_double), ("plan_p50_ms", C.c_double),
                ("plan_p95_ms", C.c_double), ("plan_p99_ms", C.c_double), ("elapsed_s", C.c_double)]


class Limits(C.Structure):
    _fields_ = [("max_links", C.c_int32), ("max_spheres", C.c_int32), ("max_self_pairs", C.c_int32),
                ("max_env_words", C.c_int32)]


# name -> argtypes (every function returns int32 status unless listed in _RESTYPE)
_vp, _i32, _i64, _f32, _u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_float, C.c_uint64
_i32p = C.POINTER(C.c_int32)
SIGNATURES = {
    "gbmp_last_error": [],
    "gbmp_status_string": [_i32],
    "gbmp_get_limits": [C.POINTER(Limits)],
    "gbmp_device_count": [_i32p],
    "gbmp_robot_create": [C.POINTER(RobotDesc), _i32, C.POINTER(_vp)],
    "gbmp_robot_destroy": [_vp],
    "gbmp_robot_info": [_vp, _i32p, _i32p, _i32p, _i32p, _i32p],
    "gbmp_robot_self_pairs": [_vp, _vp, _vp, _i32],
    "gbmp_robot_joints": [_vp, _vp, _vp, _vp, _vp],
    "gbmp_robot_use_codegen": [_vp, _i32],
    "gbmp_robot_device_status": [_vp, _i32p],
    "gbmp_robot_codegen_info": [_vp, C.c_char_p, _i64, C.POINTER(_i64), C.POINTER(_u64), C.POINTER(_i32),
                                C.POINTER(C.c_double)],
    "gbmp_env_create": [_i32, _vp, _vp, _i32, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp, C.POINTER(_vp)],
    "gbmp_env_destroy": [_vp],
    "gbmp_env_counts": [_vp, _i32p, _i32p, _i32p],
    "gbmp_fk": [_vp, _vp, _i64, _vp, _vp, _vp],
    "gbmp_check_states": [_vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp],
    "gbmp_check_states_fk": [_vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp, _vp],
    "gbmp_space_jacobian": [_vp, _vp, _i64, _vp, _vp],
    "gbmp_check_batch_create": [_i32, C.POINTER(_vp)],
    "gbmp_check_batch_run": [_vp, C.POINTER(CheckRequest), _i32, _i32, _vp],
    "gbmp_check_batch_destroy": [_vp],
    "gbmp_robot_set_edge_form": [_vp, _i32],
    "gbmp_robot_set_stage_wait": [_vp, _i32],
    "gbmp_check_edges": [_vp, _vp, _vp, _vp, _i64, _f32, _i32, _vp, _vp, _vp, _vp, _vp],
    "gbmp_check_edges_noalloc": [_vp, _vp, _vp, _vp, _i64, _f32, _i32, _vp, _vp, _vp, _vp, _vp],
    "gbmp_nearest": [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _vp],
    "gbmp_steer": [_vp, _vp, _vp, _vp, _i64, _f32, _vp],
    "gbmp_gather_states": [_i32, _vp, _i64, _vp, _i64, _vp, _vp, _vp],
    "gbmp_sample": [_vp, _u64, _u64, _i64, _vp, _vp],
    "gbmp_project_states": [_vp, C.c_void_p, _vp, _i64, _vp, _vp, _vp],
    "gbmp_constrained_motions": [_vp, _vp, C.c_void_p, _vp, _vp, _i64, _f32, _i32, _vp, _vp, _vp, _vp, _i32, _vp],
    "gbmp_planner_create": [_vp, _i32, _i32, C.POINTER(_vp)],
    "gbmp_planner_destroy": [_vp],
    "gbmp_rrtc_solve": [_vp, _vp, _vp, _vp, C.POINTER(RrtcSettings), _vp, _i32, C.POINTER(RrtcResult), _vp],
    "gbmp_rrtc_solve_goals": [_vp, _vp, _vp, _vp, _i32, C.POINTER(RrtcSettings), _vp, _i32, C.POINTER(RrtcResult),
                              _vp],
    "gbmp_batch_planner_create": [_i32, _i32, _i32, _i32, C.POINTER(_vp)],
    "gbmp_batch_planner_destroy": [_vp],
    "gbmp_rrtc_solve_batch": [_vp, _i32, C.POINTER(RrtcProblem), C.POINTER(RrtcSettings), _i32, _i32,
                              C.POINTER(RrtcResult), _vp, _vp],
    "gbmp_rrtc_solve_batch_auto": [_vp, _i32, C.POINTER(RrtcProblem), C.POINTER(RrtcSettings), _i32,
                                   C.POINTER(RrtcResult), _vp, _i32p, _vp],
    "gbmp_batch_autotune_lookup": [_i32, C.POINTER(RrtcProblem), C.POINTER(RrtcSettings), _i32, _i32p,
                                   C.POINTER(C.c_double), _i32, _i32p, _i32p],
    "gbmp_batch_autotune_reset": [],
    "gbmp_server_create": [C.POINTER(ServerConfig), C.POINTER(_vp)],
    "gbmp_server_add_robot": [_vp, _vp, _i32p],
    "gbmp_server_add_env": [_vp, _vp, _i32p],
    "gbmp_server_start": [_vp],
    "gbmp_server_submit_check": [_vp, _i32, _i32, _vp, _i64, _vp, C.POINTER(C.c_int64)],
    "gbmp_server_submit_plan": [_vp, _i32, _i32, _vp, _vp, _u64, _vp, _i32, C.POINTER(C.c_int64)],
    "gbmp_server_wait": [_vp, _i64, C.c_double, C.POINTER(RequestInfo)],
    "gbmp_server_stats": [_vp, C.POINTER(ServerMetrics)],
    "gbmp_server_destroy": [_vp],
    "gbmp_profile_enable": [_i32],
    "gbmp_profile_reset": [],
    "gbmp_profile_read": [_i32, C.POINTER(C.c_double), C.POINTER(C.c_int64)],
    "gbmp_launch_count": [C.POINTER(C.c_int64)],
    "gbmp_work_counting": [_i32],
    "gbmp_work_read": [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)],
    "gbmp_measure_fp32_peak": [C.c_double, C.POINTER(C.c_double)],
}
PROF_EDGE_WAVE, PROF_CHECK_STATES, PROF_FK, PROF_OTHER = 0, 1, 2, 3
_RESTYPE = {"gbmp_last_error": C.c_char_p, "gbmp_status_string": C.c_char_p}

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libgbmp.so, building it first if the sources are newer."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise ImportError(f"libgbmp.so not found at {path}; run isaac_sim_ros2_humble_gb300.build.build()")
    lib = C.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, C.c_int32)
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        msg = load().gbmp_last_error()
        raise GbmpError(status, msg.decode() if msg else "")


def ptr(x) -> int:
    """Device (or host) address of a torch tensor, numpy array, int or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(type(x))


def stream_handle(stream) -> int:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except Exception:
            pass
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def profile_enable(on: bool) -> None:
    check(load().gbmp_profile_enable(int(on)))


def profile_reset() -> None:
    check(load().gbmp_profile_reset())


def profile_read(family: int):
    ms, n = C.c_double(), C.c_int64()
    check(load().gbmp_profile_read(family, C.byref(ms), C.byref(n)))
    return ms.value, n.value


def launch_count() -> int:
    n = C.c_int64()
    check(load().gbmp_launch_count(C.byref(n)))
    return n.value


def work_counting(on: bool) -> None:
    check(load().gbmp_work_counting(int(on)))


def work_read():
    f, n = C.c_uint64(), C.c_uint64()
    check(load().gbmp_work_read(C.byref(f), C.byref(n)))
    return f.value, n.value


def measure_fp32_peak(seconds: float = 1.0) -> float:
    t = C.c_double()
    check(load().gbmp_measure_fp32_peak(seconds, C.byref(t)))
    return t.value


def device_count() -> int:
    c = C.c_int32(0)
    check(load().gbmp_device_count(C.byref(c)))
    return c.value
