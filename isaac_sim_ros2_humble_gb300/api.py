"""Python handles over the libgbmp C-ABI.

`Robot` and `Env` own the C handles; the operations take torch CUDA tensors
(device memory) and launch on the current torch stream.  Every call goes through
libgbmp.so; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check, ptr, stream_handle
from .workloads import Environment, RobotModel


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Robot:
    """A robot model resident on the device (replaces the SingleArmSpace tables)."""

    def __init__(self, model: RobotModel, codegen: bool = False):
        lib = _lib.load()
        self.model = model
        keep = [_c(model.joint_types, np.int32), _c(model.joint_poses.reshape(-1, 16), np.float32),
                _c(model.joint_axes, np.float32), _c(model.parent, np.int32),
                _c(model.sphere_link, np.int32), _c(model.sphere_pos, np.float32),
                _c(model.sphere_r, np.float32), _c(model.active, np.uint8), _c(model.lower, np.float32),
                _c(model.upper, np.float32), _c(model.default, np.float32), _c(model.enables, np.uint8)]
        d = _lib.RobotDesc(model.num_links, *(k.ctypes.data for k in keep[:4]), model.num_spheres,
                           *(k.ctypes.data for k in keep[4:]), float(model.resolution))
        h = C.c_void_p()
        check(lib.gbmp_robot_create(C.byref(d), _lib.ROBOT_CODEGEN if codegen else _lib.ROBOT_GENERIC,
                                    C.byref(h)))
        self.handle = h
        L, S, P, dim, cg = (C.c_int32() for _ in range(5))
        check(lib.gbmp_robot_info(h, C.byref(L), C.byref(S), C.byref(P), C.byref(dim), C.byref(cg)))
        self.L, self.S, self.P, self.dim = L.value, S.value, P.value, dim.value

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().gbmp_robot_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def self_pairs(self):
        pairs = np.zeros(2 * max(self.P, 1), np.int32)
        thr = np.zeros(max(self.P, 1), np.float32)
        check(_lib.load().gbmp_robot_self_pairs(self.handle, pairs.ctypes.data, thr.ctypes.data, max(self.P, 1)))
        return pairs[: 2 * self.P].reshape(-1, 2), thr[: self.P]

    def set_edge_form(self, form: int):
        """Edge-validation form of this handle: 0 automatic, 1 state by state, 4 or 10
        states per chunk (tuning and tests; results do not depend on it)."""
        check(_lib.load().gbmp_robot_set_edge_form(self.handle, int(form)))

    def set_stage_wait(self, polls: int):
        """Polls of the kernels' bounded staging wait before a block gives up (0: at once,
        so the give-up path runs; -1: the default).  Test control."""
        check(_lib.load().gbmp_robot_set_stage_wait(self.handle, int(polls)))

    def device_status(self) -> int:
        """GBMP_ERR_TIMEOUT once a kernel working for this handle gave up a bounded wait."""
        st = C.c_int32(-1)
        check(_lib.load().gbmp_robot_device_status(self.handle, C.byref(st)))
        return st.value

    def use_codegen(self, enable: bool):
        check(_lib.load().gbmp_robot_use_codegen(self.handle, int(enable)))

    def codegen_info(self):
        """Generated source, cache key, cache origin (0 compiled, 1 in process, 2 disk)
        and NVRTC milliseconds of a robot created with codegen=True."""
        lib = _lib.load()
        n, h, c, ms = C.c_int64(), C.c_uint64(), C.c_int32(), C.c_double()
        check(lib.gbmp_robot_codegen_info(self.handle, None, 0, C.byref(n), C.byref(h), C.byref(c), C.byref(ms)))
        buf = C.create_string_buffer(n.value)
        check(lib.gbmp_robot_codegen_info(self.handle, buf, n.value, None, None, None, None))
        return {"source": buf.value.decode(), "hash": h.value, "cache": c.value, "compile_ms": ms.value}


class Env:
    """An obstacle set resident on the device (replaces the EnvConstraint* tables)."""

    def __init__(self, env: Environment):
        lib = _lib.load()
        self.env = env
        ns, nb, nc = env.counts
        k = [_c(env.sphere_pos, np.float32), _c(env.sphere_r, np.float32), _c(env.box_pos, np.float32),
             _c(env.box_rot, np.float32), _c(env.box_min, np.float32), _c(env.box_max, np.float32),
             _c(env.cyl_pos, np.float32), _c(env.cyl_rot, np.float32), _c(env.cyl_radius, np.float32),
             _c(env.cyl_height, np.float32)]
        h = C.c_void_p()
        check(lib.gbmp_env_create(ns, k[0].ctypes.data, k[1].ctypes.data, nb, k[2].ctypes.data,
                                  k[3].ctypes.data, k[4].ctypes.data, k[5].ctypes.data, nc,
                                  k[6].ctypes.data, k[7].ctypes.data, k[8].ctypes.data, k[9].ctypes.data,
                                  C.byref(h)))
        self.handle = h
        self.counts = (ns, nb, nc)

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().gbmp_env_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _n(q, L):
    assert q.is_cuda and q.dtype.__str__() == "torch.float32" and q.is_contiguous(), "q must be contiguous CUDA float32"
    assert q.shape[-1] == L, f"last dim {q.shape[-1]} != L={L}"
    return q.numel() // L


def fk(robot: Robot, q, poses=None, centers=None, stream=None):
    n = _n(q, robot.L)
    check(_lib.load().gbmp_fk(robot.handle, ptr(q), n, ptr(poses), ptr(centers), stream_handle(stream)))


def space_jacobian(robot: Robot, q, jac, stream=None):
    """Space Jacobian of every link of the states q [n, L] into jac [n, L, L, 6]
    (gbmp_space_jacobian)."""
    n = _n(q, robot.L)
    check(_lib.load().gbmp_space_jacobian(robot.handle, ptr(q), n, ptr(jac), stream_handle(stream)))


def check_states(robot: Robot, env: Env, q, verdict=None, costs=None, total=None, mode=_lib.CHECK_VERDICT,
                 stream=None, poses=None, centers=None):
    """Collision check of the states q [n, L]; with poses [n, L, 4, 4] and / or
    centers [n, S, 3] the same FK is written out too (one launch)."""
    n = _n(q, robot.L)
    if poses is None and centers is None:
        check(_lib.load().gbmp_check_states(robot.handle, env.handle, ptr(q), n, mode, ptr(verdict), ptr(costs),
                                            ptr(total), stream_handle(stream)))
    else:
        check(_lib.load().gbmp_check_states_fk(robot.handle, env.handle, ptr(q), n, mode, ptr(verdict), ptr(costs),
                                               ptr(total), ptr(poses), ptr(centers), stream_handle(stream)))


class CheckBatch:
    """State checks of many (robot, scene) requests in one launch (gbmp_check_batch_*).
    run() takes a list of dicts with keys robot, env, q and optionally verdict, costs,
    total, poses, centers (CUDA tensors, as check_states takes them).  One handle serves
    one stream at a time."""

    def __init__(self, max_requests: int = 1024):
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.gbmp_check_batch_create(int(max_requests), C.byref(h)))
        self.handle = h
        self.max_requests = int(max_requests)

    def run(self, requests, mode=_lib.CHECK_VERDICT, stream=None):
        arr = (_lib.CheckRequest * max(1, len(requests)))()
        for i, r in enumerate(requests):
            robot = r["robot"]
            n = _n(r["q"], robot.L)
            arr[i] = _lib.CheckRequest(robot.handle, r["env"].handle, ptr(r["q"]), n, ptr(r.get("verdict")),
                                       ptr(r.get("costs")), ptr(r.get("total")), ptr(r.get("poses")),
                                       ptr(r.get("centers")))
        check(_lib.load().gbmp_check_batch_run(self.handle, arr, len(requests), int(mode), stream_handle(stream)))

    def close(self):
        if self.handle:
            _lib.load().gbmp_check_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def check_edges(robot: Robot, env: Env, q_from, q_to, resolution: float = 0.0, rule: int = _lib.STEP_L2,
                ok=None, first_hit=None, length=None, num_steps=None, stream=None):
    n = _n(q_from, robot.L)
    assert q_to.shape == q_from.shape
    check(_lib.load().gbmp_check_edges(robot.handle, env.handle, ptr(q_from), ptr(q_to), n, float(resolution),
                                       rule, ptr(ok), ptr(first_hit), ptr(length), ptr(num_steps),
                                       stream_handle(stream)))


def project_states(robot: Robot, q, task_link: int = -1, offset=None, reference=(0, 0, 0, 0, 0, 0),
                   tolerance=(0, 0, 0, 0, 0, 0), use_boundary: bool = True, iterations: int = 10, task_cost=None,
                   bound_cost=None, stream=None):
    """Project the states q [n, L] (in place) onto a task-space region of link
    `task_link` (pose of `offset` in that link, reference x y z roll pitch yaw, per-axis
    tolerances) and the joint limits; final costs into task_cost / bound_cost [n]."""
    n = _n(q, robot.L)
    p = _lib.Projection()
    p.task_link = int(task_link)
    off = np.eye(4, dtype=np.float32) if offset is None else np.asarray(offset, np.float32)
    p.offset[:] = [float(v) for v in off.reshape(16)]
    p.reference[:] = [float(v) for v in reference]
    p.tolerance[:] = [float(v) for v in tolerance]
    p.use_boundary = int(bool(use_boundary))
    p.iterations = int(iterations)
    check(_lib.load().gbmp_project_states(robot.handle, C.byref(p), ptr(q), n, ptr(task_cost), ptr(bound_cost),
                                          stream_handle(stream)))


def constrained_motions(robot: Robot, env: Env, q_from, q_to, task_link: int = -1, offset=None,
                        reference=(0, 0, 0, 0, 0, 0), tolerance=(0, 0, 0, 0, 0, 0), use_boundary: bool = True,
                        resolution: float = 0.0, max_iterations: int = 10000, ok=None, cost=None, num_states=None,
                        states=None, stream=None):
    """Constrained motions q_from[k] -> q_to[k] ([n, L] each) on the task-space region and
    the joint limits (gbmp_constrained_motions): ok / cost / num_states [n]; states
    [n, cap, L] receives the first cap recorded states of each motion."""
    n = _n(q_from, robot.L)
    assert q_to.shape == q_from.shape
    p = _lib.Projection()
    p.task_link = int(task_link)
    off = np.eye(4, dtype=np.float32) if offset is None else np.asarray(offset, np.float32)
    p.offset[:] = [float(v) for v in off.reshape(16)]
    p.reference[:] = [float(v) for v in reference]
    p.tolerance[:] = [float(v) for v in tolerance]
    p.use_boundary = int(bool(use_boundary))
    p.iterations = 2
    cap = int(states.shape[1]) if states is not None else 0
    check(_lib.load().gbmp_constrained_motions(robot.handle, env.handle, C.byref(p), ptr(q_from), ptr(q_to), n,
                                               float(resolution), int(max_iterations), ptr(ok), ptr(cost),
                                               ptr(num_states), ptr(states), cap, stream_handle(stream)))


def nearest(robot: Robot, tree, queries, out, cand=None, stream=None):
    M = _n(tree, robot.L)
    Q = _n(queries, robot.L)
    nc = cand.numel() if cand is not None else 0
    check(_lib.load().gbmp_nearest(robot.handle, ptr(tree), M, ptr(cand), nc, ptr(queries), Q, ptr(out),
                                   stream_handle(stream)))


def steer(robot: Robot, q_from, q_to, max_distance: float, idx=None, stream=None):
    n = _n(q_to, robot.L)
    check(_lib.load().gbmp_steer(robot.handle, ptr(q_from), ptr(idx), ptr(q_to), n, float(max_distance),
                                 stream_handle(stream)))


def gather_states(src, idx, out, bad=None, stream=None):
    """out[k] = src[idx[k]] (rows of src.shape[1] floats) in one launch; an index outside
    the rows gives a NaN row and sets bad[0] to 1 (bad: int32 device tensor or None)."""
    L = int(src.shape[1])
    check(_lib.load().gbmp_gather_states(L, ptr(src), int(src.shape[0]), ptr(idx), int(idx.shape[0]), ptr(out),
                                         ptr(bad), stream_handle(stream)))


def sample(robot: Robot, seed: int, offset: int, out, stream=None):
    n = _n(out, robot.L)
    check(_lib.load().gbmp_sample(robot.handle, seed, offset, n, ptr(out), stream_handle(stream)))


class Planner:
    """Device-resident RRT-Connect trees for one robot (replaces CPRRTC::RobotSolver)."""

    def __init__(self, robot: Robot, max_nodes: int = 1_000_000, path_cap: int = 65536):
        h = C.c_void_p()
        check(_lib.load().gbmp_planner_create(robot.handle, int(max_nodes), int(path_cap), C.byref(h)))
        self.handle = h
        self.robot = robot
        self.path_cap = int(path_cap)
        self._path = np.zeros((self.path_cap, robot.L), np.float32)

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().gbmp_planner_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, env: Env, start, goal, lanes: int = 1024, max_iters: int = 100000, range_: float = 0.1,
              resolution: float = 0.0, rule: int = _lib.STEP_L2, seed: int = 0, time_limit_s: float = 10.0,
              stream=None, raise_on_failure: bool = False, dynamic_domain: bool = False, dd_alpha: float = 1e-4,
              dd_radius: float = 4.0, dd_min_radius: float = 1.0, balance: int = _lib.BALANCE_DEFAULT,
              tree_ratio: float = 0.0):
        """Returns (result, path): result is a dict of the C result struct, path the
        [path_len, L] float32 waypoints (empty when not solved).  `goal` is one full joint
        vector [L] or several [n, L] (every one a root of the goal tree).  dynamic_domain
        turns on pRRTC's dynamic-domain sampling with its dd_* parameters; balance and
        tree_ratio choose pRRTC's tree-balancing strategy (gbmp_rrtc_settings)."""
        st = _lib.RrtcSettings(int(lanes), int(max_iters), float(range_), float(resolution), int(rule), int(seed),
                               float(time_limit_s), int(bool(dynamic_domain)), float(dd_alpha), float(dd_radius),
                               float(dd_min_radius), int(balance), float(tree_ratio))
        res = _lib.RrtcResult()
        s0 = _c(start, np.float32).reshape(-1)
        g0 = _c(goal, np.float32).reshape(-1, self.robot.L)
        assert s0.size == self.robot.L
        status = _lib.load().gbmp_rrtc_solve_goals(self.handle, env.handle, s0.ctypes.data, g0.ctypes.data,
                                                   int(g0.shape[0]), C.byref(st), self._path.ctypes.data,
                                                   self.path_cap, C.byref(res), stream_handle(stream))
        if status not in (_lib.OK, 6, 7) or raise_on_failure:
            check(status)
        out = {f: getattr(res, f) for f, _ in _lib.RrtcResult._fields_}
        out["status_code"] = status
        path = self._path[: res.path_len].copy() if res.solved else np.zeros((0, self.robot.L), np.float32)
        return out, path


class BatchPlanner:
    """Many heterogeneous RRT-Connect problems per launch (see gbmp_rrtc_solve_batch)."""

    def __init__(self, max_problems: int = 256, max_nodes: int = 32768, max_links: int = 16,
                 path_cap: int = 4096):
        h = C.c_void_p()
        check(_lib.load().gbmp_batch_planner_create(int(max_problems), int(max_nodes), int(max_links),
                                                    int(path_cap), C.byref(h)))
        self.handle = h
        self.max_problems, self.max_links, self.path_cap = int(max_problems), int(max_links), int(path_cap)
        self._paths = np.zeros((self.max_problems, self.path_cap, self.max_links), np.float32)

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().gbmp_batch_planner_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _inputs(problems, max_iters, range_, resolution, rule, time_limit_s, dynamic_domain, dd_alpha, dd_radius,
                dd_min_radius, balance, tree_ratio):
        n = len(problems)
        arr = (_lib.RrtcProblem * n)()
        keep = []
        for i, (R, E, s0, g0, seed) in enumerate(problems):
            a, b = _c(s0, np.float32).reshape(-1), _c(g0, np.float32).reshape(-1)
            keep += [a, b]
            arr[i] = _lib.RrtcProblem(R.handle.value, E.handle.value, a.ctypes.data, b.ctypes.data, int(seed))
        st = _lib.RrtcSettings(0, int(max_iters), float(range_), float(resolution), int(rule), 0, float(time_limit_s),
                               int(bool(dynamic_domain)), float(dd_alpha), float(dd_radius), float(dd_min_radius),
                               int(balance), float(tree_ratio))
        return arr, st, keep

    def solve(self, problems, lanes_per_problem=8, use_graph: bool = True, max_iters: int = 100000,
              range_: float = 0.1, resolution: float = 0.0, rule: int = _lib.STEP_L2, time_limit_s: float = 10.0,
              stream=None, dynamic_domain: bool = False, dd_alpha: float = 1e-4, dd_radius: float = 4.0,
              dd_min_radius: float = 1.0, balance: int = _lib.BALANCE_DEFAULT, tree_ratio: float = 0.0):
        """problems: list of (Robot, Env, start[L], goal[L], seed).  Returns a list of
        (result dict, path [path_len, L]).  lanes_per_problem="auto" lets the library's
        launch-shape autotuner choose (gbmp_rrtc_solve_batch_auto); the lanes it used are
        then in self.last_lanes."""
        n = len(problems)
        arr, st, keep = self._inputs(problems, max_iters, range_, resolution, rule, time_limit_s, dynamic_domain,
                                     dd_alpha, dd_radius, dd_min_radius, balance, tree_ratio)
        res = (_lib.RrtcResult * n)()
        paths = self._paths[:n]
        if lanes_per_problem == "auto":
            used = C.c_int32()
            check(_lib.load().gbmp_rrtc_solve_batch_auto(self.handle, n, arr, C.byref(st), int(bool(use_graph)), res,
                                                         paths.ctypes.data, C.byref(used), stream_handle(stream)))
            self.last_lanes = used.value
        else:
            check(_lib.load().gbmp_rrtc_solve_batch(self.handle, n, arr, C.byref(st), int(lanes_per_problem),
                                                    int(bool(use_graph)), res, paths.ctypes.data,
                                                    stream_handle(stream)))
            self.last_lanes = int(lanes_per_problem)
        out = []
        flat = self._paths.reshape(self.max_problems, -1)
        for i in range(n):
            r = {f: getattr(res[i], f) for f, _ in _lib.RrtcResult._fields_}
            L = problems[i][0].L
            p = flat[i, : r["path_len"] * L].reshape(-1, L).copy() if r["solved"] else np.zeros((0, L), np.float32)
            out.append((r, p))
        return out

    @classmethod
    def autotune_record(cls, problems, use_graph: bool = True, max_iters: int = 100000, range_: float = 0.1,
                        resolution: float = 0.0, rule: int = _lib.STEP_L2, time_limit_s: float = 10.0,
                        dynamic_domain: bool = False, dd_alpha: float = 1e-4, dd_radius: float = 4.0,
                        dd_min_radius: float = 1.0, balance: int = _lib.BALANCE_DEFAULT, tree_ratio: float = 0.0):
        """The autotuner's record for this batch shape: {lanes: least ms (-1 untried)} and
        the chosen lanes (-1 while exploring, None if the shape was never solved)."""
        arr, st, keep = cls._inputs(problems, max_iters, range_, resolution, rule, time_limit_s, dynamic_domain,
                                    dd_alpha, dd_radius, dd_min_radius, balance, tree_ratio)
        lanes, ms = (C.c_int32 * 16)(), (C.c_double * 16)()
        cnt, chosen = C.c_int32(), C.c_int32()
        check(_lib.load().gbmp_batch_autotune_lookup(len(problems), arr, C.byref(st), int(bool(use_graph)), lanes, ms,
                                                     16, C.byref(cnt), C.byref(chosen)))
        if cnt.value == 0:
            return {}, None
        return {lanes[i]: ms[i] for i in range(min(cnt.value, 16))}, chosen.value

    @staticmethod
    def autotune_reset():
        check(_lib.load().gbmp_batch_autotune_reset())


class Server:
    """Continuous-batching request server (gbmp_server_*): resident robots and scenes,
    FK+collision requests batched as they arrive, plan requests solved in batched
    launches.  Host arrays passed to submit_* are kept alive until wait() returns."""

    def __init__(self, num_streams: int = 4, hbm_budget_bytes: int = 1 << 30, max_batch_states: int = 1 << 20,
                 plan_workers: int = 1, plan_batch: int = 64, plan_lanes: int = 8, planner_max_nodes: int = 32768,
                 plan_path_cap: int = 4096, plan_max_iters: int = 100000, plan_range: float = 0.1,
                 plan_resolution: float = 0.01, step_rule: int = _lib.STEP_LINF, plan_time_limit_s: float = 10.0,
                 plan_max_blocks: int = 0):
        cfg = _lib.ServerConfig(num_streams, hbm_budget_bytes, max_batch_states, plan_workers, plan_batch, plan_lanes,
                                planner_max_nodes, plan_path_cap, plan_max_iters, plan_range, plan_resolution,
                                step_rule, plan_time_limit_s, int(plan_max_blocks))
        h = C.c_void_p()
        check(_lib.load().gbmp_server_create(C.byref(cfg), C.byref(h)))
        self.handle = h
        self.robots, self.envs = [], []
        self._live = {}

    def add_robot(self, robot: Robot) -> int:
        i = C.c_int32()
        check(_lib.load().gbmp_server_add_robot(self.handle, robot.handle, C.byref(i)))
        self.robots.append(robot)
        return i.value

    def add_env(self, env: Env) -> int:
        i = C.c_int32()
        check(_lib.load().gbmp_server_add_env(self.handle, env.handle, C.byref(i)))
        self.envs.append(env)
        return i.value

    def start(self):
        check(_lib.load().gbmp_server_start(self.handle))

    def submit_check(self, robot_id: int, env_id: int, q: np.ndarray, verdict: np.ndarray) -> int:
        q = np.ascontiguousarray(q, np.float32)
        assert verdict.dtype == np.uint8 and verdict.flags.c_contiguous and verdict.size >= q.shape[0]
        t = C.c_int64()
        check(_lib.load().gbmp_server_submit_check(self.handle, robot_id, env_id, q.ctypes.data, q.shape[0],
                                                   verdict.ctypes.data, C.byref(t)))
        self._live[t.value] = (q, verdict)
        return t.value

    def submit_plan(self, robot_id: int, env_id: int, start, goal, seed: int, path: np.ndarray) -> int:
        s0, g0 = _c(start, np.float32).reshape(-1), _c(goal, np.float32).reshape(-1)
        t = C.c_int64()
        check(_lib.load().gbmp_server_submit_plan(self.handle, robot_id, env_id, s0.ctypes.data, g0.ctypes.data,
                                                  int(seed), path.ctypes.data, path.shape[0], C.byref(t)))
        self._live[t.value] = (s0, g0, path)
        return t.value

    def wait(self, ticket: int, timeout_s: float = 60.0):
        info = _lib.RequestInfo()
        st = _lib.load().gbmp_server_wait(self.handle, ticket, float(timeout_s), C.byref(info))
        if st == 6:
            return None
        check(st)
        self._live.pop(ticket, None)
        return {f: getattr(info, f) for f, _ in _lib.RequestInfo._fields_}

    def stats(self):
        m = _lib.ServerMetrics()
        check(_lib.load().gbmp_server_stats(self.handle, C.byref(m)))
        return {f: getattr(m, f) for f, _ in _lib.ServerMetrics._fields_}

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().gbmp_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
