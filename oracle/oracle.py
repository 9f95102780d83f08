"""ctypes wrapper around the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
import this module, and only as the checker or the timed CPU restatement of the
reference algorithm.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
if _HERE not in sys.path:
    sys.path.insert(0, _HERE)
import build as _build  # noqa: E402

STEP_L2, STEP_LINF, STEP_COUNT = 0, 1, 2

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class _Robot(C.Structure):
    _fields_ = [("L", C.c_int32), ("type", C.c_void_p), ("pose", C.c_void_p), ("axis", C.c_void_p),
                ("parent", C.c_void_p), ("S", C.c_int32), ("sph_link", C.c_void_p),
                ("sph_pos", C.c_void_p), ("sph_r", C.c_void_p)]


class _Env(C.Structure):
    _fields_ = [("ns", C.c_int32), ("sph", C.c_void_p), ("nb", C.c_int32), ("box_inv", C.c_void_p),
                ("box_min", C.c_void_p), ("box_max", C.c_void_p), ("nc", C.c_int32),
                ("cyl_inv", C.c_void_p), ("cyl_r", C.c_void_p), ("cyl_h", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.or_fk_f32.argtypes = [vp, _f32p, C.c_int64, _f32p]
        L.or_fk_f64.argtypes = [vp, _f64p, C.c_int64, _f64p]
        L.or_sphere_centers_f32.argtypes = [vp, _f32p, C.c_int64, _f32p]
        L.or_sphere_centers_f64.argtypes = [vp, _f64p, C.c_int64, _f64p]
        L.or_self_pairs.argtypes = [vp, vp, _i32p, _f32p, C.c_int32]
        L.or_self_pairs.restype = C.c_int32
        L.or_inverse_pose.argtypes = [_f32p, _f32p, _f32p]
        L.or_check_states.argtypes = [vp, vp, C.c_int32, _i32p, _f32p, _f32p, C.c_int64, vp, vp, C.c_int32]
        L.or_clearance_f64.argtypes = [vp, vp, C.c_int32, _i32p, _f64p, C.c_int64, _f64p, C.c_int32]
        L.or_edge_steps.argtypes = [_f32p, _f32p, C.c_int32, C.c_float, C.c_int32, _f32p, vp]
        L.or_edge_steps.restype = C.c_int32
        L.or_edge_state.argtypes = [_f32p, _f32p, _f32p, C.c_int32, C.c_int32, C.c_int32, _f32p]
        L.or_check_motions.argtypes = [vp, vp, C.c_int32, _i32p, _f32p, _f32p, _f32p, C.c_int64,
                                       C.c_float, C.c_int32, C.c_int32, _u8p, _i32p, _i32p, _f32p, C.c_int32]
        L.or_nearest.argtypes = [_f32p, C.c_int64, C.c_int32, vp, vp, C.c_int64, _f32p, C.c_int64,
                                 _i32p, C.c_int32]
        L.or_steer.argtypes = [_f32p, _f32p, C.c_int64, C.c_int32, C.c_float]
        L.or_sample.argtypes = [_f32p, _f32p, _u8p, _f32p, C.c_int32, C.c_uint64, C.c_uint64, C.c_int64, _f32p]
        L.or_rrtc.argtypes = [vp, vp, C.c_int32, _i32p, _f32p, _f32p, _f32p, _u8p, _f32p, _f32p, _f32p,
                              C.c_float, C.c_float, C.c_int32, C.c_uint64, C.c_int32, C.c_int32, _f32p, C.c_int32,
                              C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_int32), _i32p]
        L.or_rrtc.restype = C.c_int32
        L.or_rrtc_lanes.argtypes = [vp, vp, C.c_int32, _i32p, _f32p, _f32p, _f32p, _u8p, _f32p, _f32p, _f32p,
                                    C.c_float, C.c_float, C.c_int32, C.c_uint64, C.c_int32, C.c_int32, C.c_float,
                                    C.c_int32, C.c_int32, _f32p, C.c_int32, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_float), C.POINTER(C.c_int32), _i32p, C.c_int32]
        L.or_rrtc_lanes.restype = C.c_int32
        L.or_balance_tree.argtypes = [C.c_int32, C.c_float, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_int32]
        L.or_balance_tree.restype = C.c_int32
        L.or_num_threads.restype = C.c_int32
        L.or_project.argtypes = [vp, _u8p, _f32p, _f32p, vp, _f32p, C.c_int64, vp, vp, C.c_int32]
        L.or_constrained_motions.argtypes = [vp, vp, C.c_int32, _i32p, _f32p, _u8p, _f32p, _f32p, vp, _f32p, _f32p,
                                             C.c_int64, C.c_float, C.c_int32, _u8p, _f32p, _i32p, vp, C.c_int32,
                                             C.c_int32]
        _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Projection(C.Structure):
    """Task-space + joint-limit projection settings (layout of or_projection)."""
    _fields_ = [("task_link", C.c_int32), ("offset", C.c_float * 16), ("reference", C.c_float * 6),
                ("tolerance", C.c_float * 6), ("use_boundary", C.c_int32), ("iterations", C.c_int32)]


def projection(task_link=-1, offset=None, reference=(0, 0, 0, 0, 0, 0), tolerance=(0, 0, 0, 0, 0, 0),
               use_boundary=True, iterations=10) -> Projection:
    p = Projection()
    p.task_link = int(task_link)
    off = np.eye(4, dtype=np.float32) if offset is None else np.asarray(offset, np.float32).reshape(16)
    p.offset[:] = [float(v) for v in np.asarray(off, np.float32).reshape(16)]
    p.reference[:] = [float(v) for v in reference]
    p.tolerance[:] = [float(v) for v in tolerance]
    p.use_boundary = int(bool(use_boundary))
    p.iterations = int(iterations)
    return p


class OracleModel:
    """Robot + environment + self-pair list laid out for the C oracle."""

    def __init__(self, robot, env=None):
        self.robot = robot
        self._keep = []
        k = lambda a, dt: self._keep.append(_c(a, dt)) or self._keep[-1]
        self.L, self.S = robot.num_links, robot.num_spheres
        self.r = _Robot(self.L, k(robot.joint_types, np.int32).ctypes.data,
                        k(robot.joint_poses, np.float32).ctypes.data,
                        k(robot.joint_axes, np.float32).ctypes.data,
                        k(robot.parent, np.int32).ctypes.data, self.S,
                        k(robot.sphere_link, np.int32).ctypes.data,
                        k(robot.sphere_pos, np.float32).ctypes.data,
                        k(robot.sphere_r, np.float32).ctypes.data)
        en = k(robot.enables, np.uint8)
        cap = self.S * self.S
        pairs = np.zeros(2 * cap + 2, np.int32)
        thr = np.zeros(cap + 1, np.float32)
        n = lib().or_self_pairs(C.byref(self.r), en.ctypes.data, pairs, thr, cap)
        self.pairs = pairs[: 2 * n].copy()
        self.thr_sq = thr[:n].copy()
        self.npairs = n
        self.set_env(env)

    def set_env(self, env):
        from isaac_sim_ros2_humble_gb300.workloads import Environment
        env = env if env is not None else Environment.empty()
        self.env = env
        ns, nb, nc = env.counts
        sph = _c(np.concatenate([env.sphere_pos.reshape(-1, 3), env.sphere_r.reshape(-1, 1)], 1), np.float32)
        binv = np.zeros((max(nb, 1), 12), np.float32)
        for i in range(nb):
            lib().or_inverse_pose(_c(env.box_pos[i], np.float32), _c(env.box_rot[i].reshape(9), np.float32), binv[i])
        cinv = np.zeros((max(nc, 1), 12), np.float32)
        for i in range(nc):
            lib().or_inverse_pose(_c(env.cyl_pos[i], np.float32), _c(env.cyl_rot[i].reshape(9), np.float32), cinv[i])
        self.box_inv, self.cyl_inv = binv, cinv
        bmin = _c(env.box_min, np.float32)
        bmax = _c(env.box_max, np.float32)
        cr = _c(env.cyl_radius, np.float32)
        ch = _c(env.cyl_height, np.float32)
        self._env_keep = [sph, binv, cinv, bmin, bmax, cr, ch]
        self.e = _Env(ns, sph.ctypes.data, nb, binv.ctypes.data, bmin.ctypes.data, bmax.ctypes.data,
                      nc, cinv.ctypes.data, cr.ctypes.data, ch.ctypes.data)

    # ---- kinematics ----
    def fk(self, q, f64=False):
        q = np.asarray(q).reshape(-1, self.L)
        n = q.shape[0]
        if f64:
            out = np.zeros((n, self.L, 16), np.float64)
            lib().or_fk_f64(C.byref(self.r), _c(q, np.float64), n, out)
        else:
            out = np.zeros((n, self.L, 16), np.float32)
            lib().or_fk_f32(C.byref(self.r), _c(q, np.float32), n, out)
        return out

    def space_jacobian(self, q, f64=True):
        """Space Jacobian of every link, [n, L, L, 6] (state, link, joint, column), from
        the oracle's FK (FP64 by default): the reference's kin_space_jacobian_per_link_kernel
        (SingleArmStates.cu:223-338) restated in numpy -- for link i and joint j, w = R_j
        a_j with a_j the joint axis as given; a revolute column is (w, w x (p_i - p_j)), a
        prismatic one (0, w); link 0, joint 0, j > i and other joint types give zeros."""
        P = self.fk(q, f64=f64)
        n, L = P.shape[0], self.L
        dt = np.float64 if f64 else np.float32
        R = P[:, :, [0, 1, 2, 4, 5, 6, 8, 9, 10]].reshape(n, L, 3, 3).astype(dt)
        p = P[:, :, [3, 7, 11]].astype(dt)
        axes = np.asarray(self.robot.joint_axes, dt).reshape(L, 3)
        types = np.asarray(self.robot.joint_types).reshape(L)
        w = np.einsum("njab,jb->nja", R, axes)            # [n, L(joint), 3]
        out = np.zeros((n, L, L, 6), dt)
        for i in range(1, L):
            for j in range(1, i + 1):
                if types[j] == 1:
                    d = p[:, i] - p[:, j]
                    out[:, i, j, :3] = w[:, j]
                    out[:, i, j, 3:] = np.cross(w[:, j], d)
                elif types[j] == 2:
                    out[:, i, j, 3:] = w[:, j]
        return out

    def sphere_centers(self, poses):
        n = poses.shape[0]
        if poses.dtype == np.float64:
            out = np.zeros((n, self.S, 3), np.float64)
            lib().or_sphere_centers_f64(C.byref(self.r), _c(poses, np.float64), n, out)
        else:
            out = np.zeros((n, self.S, 3), np.float32)
            lib().or_sphere_centers_f32(C.byref(self.r), _c(poses, np.float32), n, out)
        return out

    # ---- collision ----
    def check_states(self, q, nthreads=0):
        q = _c(np.asarray(q).reshape(-1, self.L), np.float32)
        n = q.shape[0]
        costs = np.zeros((4, n), np.float32)
        total = np.zeros(n, np.float32)
        lib().or_check_states(C.byref(self.r), C.byref(self.e), self.npairs, self.pairs, self.thr_sq,
                              q, n, costs.ctypes.data, total.ctypes.data, nthreads)
        return costs, total

    def clearance(self, q, nthreads=0):
        q = _c(np.asarray(q).reshape(-1, self.L), np.float64)
        out = np.zeros(q.shape[0], np.float64)
        lib().or_clearance_f64(C.byref(self.r), C.byref(self.e), self.npairs, self.pairs, q,
                               q.shape[0], out, nthreads)
        return out

    # ---- edges ----
    def edge_steps(self, f, t, res, rule=STEP_L2):
        f = _c(f, np.float32)
        t = _c(t, np.float32)
        d = np.zeros(self.L, np.float32)
        n = lib().or_edge_steps(f, t, self.L, res, rule, d, None)
        return n, d

    def edge_states(self, f, t, res, rule=STEP_L2):
        n, d = self.edge_steps(f, t, res, rule)
        out = np.zeros((n, self.L), np.float32)
        f = _c(f, np.float32)
        t = _c(t, np.float32)
        for k in range(n):
            lib().or_edge_state(f, t, d, self.L, n, k, out[k])
        return out

    def project(self, q, proj: Projection, nthreads=0):
        """Projected copies of q [n, L] and the final task-space / joint-limit costs."""
        rb = self.robot
        q = _c(np.asarray(q).reshape(-1, self.L), np.float32).copy()
        n = q.shape[0]
        tc = np.zeros(n, np.float32)
        bc = np.zeros(n, np.float32)
        lib().or_project(C.byref(self.r), _c(rb.active, np.uint8), _c(rb.lower, np.float32), _c(rb.upper, np.float32),
                         C.byref(proj), q, n, tc.ctypes.data, bc.ctypes.data, nthreads)
        return q, tc, bc

    def constrained_motions(self, q_from, q_to, proj: Projection, res, max_iters=10000, cap=0, nthreads=0):
        """Constrained motions (computeConstrainedMotions): ok [n], cost [n], recorded
        state counts [n] and, with cap > 0, the first cap recorded states [n, cap, L]."""
        rb = self.robot
        f = _c(np.asarray(q_from).reshape(-1, self.L), np.float32)
        t = _c(np.asarray(q_to).reshape(-1, self.L), np.float32)
        n = f.shape[0]
        ok = np.zeros(n, np.uint8)
        cost = np.zeros(n, np.float32)
        cnt = np.zeros(n, np.int32)
        st = np.zeros((n, max(cap, 1), self.L), np.float32)
        lib().or_constrained_motions(C.byref(self.r), C.byref(self.e), self.npairs, self.pairs, self.thr_sq,
                                     _c(rb.active, np.uint8), _c(rb.lower, np.float32), _c(rb.upper, np.float32),
                                     C.byref(proj), f, t, n, res, max_iters, ok, cost, cnt,
                                     st.ctypes.data if cap > 0 else None, cap, nthreads)
        return ok.astype(bool), cost, cnt, (st if cap > 0 else None)

    def check_motions(self, q_from, q_to, res, rule=STEP_L2, early_exit=True, nthreads=0):
        f = _c(np.asarray(q_from).reshape(-1, self.L), np.float32)
        t = _c(np.asarray(q_to).reshape(-1, self.L), np.float32)
        E = f.shape[0]
        ok = np.zeros(E, np.uint8)
        hit = np.zeros(E, np.int32)
        ns = np.zeros(E, np.int32)
        ln = np.zeros(E, np.float32)
        lib().or_check_motions(C.byref(self.r), C.byref(self.e), self.npairs, self.pairs, self.thr_sq,
                               f, t, E, res, rule, int(early_exit), ok, hit, ns, ln, nthreads)
        return ok.astype(bool), hit, ns, ln


def rrtc(model, start, goal, range_=0.1, res=0.01, rule=STEP_LINF, seed=0, max_nodes=200000,
         max_iters=200000, path_cap=65536):
    """Sequential RRT-Connect (one thread) with the planner's primitives."""
    rb = model.robot
    path = np.zeros((path_cap, model.L), np.float32)
    pl, it = C.c_int32(), C.c_int32()
    cost = C.c_float()
    sizes = np.zeros(2, np.int32)
    ok = lib().or_rrtc(C.byref(model.r), C.byref(model.e), model.npairs, model.pairs, model.thr_sq,
                       _c(start, np.float32), _c(goal, np.float32), _c(rb.active, np.uint8),
                       _c(rb.lower, np.float32), _c(rb.upper, np.float32), _c(rb.default, np.float32),
                       range_, res, rule, seed, max_nodes, max_iters, path, path_cap, C.byref(pl), C.byref(cost),
                       C.byref(it), sizes)
    return {"solved": int(ok), "path_len": pl.value, "cost": cost.value, "iterations": it.value,
            "tree_sizes": sizes.tolist()}, path[: pl.value].copy()


def rrtc_lanes(model, start, goal, lanes=64, range_=0.1, res=0.01, rule=STEP_LINF, seed=0, balance=3,
               tree_ratio=0.5, max_nodes=200000, max_iters=20000, path_cap=65536, nthreads=0):
    """Lane-parallel RRT-Connect in synchronous rounds: the device planner's per-lane rule
    (same Philox streams, balance rule, step rules), `lanes` lanes per round."""
    rb = model.robot
    path = np.zeros((path_cap, model.L), np.float32)
    pl, it = C.c_int32(), C.c_int32()
    cost = C.c_float()
    sizes = np.zeros(2, np.int32)
    ok = lib().or_rrtc_lanes(C.byref(model.r), C.byref(model.e), model.npairs, model.pairs, model.thr_sq,
                             _c(start, np.float32), _c(goal, np.float32), _c(rb.active, np.uint8),
                             _c(rb.lower, np.float32), _c(rb.upper, np.float32), _c(rb.default, np.float32),
                             range_, res, rule, seed, lanes, balance, tree_ratio, max_nodes, max_iters, path,
                             path_cap, C.byref(pl), C.byref(cost), C.byref(it), sizes, nthreads)
    return {"solved": int(ok), "path_len": pl.value, "cost": cost.value, "iterations": it.value,
            "tree_sizes": sizes.tolist()}, path[: pl.value].copy()


def balance_tree(balance, tree_ratio, lanes, n0, n1, h, cur):
    return lib().or_balance_tree(balance, tree_ratio, lanes, n0, n1, h, cur)


def nearest(tree, queries, active=None, cand=None, nthreads=0):
    tree = _c(tree, np.float32)
    queries = _c(queries, np.float32)
    M, J = tree.shape
    Q = queries.shape[0]
    out = np.zeros(Q, np.int32)
    act = _c(active, np.uint8) if active is not None else None
    cd = _c(cand, np.int32) if cand is not None else None
    lib().or_nearest(tree, M, J, act.ctypes.data if act is not None else None,
                     cd.ctypes.data if cd is not None else None, len(cd) if cd is not None else M,
                     queries, Q, out, nthreads)
    return out


def steer(q_from, q_to, max_distance):
    f = _c(q_from, np.float32)
    t = _c(q_to, np.float32).copy()
    lib().or_steer(f, t, f.shape[0], f.shape[1], max_distance)
    return t


def sample(robot, seed, offset, n):
    q = np.zeros((n, robot.num_links), np.float32)
    lib().or_sample(_c(robot.lower, np.float32), _c(robot.upper, np.float32), _c(robot.active, np.uint8),
                    _c(robot.default, np.float32), robot.num_links, seed, offset, n, q)
    return q


def num_threads():
    return lib().or_num_threads()
