"""The C++ facade include/gbmp_cudampl.hpp (CUDAMPLib::SingleArmSpace / SingleArmStates /
SingleArmStateManager and CPRRTC::RobotSolver over the C-ABI) and its RRG planner
(include/gbmp_cudampl_rrg.hpp) compile against gbmp.h and libgbmp, and a C++ program
driving them the way the reference's callers do gives the oracle's results: collision
verdicts and per-constraint costs, link poses, motion feasibility and costs, samples,
nearest neighbours, and RobotSolver and RRG paths that the oracle re-validates."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from isaac_sim_ros2_humble_gb300 import _lib, workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "cudampl_facade_check.cpp")
RES = 0.02
BAND = 1e-4


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "include", "cuda_runtime.h")):
            return c
    return None


def build_facade_check(out_dir):
    cuda = _cuda_home()
    if cuda is None or shutil.which("g++") is None:
        pytest.skip("no g++ or CUDA headers")
    _lib.load()   # builds libgbmp when it is missing
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = os.path.join(str(out_dir), "cudampl_facade_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), SRC, "-o", exe, "-L", libdir, "-lgbmp",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{libdir}",
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles_and_links(tmp_path):
    exe = build_facade_check(tmp_path)
    assert os.access(exe, os.X_OK)


def _write_problem(path, robot, env, states, e_from, e_to, queries, start, goal, shelf, region):
    L = robot.num_links
    f = lambda a: " ".join("%.9g" % v for v in np.asarray(a, np.float32).ravel())
    i = lambda a: " ".join(str(int(v)) for v in np.asarray(a).ravel())
    act = robot.active.astype(bool)
    lines = [f"{L} {robot.dim} {robot.num_spheres}", i(robot.joint_types), f(robot.joint_poses),
             f(robot.joint_axes), i(robot.parent), i(robot.sphere_link), f(robot.sphere_pos), f(robot.sphere_r),
             i(robot.active), f(robot.lower), f(robot.upper), f(robot.default), i(robot.enables), "%.9g" % RES,
             str(len(env.sphere_r)), f(env.sphere_pos), f(env.sphere_r),
             str(len(env.box_pos)), f(env.box_pos), f(env.box_rot), f(env.box_min), f(env.box_max),
             str(len(env.cyl_radius)), f(env.cyl_pos), f(env.cyl_rot), f(env.cyl_radius), f(env.cyl_height),
             str(len(states)), f(states[:, act]), str(len(e_from)), f(e_from[:, act]), f(e_to[:, act]),
             str(len(queries)), f(queries[:, act]), f(start[act]), f(goal[act]),
             str(len(shelf.box_pos)), f(shelf.box_pos), f(shelf.box_min), f(shelf.box_max),
             str(region[0]), f(region[1]), f(region[2])]
    with open(path, "w") as fp:
        fp.write("\n".join(lines) + "\n")


def _read_results(path):
    out = {}
    with open(path) as fp:
        rows = fp.read().split("\n")
    k = 0
    while k + 1 < len(rows) and rows[k]:
        name, n = rows[k].split()
        vals = rows[k + 1].split()
        assert len(vals) == int(n), name
        out[name] = np.array([float(v) for v in vals], np.float64)
        k += 2
    return out


@pytest.mark.gpu
def test_facade_matches_oracle(tmp_path):
    import oracle as O
    import torch
    from isaac_sim_ros2_humble_gb300 import api
    exe = build_facade_check(tmp_path)
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    env = W.random_env(21, 64, 16, 4, oriented=True)
    shelf = W.shelf_env(0)
    rng = np.random.default_rng(5)
    states = robot.sample_full(rng, 512)
    e_from, e_to = robot.sample_full(rng, 256), robot.sample_full(rng, 256)
    queries = robot.sample_full(rng, 64)
    ms = O.OracleModel(robot, shelf)
    checker = lambda q: ms.check_states(q)[1] == 0
    edge_free = lambda a, b: bool(ms.check_motions(a[None], b[None], RES, 0)[0][0])
    _, _, free = W.planning_workload(0, checker, robot=robot, env=shelf)
    start, goal = W.pick_problem(free, edge_free, 0)
    # goal region: the last link's origin within 5 cm of where a free state puts it
    tip = robot.num_links - 1
    free_q = states[O.OracleModel(robot, env).check_states(states)[1] == 0][0]
    tip_pos = W.fk_numpy(robot, free_q[None])[0][tip][:3, 3]
    region = (tip, [*tip_pos, 0.0, 0.0, 0.0], [0.05, 0.05, 0.05, 7.0, 7.0, 7.0])
    prob, resf = tmp_path / "problem.txt", tmp_path / "results.txt"
    _write_problem(prob, robot, env, states, e_from, e_to, queries, start, goal, shelf, region)
    r = subprocess.run([exe, str(prob), str(resf)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = _read_results(resf)
    L, n, act = robot.num_links, len(states), robot.active.astype(bool)

    m = O.OracleModel(robot, env)
    oc, ot = m.check_states(states)
    cl = m.clearance(states)
    clear = np.abs(cl) > BAND
    feas = got["feasible"].astype(bool)
    assert feas.any() and not feas.all()
    np.testing.assert_array_equal(feas[clear], (ot == 0)[clear])
    np.testing.assert_allclose(got["total"], ot, rtol=1e-4, atol=2e-5)
    np.testing.assert_allclose(got["costs"].reshape(n, 4), oc.T, rtol=1e-4, atol=2e-5)
    p64 = m.fk(states.astype(np.float64), f64=True)
    assert np.abs(got["poses"].reshape(n, L, 16) - p64).max() < 1e-5
    jac = m.space_jacobian(states)[:, L - 1]          # [n, joints, 6]
    assert np.abs(got["jacobian_last"].reshape(n, L, 6) - jac).max() < 2e-5

    o_ok, o_fh, o_ns, o_ln = m.check_motions(e_from, e_to, RES, 0)
    ok = got["motion_ok"].astype(bool)
    for k in np.nonzero(ok != o_ok)[0]:
        st = m.edge_states(e_from[k], e_to[k], RES, 0)
        assert np.any(np.abs(m.clearance(st)) <= BAND), f"edge {k} differs outside the clearance band"
    np.testing.assert_array_equal(got["motion_cost"].astype(np.float32), o_ln)

    np.testing.assert_array_equal(got["sample"].astype(np.float32).reshape(64, L), O.sample(robot, 0x5EED, 0, 64))
    np.testing.assert_array_equal(got["nearest"].astype(np.int32), O.nearest(states, queries, active=robot.active))
    assert int(got["gather_ok"][0]) == 1   # get_states rows equal the stored rows bit for bit

    path = got["path"].astype(np.float32).reshape(-1, robot.dim)
    assert len(path) >= 2
    _check_path(ms, robot, path, start, goal)

    # RRG over the shelf space: a dense path, waypoints interpolated with the reference's
    # rule (util.cpp:205-248: floor(d / res) steps, so spacing in [res, 2 res), and each
    # segment ends on its waypoint again)
    rrg = got["rrg_path"].astype(np.float32).reshape(-1, robot.dim)
    assert len(rrg) >= 2 and got["rrg_vertices"][0] > 4
    _check_path(ms, robot, rrg, start, goal)
    assert np.all(np.linalg.norm(np.diff(rrg, axis=0), axis=1) < 2 * RES)

    # goal-region states: in the region, inside the limits, collision-free (oracle)
    goals = got["region_goals"].astype(np.float32).reshape(-1, robot.dim)
    assert len(goals) >= 1
    full_g = robot.full_from_active(goals)
    pos = m.fk(full_g.astype(np.float64), f64=True)[:, tip].reshape(-1, 4, 4)[:, :3, 3]
    assert np.abs(pos - np.asarray(region[1][:3])).max() < 0.05 + 2e-4
    assert np.all(full_g[:, act] >= robot.lower[act] - 1e-6) and np.all(full_g[:, act] <= robot.upper[act] + 1e-6)
    assert np.all(m.clearance(full_g) > -BAND)

    # constrained motions between region goals: the facade's verdicts and lengths are the
    # C-ABI's (same kernel); the path through three goals stays in the region and the
    # limits, is collision-free and moves at most 5 x resolution a state within a motion
    nm = len(got.get("region_motion_ok", []))
    if nm:
        full_a, full_b = full_g[:nm], full_g[1:nm + 1]
        R, E = api.Robot(robot), api.Env(env)
        region_kw = dict(task_link=region[0], reference=region[1], tolerance=region[2], use_boundary=True)
        okc = torch.zeros(nm, dtype=torch.uint8, device="cuda")
        costc = torch.zeros(nm, device="cuda")
        api.constrained_motions(R, E, torch.from_numpy(full_a.copy()).cuda(), torch.from_numpy(full_b.copy()).cuda(),
                                resolution=RES, ok=okc, cost=costc, **region_kw)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(got["region_motion_ok"].astype(bool), okc.cpu().numpy().astype(bool))
        np.testing.assert_array_equal(got["region_motion_cost"].astype(np.float32), costc.cpu().numpy())
        rp = got["region_path"].astype(np.float32).reshape(-1, robot.dim)
        if len(rp):
            full_p = robot.full_from_active(rp)
            _, tc, bc = m.project(full_p, O.projection(iterations=0, **region_kw))
            assert (tc == 0).all() and (bc == 0).all()
            assert (m.check_states(full_p)[1] == 0).all()
            assert np.linalg.norm(np.diff(full_p, axis=0), axis=1).max() <= 6 * RES * (1 + 1e-5)


def _check_path(ms, robot, path, start, goal):
    act = robot.active.astype(bool)
    np.testing.assert_array_equal(path[0], start[act])
    np.testing.assert_array_equal(path[-1], goal[act])
    full = robot.full_from_active(path)
    p_ok, p_fh, _, _ = ms.check_motions(full[:-1], full[1:], RES, 0)
    for k in np.nonzero(~p_ok)[0]:
        st = ms.edge_states(full[k], full[k + 1], RES, 0)
        assert np.any(np.abs(ms.clearance(st[: p_fh[k] + 1])) <= BAND), f"path edge {k} collides"
