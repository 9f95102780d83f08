"""Parallel RRT-Connect on the GPU: every returned path is re-validated by the oracle's
checkMotions restatement, and every stop condition (deadline, node cap) ends the launch
with a status instead of a hang."""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RES, RULE = 0.01, _lib.STEP_LINF


@pytest.fixture(scope="module")
def scene():
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    env = W.shelf_env(0)
    m = O.OracleModel(robot, env)
    checker = lambda q: m.check_states(q)[1] == 0
    edge_free = lambda a, b: bool(m.check_motions(a[None], b[None], RES, RULE)[0][0])
    robot, env, free = W.planning_workload(0, checker, robot=robot, env=env)
    R, E = api.Robot(robot), api.Env(env)
    return robot, env, m, free, edge_free, R, E


def _validate_path(m, path, start, goal):
    np.testing.assert_array_equal(path[0], start)
    np.testing.assert_array_equal(path[-1], goal)
    ok, fh, ns, ln = m.check_motions(path[:-1], path[1:], RES, RULE)
    for k in np.nonzero(~ok)[0]:
        st = m.edge_states(path[k], path[k + 1], RES, RULE)
        cl = m.clearance(st[: fh[k] + 1])
        assert np.any(np.abs(cl) <= 1e-4), f"edge {k} collides at state {fh[k]}"
    return ln


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_rrtc_paths_are_valid(scene, seed):
    robot, env, m, free, edge_free, R, E = scene
    start, goal = W.pick_problem(free, edge_free, seed)
    planner = api.Planner(R, max_nodes=200_000, path_cap=8192)
    res, path = planner.solve(E, start, goal, lanes=512, range_=0.1, resolution=RES, rule=RULE, seed=seed,
                              time_limit_s=20.0)
    assert res["solved"] == 1, res
    assert res["path_len"] == len(path) >= 2
    ln = _validate_path(m, path, start, goal)
    act = robot.active.astype(bool)
    seg = np.linalg.norm(np.diff(path[:, act], axis=0), axis=1)
    assert np.all(seg <= 0.1 + 1e-5)
    assert res["cost"] == pytest.approx(float(seg.sum()), rel=1e-4)


def test_rrtc_deadline_returns_timeout(scene):
    robot, env, m, free, edge_free, R, E = scene
    # goal in collision: no path exists; the device deadline must end the launch
    goal = free[0].copy()
    bad = None
    rng = np.random.default_rng(0)
    for _ in range(100):
        q = robot.sample_full(rng, 256)
        c = m.check_states(q)[1] > 0
        if c.any():
            bad = q[np.argmax(c)]
            break
    assert bad is not None
    planner = api.Planner(R, max_nodes=500_000, path_cap=1024)
    res, path = planner.solve(E, goal, bad, lanes=256, max_iters=10**9, time_limit_s=0.3, resolution=RES, rule=RULE)
    assert res["solved"] == 0 and res["status"] == 4 and res["status_code"] == 6
    assert len(path) == 0


def test_rrtc_node_cap(scene):
    robot, env, m, free, edge_free, R, E = scene
    start, goal = W.pick_problem(free, edge_free, 0)
    planner = api.Planner(R, max_nodes=16, path_cap=1024)
    res, path = planner.solve(E, start, goal, lanes=64, time_limit_s=5.0, resolution=RES, rule=RULE)
    if not res["solved"]:
        assert res["status"] == 2 and res["status_code"] == 7
        assert res["start_tree_size"] <= 16 and res["goal_tree_size"] <= 16


def test_rrtc_count_rule_several_goals(scene):
    """pRRTC's form of a solve: several goals (each a root of the goal tree) and edges
    checked at a fixed count of equal steps.  The path ends at one of the goals and every
    state the planner checked on it is collision-free by the oracle."""
    robot, env, m, free, edge_free, R, E = scene
    start, g0 = W.pick_problem(free, edge_free, 4)
    goals = np.stack([g0, free[5], free[9]])
    G = 8
    planner = api.Planner(R, max_nodes=200_000, path_cap=8192)
    res, path = planner.solve(E, start, goals, lanes=512, range_=0.1, resolution=G, rule=_lib.STEP_COUNT, seed=4,
                              time_limit_s=20.0)
    assert res["solved"] == 1, res
    np.testing.assert_array_equal(path[0], start)
    assert any(np.array_equal(path[-1], g) for g in goals)
    states = np.concatenate([m.edge_states(a, b, G, O.STEP_COUNT)[1:] for a, b in zip(path[:-1], path[1:])])
    assert np.all(m.clearance(states) > -1e-4)
    with pytest.raises(_lib.GbmpError):
        planner.solve(E, start, goals, resolution=0.5, rule=_lib.STEP_COUNT)


def test_rrtc_many_goals_then_one(scene):
    """More goals than the solve stages in its pinned input block (64): the rest are
    copied into the goal tree after the reset.  The path ends at one of the goals, every
    goal is a root (the goal tree holds at least all of them), and a following one-goal
    solve on the same planner finds none of the earlier goal rows left."""
    robot, env, m, free, edge_free, R, E = scene
    start, g0 = W.pick_problem(free, edge_free, 5)
    others = [q for q in free if not np.array_equal(q, start)]
    goals = np.stack([g0] + [others[i % len(others)] for i in range(99)])
    planner = api.Planner(R, max_nodes=100_000, path_cap=8192)
    res, path = planner.solve(E, start, goals, lanes=512, range_=0.1, resolution=RES, rule=RULE, seed=6,
                              time_limit_s=20.0)
    assert res["solved"] == 1, res
    assert res["goal_tree_size"] >= len(goals)
    np.testing.assert_array_equal(path[0], start)
    assert any(np.array_equal(path[-1], g) for g in goals)
    _validate_path(m, path, start, path[-1])
    res, path = planner.solve(E, start, g0, lanes=512, range_=0.1, resolution=RES, rule=RULE, seed=7,
                              time_limit_s=20.0)
    assert res["solved"] == 1, res
    _validate_path(m, path, start, g0)


def test_rrtc_dynamic_domain_paths_are_valid(scene):
    """pRRTC's dynamic domain (samples beyond a node's radius skipped, radii set, shrunk
    and grown as extensions fail and succeed) changes which samples are used, not what a
    valid path is; bad parameters are argument errors."""
    robot, env, m, free, edge_free, R, E = scene
    start, goal = W.pick_problem(free, edge_free, 1)
    planner = api.Planner(R, max_nodes=200_000, path_cap=8192)
    for dd_radius in (4.0, 0.3):
        res, path = planner.solve(E, start, goal, lanes=512, range_=0.1, resolution=RES, rule=RULE, seed=1,
                                  time_limit_s=20.0, dynamic_domain=True, dd_alpha=1e-3, dd_radius=dd_radius,
                                  dd_min_radius=0.2)
        assert res["solved"] == 1, res
        _validate_path(m, path, start, goal)
    with pytest.raises(_lib.GbmpError):
        planner.solve(E, start, goal, resolution=RES, rule=RULE, dynamic_domain=True, dd_alpha=1.5)
