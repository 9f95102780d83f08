"""CPU tests of the oracle (the checker) and of the synthetic workloads.

The oracle is pinned here against independent float64 implementations and, where
oracle/_ref has been built from the reference tree, against the reference's own
generated kernels (tests/test_reference_pin.py)."""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import workloads as W


@pytest.fixture(scope="module")
def arm7():
    robot, env, q = W.plain_check_workload(n=512)
    return robot, env, q, O.OracleModel(robot, env)


@pytest.fixture(scope="module")
def arm8():
    robot, env, qf, qt = W.edge_workload(n_edges=64)
    return robot, env, qf, qt, O.OracleModel(robot, env)


def test_workloads_are_deterministic():
    a = W.plain_check_workload(seed=3, n=16)
    b = W.plain_check_workload(seed=3, n=16)
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_array_equal(a[0].joint_poses, b[0].joint_poses)
    np.testing.assert_array_equal(a[1].sphere_pos, b[1].sphere_pos)


def test_workload_shapes():
    robot, env, q = W.plain_check_workload(n=8)
    assert robot.num_links == 8 and robot.num_spheres == 59 and robot.dim == 7
    assert env.counts == (32, 8, 0)
    robot2, env2, qf, qt = W.edge_workload(n_edges=8)
    assert robot2.num_links == 9 and robot2.num_spheres == 110 and robot2.dim == 8
    assert robot2.joint_types[1] == W.PRISMATIC
    assert env2.counts == (256, 64, 16)
    assert np.all((qf >= robot2.lower) & (qf <= robot2.upper))


def test_fk_f32_matches_f64(arm7):
    robot, env, q, m = arm7
    p32 = m.fk(q)
    p64 = m.fk(q.astype(np.float64), f64=True)
    assert np.abs(p32 - p64).max() < 1e-5
    # last row of every pose is (0, 0, 0, 1) (KernelGenerator.h:275)
    np.testing.assert_array_equal(p32[:, :, 12:], np.tile([0, 0, 0, 1], (q.shape[0], robot.num_links, 1)))


def test_fk_f64_matches_independent_numpy(arm7, arm8):
    for robot, q, m in ((arm7[0], arm7[2], arm7[3]), (arm8[0], arm8[2], arm8[4])):
        p64 = m.fk(q.astype(np.float64), f64=True).reshape(-1, robot.num_links, 4, 4)
        ref = W.fk_numpy(robot, q)
        assert np.abs(p64 - ref).max() < 1e-6


def test_sphere_centers_match_numpy(arm8):
    robot, env, qf, qt, m = arm8
    c = m.sphere_centers(m.fk(qf.astype(np.float64), f64=True))
    np.testing.assert_allclose(c, W.sphere_centers_numpy(robot, qf), atol=1e-9)


def test_self_pairs_follow_reference_rule(arm7):
    robot, env, q, m = arm7
    pairs = m.pairs.reshape(-1, 2)
    assert np.all(pairs[:, 0] < pairs[:, 1])
    li, lj = robot.sphere_link[pairs[:, 0]], robot.sphere_link[pairs[:, 1]]
    assert np.all(li != lj)
    assert np.all(robot.enables[li, lj] == 1)
    s = robot.sphere_r[pairs[:, 0]] + robot.sphere_r[pairs[:, 1]]
    np.testing.assert_array_equal(m.thr_sq, (s * s).astype(np.float32))
    # count every admissible pair exactly once
    S = robot.num_spheres
    expect = sum(1 for i in range(S) for j in range(i + 1, S)
                 if robot.sphere_link[i] != robot.sphere_link[j]
                 and robot.enables[robot.sphere_link[i], robot.sphere_link[j]])
    assert m.npairs == expect


def test_costs_agree_with_clearance(arm7, arm8):
    for robot, q, m in ((arm7[0], arm7[2], arm7[3]), (arm8[0], arm8[2], arm8[4])):
        costs, total = m.check_states(q)
        cl = m.clearance(q)
        clear = np.abs(cl) > 1e-4
        np.testing.assert_array_equal((total > 0)[clear], (cl < 0)[clear])
        np.testing.assert_allclose(total, costs.sum(0), rtol=1e-6, atol=1e-7)
        assert (total > 0).any() and (total == 0).any()


def test_cost_terms_by_hand():
    """One sphere on link 1 against one obstacle of each kind, checked by hand."""
    robot = W.serial_arm(11, dof=1, n_spheres=1)
    robot.sphere_pos[:] = 0.0
    robot.sphere_r[:] = 0.1
    robot.joint_poses[1] = np.eye(4, dtype=np.float32)
    e = W.Environment.empty()
    e.sphere_pos = np.array([[0.15, 0, 0]], np.float32)
    e.sphere_r = np.array([0.1], np.float32)
    e.box_pos = np.array([[0, 0.17, 0]], np.float32)
    e.box_rot = np.eye(3, dtype=np.float32)[None]
    e.box_min = np.array([[-0.1, -0.1, -0.1]], np.float32)
    e.box_max = np.array([[0.1, 0.1, 0.1]], np.float32)
    e.cyl_pos = np.array([[0, 0, -0.35]], np.float32)
    e.cyl_rot = np.eye(3, dtype=np.float32)[None]
    e.cyl_radius = np.array([0.05], np.float32)
    e.cyl_height = np.array([0.5], np.float32)
    m = O.OracleModel(robot, e)
    costs, total = m.check_states(np.zeros((1, robot.num_links), np.float32))
    assert costs[1, 0] == pytest.approx(0.05, abs=1e-6)      # 0.2 - 0.15
    assert costs[2, 0] == pytest.approx(0.03, abs=1e-6)      # r - (0.17 - 0.1)
    assert costs[3, 0] == pytest.approx(0.0, abs=1e-7)       # cylinder top at z = -0.1: touching
    assert costs[0, 0] == 0.0


def test_edge_steps_reference_rule():
    J = 4
    f = np.zeros(J, np.float32)
    t = np.array([0.3, 0.4, 0, 0], np.float32)            # |d| = 0.5
    m = O.OracleModel(W.serial_arm(5, dof=3, n_spheres=3))
    n, d = m.edge_steps(f, t, 0.1, O.STEP_L2)
    assert n == int(np.float32(0.5) / np.float32(0.1)) + 1
    st = m.edge_states(f, t, 0.1, O.STEP_L2)
    np.testing.assert_array_equal(st[0], f)
    np.testing.assert_array_equal(st[-1], t)
    n2, _ = m.edge_steps(f, t, 0.1, O.STEP_LINF)
    assert n2 == int(np.float32(0.4) / np.float32(0.1)) + 1
    # single-step edge: only the goal state is checked (KernelGenerator.h:508-516)
    n3, _ = m.edge_steps(f, f + np.float32(1e-3), 0.1, O.STEP_L2)
    assert n3 == 1
    np.testing.assert_array_equal(m.edge_states(f, f + np.float32(1e-3), 0.1)[0], f + np.float32(1e-3))


def test_check_motions_early_exit_same_outputs(arm8):
    robot, env, qf, qt, m = arm8
    a = m.check_motions(qf[:16], qt[:16], 0.05, O.STEP_LINF, early_exit=True)
    b = m.check_motions(qf[:16], qt[:16], 0.05, O.STEP_LINF, early_exit=False)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    ok, hit, ns, ln = a
    assert np.all(ok == (hit < 0))
    np.testing.assert_allclose(ln, np.linalg.norm(qt[:16] - qf[:16], axis=1), rtol=1e-5)


def test_nearest_matches_bruteforce():
    rng = np.random.default_rng(0)
    tree = rng.random((1000, 8), dtype=np.float32)
    qs = rng.random((50, 8), dtype=np.float32)
    act = np.ones(8, np.uint8)
    act[0] = 0
    out = O.nearest(tree, qs, active=act)
    d = ((qs[:, None, 1:] - tree[None, :, 1:]) ** 2).sum(-1)
    np.testing.assert_array_equal(out, d.argmin(1))
    cand = rng.choice(1000, 100, replace=False).astype(np.int32)
    out2 = O.nearest(tree, qs, active=act, cand=cand)
    np.testing.assert_array_equal(out2, cand[d[:, cand].argmin(1)])


def test_steer_limits_distance():
    rng = np.random.default_rng(1)
    f = rng.random((20, 5), dtype=np.float32)
    t = f + rng.normal(size=(20, 5)).astype(np.float32)
    out = O.steer(f, t, 0.3)
    d_in = np.linalg.norm(t - f, axis=1)
    d_out = np.linalg.norm(out - f, axis=1)
    assert np.all(d_out <= 0.3 + 1e-5)
    np.testing.assert_array_equal(out[d_in <= 0.3], t[d_in <= 0.3])


def test_sampler_in_limits_and_reproducible():
    robot = W.edge_workload(n_edges=1)[0]
    a = O.sample(robot, 123, 0, 1000)
    b = O.sample(robot, 123, 500, 500)
    np.testing.assert_array_equal(a[500:], b)
    assert np.all(a >= robot.lower) and np.all(a <= robot.upper)
    np.testing.assert_array_equal(a[:, 0], robot.default[0])
    # uniformity (loose): mean of the unit-range coordinate
    u = (a[:, 2] - robot.lower[2]) / (robot.upper[2] - robot.lower[2])
    assert abs(u.mean() - 0.5) < 0.05


def test_projection_restatement_converges_where_the_method_is_consistent():
    """The projection restatement (SingleArmSpace.cu:1631-1662) reaches position targets
    and zero-orientation frame targets from nearby states; with a general target
    orientation the reference's Euler-angle error does not act as an angular error and the
    iteration does not converge (a property of the reference method, kept as is)."""
    import math
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    m = O.OracleModel(robot)
    rng = np.random.default_rng(0)
    q0 = robot.sample_full(rng, 1)
    tip = robot.num_links - 1
    T = W.fk_numpy(robot, q0)[0][tip]
    near = (q0 + 0.01 * rng.standard_normal((100, robot.num_links)) * robot.active).astype(np.float32)
    pos_only = O.projection(task_link=tip, reference=[T[0, 3], T[1, 3], T[2, 3], 0, 0, 0],
                            tolerance=(1e-3,) * 3 + (2 * math.pi,) * 3, use_boundary=False)
    assert (m.project(near, pos_only)[1] == 0).all()
    off = np.eye(4, dtype=np.float32)
    off[:3, :3] = T[:3, :3].T
    full = O.projection(task_link=tip, offset=off, reference=[T[0, 3], T[1, 3], T[2, 3], 0, 0, 0],
                        tolerance=(1e-3,) * 3 + (1e-2,) * 3, use_boundary=False)
    assert (m.project(near, full)[1] == 0).all()
    rpy = [math.atan2(T[2, 1], T[2, 2]), math.asin(-T[2, 0]), math.atan2(T[1, 0], T[0, 0])]
    general = O.projection(task_link=tip, reference=[T[0, 3], T[1, 3], T[2, 3]] + rpy,
                           tolerance=(1e-3,) * 3 + (1e-2,) * 3, use_boundary=False)
    assert (m.project(near, general)[1] == 0).mean() < 0.5


def test_count_rule_steps():
    """pRRTC's granularity rule (pRRTC.cu:430-440): G equal steps whatever the edge
    length, G + 1 states from the start to the end."""
    robot = W.edge_workload(n_edges=1)[0]
    m = O.OracleModel(robot)
    q = robot.sample_full(np.random.default_rng(1), 2)
    for G in (1, 5, 64):
        n, d = m.edge_steps(q[0], q[1], G, O.STEP_COUNT)
        assert n == G + 1
        st = m.edge_states(q[0], q[1], G, O.STEP_COUNT)
        np.testing.assert_array_equal(st[0], q[0])
        np.testing.assert_array_equal(st[-1], q[1])
        k = min(2, G - 1)
        np.testing.assert_allclose(st[k], q[0] + k * (q[1] - q[0]) / G, atol=1e-6)


def test_balance_rule_follows_prrtc():
    """The oracle's tree choice (pRRTC.cu:348-371): half the lanes per tree at a lane's
    first iteration and with balancing off; strategy 1 proportional while the trees are
    within 1.5 x lanes nodes, else the smaller tree by tree_ratio; strategy 2 swaps
    while the relative size difference is below tree_ratio."""
    assert O.balance_tree(1, 0.5, 64, 10, 500, 0.3, -1) == 0
    assert O.balance_tree(1, 0.5, 64, 10, 500, 0.7, -1) == 1
    assert O.balance_tree(0, 0.5, 64, 10, 500, 0.7, 0) == 1
    # strategy 1, trees within 1.5 x 64 nodes: tree 0 below 1 - n0 / (n0 + n1) = 0.6
    assert O.balance_tree(1, 0.5, 64, 40, 60, 0.59, 1) == 0
    assert O.balance_tree(1, 0.5, 64, 40, 60, 0.61, 0) == 1
    # strategy 1, far apart: every lane grows the smaller tree
    assert O.balance_tree(1, 0.5, 64, 100, 900, 0.99, 1) == 0
    assert O.balance_tree(1, 0.5, 64, 900, 100, 0.01, 0) == 1
    # strategy 2: swap while |nt - no| / nt < tree_ratio
    assert O.balance_tree(2, 1.0, 64, 100, 90, 0.2, 0) == 1
    assert O.balance_tree(2, 0.05, 64, 100, 90, 0.2, 0) == 0
    # proportional at every size (the device default)
    assert O.balance_tree(3, 0.5, 64, 100, 900, 0.89, 1) == 0
    assert O.balance_tree(3, 0.5, 64, 100, 900, 0.91, 0) == 1
    # a lane on the large tree swaps to the small one; a lane on the small tree stays
    assert O.balance_tree(2, 1.0, 64, 1000, 10, 0.2, 0) == 1
    assert O.balance_tree(2, 1.0, 64, 1000, 10, 0.2, 1) == 1


def test_lane_parallel_rrtc_is_valid_and_thread_independent():
    """The lane-parallel restatement returns collision-free paths from start to goal, and
    the same result whatever the number of threads (commits keep lane order)."""
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    env = W.shelf_env(2)
    m = O.OracleModel(robot, env)
    _, _, fs = W.planning_workload(2, lambda q: m.check_states(q)[1] == 0, robot=robot, env=env)
    s0, g0 = W.pick_problem(fs, lambda a, b: bool(m.check_motions(a[None], b[None], 0.01, 1)[0][0]), 2)
    a = O.rrtc_lanes(m, s0, g0, lanes=16, seed=7, nthreads=1)
    b = O.rrtc_lanes(m, s0, g0, lanes=16, seed=7, nthreads=4)
    assert a[0]["solved"] and a[0] == b[0]
    np.testing.assert_array_equal(a[1], b[1])
    path = a[1]
    np.testing.assert_array_equal(path[0], s0)
    np.testing.assert_array_equal(path[-1], g0)
    assert m.check_motions(path[:-1], path[1:], 0.01, 1)[0].all()
