"""Constraint projection (gbmp_project_states) against the oracle's restatement of
SingleArmSpace::projectStates with TaskSpaceConstraint and BoundaryConstraint.

The step of each iteration solves (J_a J_a^T + 1e-4 I) x = error, whose conditioning
(up to ~1e4) amplifies the last-bit differences of asinf / atan2f / sincosf between the GPU
and the host into joint differences along directions that hardly move the task frame.
(Moving the inputs by one ulp moves the oracle's own result by as much.)  Bars,
therefore: after one iteration, on every state whose step the oracle finds insensitive
to rounding (its result moves less than 1e-5 when the joints move by one ulp), the
projected joints equal the oracle's within 1e-4; after the reference's 10 iterations on
position targets both sides reach the region on the same states up to 6 % (borderline
states) and every state the GPU reports in the region is in it by the oracle's FP64 FK;
the joint-limit pull is bit-identical.  Also: the goal-region sampling flow of
SingleArmTask (sample, project, check) yields collision-free states in the region."""
import math

import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def arm():
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    return robot, api.Robot(robot), O.OracleModel(robot)


def _target(robot, seed):
    q0 = robot.sample_full(np.random.default_rng(seed), 1)
    tip = robot.num_links - 1
    T = W.fk_numpy(robot, q0)[0][tip]
    off = np.eye(4, dtype=np.float32)
    off[:3, :3] = T[:3, :3].T          # constrained frame with zero roll / pitch / yaw at q0
    return q0, tip, off, [float(T[0, 3]), float(T[1, 3]), float(T[2, 3]), 0.0, 0.0, 0.0]


def _frame_pos(m, q, tip, off):
    """Base-frame position of the constrained frame (FP64 FK of the oracle)."""
    P = m.fk(np.asarray(q, np.float64), f64=True)[:, tip].reshape(-1, 4, 4)
    return (P @ off.astype(np.float64))[:, :3, 3]


def _gpu(R, q, **kw):
    d = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    tc = torch.zeros(len(q), device="cuda")
    bc = torch.zeros(len(q), device="cuda")
    api.project_states(R, d, task_cost=tc, bound_cost=bc, **kw)
    torch.cuda.synchronize()
    return d.cpu().numpy(), tc.cpu().numpy(), bc.cpu().numpy()


def test_one_iteration_matches_oracle(arm):
    robot, R, m = arm
    q0, tip, off, ref = _target(robot, 3)
    rng = np.random.default_rng(4)
    q = (q0 + 0.1 * rng.standard_normal((2000, robot.num_links)) * robot.active).astype(np.float32)
    kw = dict(task_link=tip, offset=off, reference=ref, tolerance=(1e-3,) * 3 + (1e-2,) * 3, iterations=1)
    qg, tg, bg = _gpu(R, q, **kw)
    qo, to, bo = m.project(q, O.projection(**kw))
    act = robot.active.astype(bool)
    q_ulp = q.copy()
    q_ulp[:, act] = np.nextafter(q[:, act], np.float32(np.inf))
    qu, _, _ = m.project(q_ulp, O.projection(**kw))
    stable = np.abs(qu - qo).max(axis=1) < 1e-5
    assert stable.mean() > 0.8
    assert np.abs(qg[stable] - qo[stable]).max() < 1e-4
    np.testing.assert_allclose(tg[stable], to[stable], atol=1e-4)


def test_position_targets_reach_the_region_like_the_oracle(arm):
    robot, R, m = arm
    q0, tip, off, ref = _target(robot, 5)
    rng = np.random.default_rng(6)
    q = (q0 + 0.15 * rng.standard_normal((2000, robot.num_links)) * robot.active).astype(np.float32)
    kw = dict(task_link=tip, offset=off, reference=ref, tolerance=(1e-3,) * 3 + (2 * math.pi,) * 3,
              use_boundary=False, iterations=10)
    qg, tg, _ = _gpu(R, q, **kw)
    qo, to, _ = m.project(q, O.projection(**kw))
    reached_g, reached_o = tg == 0, to == 0
    assert reached_o.mean() > 0.5
    assert np.mean(reached_g != reached_o) <= 0.06
    # the GPU's reached states really are in the region (checked by the oracle's FK)
    pos = _frame_pos(m, qg[reached_g], tip, off)
    assert np.abs(pos - np.asarray(ref[:3])).max() < 1e-3 + 2e-4


def test_joint_limit_pull_is_exact(arm):
    robot, R, m = arm
    rng = np.random.default_rng(8)
    q = robot.sample_full(rng, 1000)
    act = robot.active.astype(bool)
    q[:, act] += rng.uniform(-1.0, 1.0, size=(1000, act.sum())).astype(np.float32)
    kw = dict(task_link=-1, use_boundary=True, iterations=1)
    qg, tg, bg = _gpu(R, q, **kw)
    qo, to, bo = m.project(q, O.projection(**kw))
    np.testing.assert_array_equal(qg, qo)
    np.testing.assert_array_equal(bg, bo)
    assert np.all(bg == 0)


def test_goal_region_sampling_flow(arm):
    """SingleArmTask's goal-region constructor (SingleArmTask.cpp:12-39): sample, project,
    keep the feasible states."""
    robot, R, m = arm
    env = W.random_env(11, 24, 4, 2, oriented=True)
    E = api.Env(env)
    q0, tip, off, ref = _target(robot, 9)
    n = 4096
    d = torch.zeros((n, robot.num_links), device="cuda")
    api.sample(R, 77, 0, d)
    tc = torch.zeros(n, device="cuda")
    bc = torch.zeros(n, device="cuda")
    api.project_states(R, d, task_link=tip, offset=off, reference=ref, tolerance=(0.02,) * 3 + (2 * math.pi,) * 3,
                       iterations=10, task_cost=tc, bound_cost=bc)
    v = torch.zeros(n, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, d, verdict=v)
    torch.cuda.synchronize()
    good = ((tc == 0) & (bc == 0) & (v == 0)).cpu().numpy()
    assert good.sum() > 20
    q = d.cpu().numpy()[good]
    cl = O.OracleModel(robot, env).clearance(q)
    assert np.all(cl > -1e-4)
    pos = _frame_pos(m, q, tip, off)
    assert np.abs(pos - np.asarray(ref[:3])).max() < 0.02 + 2e-4


def test_projection_arguments(arm):
    robot, R, m = arm
    d = torch.zeros((4, robot.num_links), device="cuda")
    with pytest.raises(_lib.GbmpError):
        api.project_states(R, d, task_link=robot.num_links)
    with pytest.raises(_lib.GbmpError):
        api.project_states(R, d, iterations=-1)
    api.project_states(R, d[:0], task_link=0)   # nothing to do
