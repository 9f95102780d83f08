"""Constrained motions (gbmp_constrained_motions) against the oracle's restatement of
SingleArmSpace::computeConstrainedMotions (SingleArmSpace.cu:1049-1366).

Workload: the 7-DOF arm holding its tip at a fixed height (task-space region: z within
1 cm, x, y and orientation free) plus the joint limits, in a scene of 24 spheres, 6
oriented boxes and 3 cylinders; 200 motions between collision-free states in the region.

Each iteration of a motion runs two projection passes whose damped 6x6 solve amplifies
last-bit differences of asinf / atan2f / sincosf between the GPU and the host (the
projection tests show the oracle's own one-ulp response), so the bars are: feasibility
verdicts equal on at least 95 % of the motions; on motions feasible on both sides, the
recorded state counts equal on at least 90 % and within 2 everywhere, and where they are
equal, states within 1e-3 and lengths within 1e-3 relative.  And the bar that does not
depend on rounding: every motion the GPU reports feasible is re-validated by the oracle
(every recorded state collision-free in FP32 cost mode, in the region and the limits,
consecutive states at most 5 x resolution apart, the last within resolution of the
goal)."""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RES = 0.02
CAP = 1024


@pytest.fixture(scope="module")
def case():
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    env = W.random_env(7, 24, 6, 3, oriented=True)
    m = O.OracleModel(robot, env)
    tip = robot.num_links - 1
    rng = np.random.default_rng(0)
    q0 = robot.sample_full(rng, 1)
    T = W.fk_numpy(robot, q0)[0][tip]
    region = dict(task_link=tip, reference=[0.0, 0.0, float(T[2, 3]), 0.0, 0.0, 0.0],
                  tolerance=[10.0, 10.0, 0.01, 10.0, 10.0, 10.0], use_boundary=True)
    proj = O.projection(iterations=10, **region)
    q = q0 + 0.6 * (robot.sample_full(rng, 4000) - q0)
    qp, tc, bc = m.project(q, proj)
    good = qp[(tc == 0) & (bc == 0) & (m.check_states(qp)[1] == 0)]
    assert len(good) >= 400
    return robot, env, m, region, good[:200], good[200:400], api.Robot(robot), api.Env(env)


def _gpu(case, a, b):
    robot, env, m, region, _, _, R, E = case
    n = a.shape[0]
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    cost = torch.zeros(n, device="cuda")
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = torch.zeros((n, CAP, robot.num_links), device="cuda")
    api.constrained_motions(R, E, torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), resolution=RES, ok=ok,
                            cost=cost, num_states=cnt, states=st, **region)
    torch.cuda.synchronize()
    return ok.cpu().numpy().astype(bool), cost.cpu().numpy(), cnt.cpu().numpy(), st.cpu().numpy()


def test_constrained_motions_match_the_oracle(case):
    robot, env, m, region, A, B, R, E = case
    g_ok, g_cost, g_cnt, g_st = _gpu(case, A, B)
    o_ok, o_cost, o_cnt, o_st = m.constrained_motions(A, B, O.projection(iterations=2, **region), RES, cap=CAP)
    assert 10 <= g_ok.sum() <= len(A) - 10   # both outcomes occur
    agree = (g_ok == o_ok).mean()
    assert agree >= 0.95, agree
    both = g_ok & o_ok
    same = both & (g_cnt == o_cnt)
    assert same.sum() >= 0.9 * both.sum(), (same.sum(), both.sum())
    assert np.abs(g_cnt[both] - o_cnt[both]).max() <= 2
    for k in np.nonzero(same)[0]:
        c = min(g_cnt[k], CAP)
        assert np.abs(g_st[k, :c] - o_st[k, :c]).max() < 1e-3, k
        assert abs(g_cost[k] - o_cost[k]) <= 1e-3 * max(1.0, o_cost[k]), k
    assert (g_cost[~g_ok] == 0).all()


def test_feasible_constrained_motions_revalidate_on_the_oracle(case):
    robot, env, m, region, A, B, R, E = case
    g_ok, g_cost, g_cnt, g_st = _gpu(case, A, B)
    check = O.projection(iterations=0, **region)
    for k in np.nonzero(g_ok)[0]:
        c = g_cnt[k]
        assert 1 <= c <= CAP
        path = g_st[k, :c]
        assert (m.check_states(path)[1] == 0).all(), k
        _, tc, bc = m.project(path, check)
        assert (tc == 0).all() and (bc == 0).all(), k
        steps = np.linalg.norm(np.diff(np.vstack([A[k][None], path]), axis=0), axis=1)
        assert steps.max() <= 5 * RES * (1 + 1e-5), k
        assert np.linalg.norm(path[-1] - B[k]) < RES, k
        assert abs(g_cost[k] - np.linalg.norm(np.diff(path, axis=0), axis=1).sum()) < 1e-3 * max(1.0, g_cost[k])


def test_constrained_motion_arguments(case):
    robot, env, m, region, A, B, R, E = case
    lib = _lib.load()
    p = _lib.Projection()
    p.task_link = robot.num_links   # out of range
    st = lib.gbmp_constrained_motions(R.handle, E.handle, C_byref(p), None, None, 1, RES, 100, None, None, None, None,
                                      0, None)
    assert st == 1
    p.task_link = -1
    assert lib.gbmp_constrained_motions(R.handle, E.handle, C_byref(p), None, None, 0, RES, 100, None, None, None,
                                        None, 0, None) == _lib.OK


def C_byref(x):
    import ctypes
    return ctypes.byref(x)
