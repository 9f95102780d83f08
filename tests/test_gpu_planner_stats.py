"""Statistical parity of the parallel RRT-Connect planner.

The reference planners (CPRRTC, cudampl/CPRRTC/src/RobotSolver.cu:562-796; pRRTC,
pRRTC/src/planning/pRRTC.cu:340-601) are randomised and lane-parallel, so a solve is not
reproducible to the bit: which lane connects first depends on timing.  The bar is
statistical.  On a fixed set of seeded shelf problems (7-DOF arm, 5 slabs + 40 boxes,
collision-free start and goal whose straight edge collides), the device planner is
compared with the oracle's lane-parallel restatement (oracle.rrtc_lanes: the same
per-lane rule, Philox streams, balance rule and step rule, lanes in synchronous rounds):

  * success rate: two-proportion z statistic |z| < 3;
  * path length (L2 over the active joints): Mann-Whitney U two-sided p > 0.01 over the
    solved problems, and the median of the per-problem ratios device / oracle within
    [0.9, 1.1].

Every device path is also re-validated by the oracle's edge checker (up to the 1e-4 m
clearance band, as every verdict test here).  The same bar
compares batched solves (one persistent launch, lanes migrating between problems) with
single solves, and pRRTC's balance strategies 1 and 2 on the device with the oracle.
"""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
scipy_stats = pytest.importorskip("scipy.stats")
pytestmark = pytest.mark.gpu

N_PROBLEMS = 60
LANES = 32
RANGE = 0.1
RES = 0.01
RULE = _lib.STEP_LINF
MAX_NODES = 200_000
MAX_ITERS = 20_000
Z_MAX = 3.0
MWU_P_MIN = 0.01
RATIO_BAND = (0.9, 1.1)


def _z_two_proportions(k1, n1, k2, n2):
    p = (k1 + k2) / (n1 + n2)
    if p in (0.0, 1.0):
        return 0.0
    return (k1 / n1 - k2 / n2) / np.sqrt(p * (1 - p) * (1 / n1 + 1 / n2))


def _compare(name, a, b):
    """a, b: lists of (solved, cost) per problem, same problem order.  Returns a summary
    and asserts the statistical bar."""
    sa = np.array([s for s, _ in a], bool)
    sb = np.array([s for s, _ in b], bool)
    z = _z_two_proportions(sa.sum(), len(sa), sb.sum(), len(sb))
    ca = np.array([c for s, c in a if s])
    cb = np.array([c for s, c in b if s])
    both = sa & sb
    ratio = float(np.median(np.array([x[1] for x in a])[both] / np.array([x[1] for x in b])[both]))
    p = float(scipy_stats.mannwhitneyu(ca, cb, alternative="two-sided").pvalue)
    summary = (f"{name}: success {sa.sum()}/{len(sa)} vs {sb.sum()}/{len(sb)} (z {z:.2f}); path length median "
               f"{np.median(ca):.3f} vs {np.median(cb):.3f}, Mann-Whitney p {p:.3f}, median per-problem ratio "
               f"{ratio:.3f}")
    print(summary)
    assert abs(z) < Z_MAX, summary
    assert p > MWU_P_MIN, summary
    assert RATIO_BAND[0] <= ratio <= RATIO_BAND[1], summary
    return summary


@pytest.fixture(scope="module")
def shelf():
    """Seeded shelf problems chosen with the oracle's checker (so the problem set does
    not depend on the kernels under test)."""
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    models, problems = {}, []
    for seed in range(N_PROBLEMS):
        sc = seed % 10
        if sc not in models:
            env = W.shelf_env(sc)
            models[sc] = (env, O.OracleModel(robot, env))
        env, m = models[sc]

        def free(q, m=m):
            return m.check_states(q)[1] == 0

        def edge_free(a, b, m=m):
            return bool(m.check_motions(a[None], b[None], RES, RULE)[0][0])

        _, _, fs = W.planning_workload(seed, free, robot=robot, env=env)
        s0, g0 = W.pick_problem(fs, edge_free, seed)
        problems.append((seed, sc, s0, g0))
    R = api.Robot(robot)
    envs = {sc: api.Env(models[sc][0]) for sc in models}
    return robot, R, models, envs, problems


BAND = 1e-4


def _valid(m, path, s0, g0):
    """Start and goal at the ends; every path edge free by the oracle, except where a
    state up to the oracle's first hit lies within the 1e-4 m clearance band (the
    device's expanded sphere test and the oracle's cost formula round differently at the
    contact surface)."""
    assert np.allclose(path[0], s0) and np.allclose(path[-1], g0)
    ok, fh, _, _ = m.check_motions(path[:-1], path[1:], RES, RULE)
    for k in np.nonzero(~ok)[0]:
        st = m.edge_states(path[k], path[k + 1], RES, RULE)
        assert np.any(np.abs(m.clearance(st[: fh[k] + 1])) <= BAND), f"path edge {k} collides"


def _device_single(shelf, balance=_lib.BALANCE_DEFAULT, problems=None):
    robot, R, models, envs, probs = shelf
    planner = api.Planner(R, max_nodes=MAX_NODES, path_cap=65536)
    out = []
    for seed, sc, s0, g0 in (problems or probs):
        r, path = planner.solve(envs[sc], s0, g0, lanes=LANES, max_iters=MAX_ITERS, range_=RANGE, resolution=RES,
                                rule=RULE, seed=seed, time_limit_s=30.0, balance=balance)
        if r["solved"]:
            # the device's own state check agrees that every waypoint is free (a planner
            # that appended an unchecked node would fail here, whatever the rounding)
            v = torch.zeros(len(path), dtype=torch.uint8, device="cuda")
            api.check_states(R, envs[sc], torch.from_numpy(np.ascontiguousarray(path)).cuda(), verdict=v)
            torch.cuda.synchronize()
            bad = np.nonzero(v.cpu().numpy())[0]
            assert len(bad) == 0, (seed, bad.tolist(), path[bad].tolist())
            _valid(models[sc][1], path, s0, g0)
        out.append((bool(r["solved"]), float(r["cost"])))
    return out


def _oracle_lanes(shelf, balance=3, problems=None):
    robot, R, models, envs, probs = shelf
    out = []
    for seed, sc, s0, g0 in (problems or probs):
        r, path = O.rrtc_lanes(models[sc][1], s0, g0, lanes=LANES, range_=RANGE, res=RES, rule=RULE, seed=seed,
                               balance=balance, tree_ratio=1.0 if balance == 2 else 0.5, max_nodes=MAX_NODES,
                               max_iters=MAX_ITERS)
        out.append((bool(r["solved"]), float(r["cost"])))
    return out


@pytest.fixture(scope="module")
def single(shelf):
    return _device_single(shelf)


def test_device_planner_matches_the_lane_parallel_oracle(shelf, single):
    ora = _oracle_lanes(shelf)
    _compare("device vs oracle (proportional balance)", single, ora)


def test_balance_strategy_one_matches_the_oracle(shelf):
    half = shelf[4][N_PROBLEMS // 2:]
    dev = _device_single(shelf, balance=_lib.BALANCE_SIZE, problems=half)
    ora = _oracle_lanes(shelf, balance=1, problems=half)
    _compare("device vs oracle (balance 1)", dev, ora)


def test_batched_solves_match_single_solves(shelf, single):
    robot, R, models, envs, probs = shelf
    bp = api.BatchPlanner(max_problems=len(probs), max_nodes=32768, max_links=16, path_cap=4096)
    batch = bp.solve([(R, envs[sc], s0, g0, seed) for seed, sc, s0, g0 in probs], lanes_per_problem=LANES,
                     use_graph=True, max_iters=MAX_ITERS, range_=RANGE, resolution=RES, rule=RULE,
                     time_limit_s=30.0)
    out = []
    for (r, path), (seed, sc, s0, g0) in zip(batch, probs):
        if r["solved"]:
            _valid(models[sc][1], path, s0, g0)
        out.append((bool(r["solved"]), float(r["cost"])))
    _compare("batched vs single", out, single)


def test_balance_strategy_two_matches_the_oracle(shelf):
    half = shelf[4][: N_PROBLEMS // 2]
    dev = _device_single(shelf, balance=_lib.BALANCE_SWAP, problems=half)
    ora = _oracle_lanes(shelf, balance=2, problems=half)
    _compare("device vs oracle (balance 2)", dev, ora)
