"""Batched planning over heterogeneous problems: every path valid under the oracle,
graph replay and direct launch both correct, and each problem solved in the mix is
also solved alone (and vice versa) on these easy-to-moderate problems."""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RES, RULE = 0.01, _lib.STEP_LINF


@pytest.fixture(scope="module")
def batch():
    def feasible(robot, env):
        q = robot.sample_full(np.random.default_rng(0), 1000)
        return (O.OracleModel(robot, env).check_states(q)[1] == 0).mean() >= 0.02

    models = W.uneven_batch_models(1, n=24, feasible=feasible)
    probs, oracles = [], []
    for i, (robot, env) in enumerate(models):
        m = O.OracleModel(robot, env)
        checker = lambda q, m=m: m.check_states(q)[1] == 0
        edge_free = lambda a, b, m=m: bool(m.check_motions(a[None], b[None], RES, RULE)[0][0])
        _, _, free = W.planning_workload(i, checker, robot=robot, env=env, max_draws=40000)
        s, g = W.pick_problem(free, edge_free, i)
        R, E = api.Robot(robot), api.Env(env)
        probs.append((R, E, s, g, 100 + i))
        oracles.append(m)
    return models, probs, oracles


def _valid(m, path, s, g):
    np.testing.assert_array_equal(path[0], s)
    np.testing.assert_array_equal(path[-1], g)
    ok, fh, ns, ln = m.check_motions(path[:-1], path[1:], RES, RULE)
    for k in np.nonzero(~ok)[0]:
        st = m.edge_states(path[k], path[k + 1], RES, RULE)
        assert np.any(np.abs(m.clearance(st[: fh[k] + 1])) <= 1e-4)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_paths_valid(batch, use_graph):
    models, probs, oracles = batch
    bp = api.BatchPlanner(max_problems=32, max_nodes=32768, max_links=16, path_cap=4096)
    for rep in range(2):                      # second call replays the graph / reuses the trees
        out = bp.solve(probs, lanes_per_problem=8, use_graph=use_graph, range_=0.1, resolution=RES, rule=RULE,
                       time_limit_s=10.0)
        solved = 0
        for (r, path), (R, E, s, g, seed), m in zip(out, probs, oracles):
            if r["solved"]:
                solved += 1
                _valid(m, path, s, g)
        assert solved >= 0.9 * len(probs)


def test_batch_matches_alone(batch):
    models, probs, oracles = batch
    bp = api.BatchPlanner(max_problems=32, max_nodes=32768, max_links=16, path_cap=4096)
    mix = bp.solve(probs, lanes_per_problem=8, use_graph=True, range_=0.1, resolution=RES, rule=RULE)
    for (r, path), (R, E, s, g, seed), m in zip(mix, probs, oracles):
        planner = api.Planner(R, max_nodes=32768, path_cap=4096)
        r1, p1 = planner.solve(E, s, g, lanes=8, range_=0.1, resolution=RES, rule=RULE, seed=seed)
        assert r1["solved"] == r["solved"]
        if r1["solved"]:
            _valid(m, p1, s, g)


def test_autotuned_batch_explores_then_keeps_the_fastest(batch):
    """gbmp_rrtc_solve_batch_auto: a new batch shape tries 4, 8, 16, 32 and 64 lanes per
    problem twice each, in that order, on the caller's own solves, then keeps the one with
    the least time; every solve along the way returns valid paths; another shape (fewer
    problems) gets a decision of its own."""
    models, probs, oracles = batch
    api.BatchPlanner.autotune_reset()
    bp = api.BatchPlanner(max_problems=32, max_nodes=32768, max_links=16, path_cap=4096)
    kw = dict(use_graph=True, range_=0.1, resolution=RES, rule=RULE, time_limit_s=10.0)
    assert api.BatchPlanner.autotune_record(probs, **kw) == ({}, None)
    used = []
    for call in range(12):
        out = bp.solve(probs, lanes_per_problem="auto", **kw)
        used.append(bp.last_lanes)
        assert sum(r["solved"] for r, _ in out) >= 0.9 * len(probs)
        for (r, path), (R, E, s, g, seed), m in zip(out, probs, oracles):
            if r["solved"]:
                _valid(m, path, s, g)
    assert used[:10] == [4, 4, 8, 8, 16, 16, 32, 32, 64, 64]
    times, chosen = api.BatchPlanner.autotune_record(probs, **kw)
    assert sorted(times) == [4, 8, 16, 32, 64] and all(t > 0 for t in times.values())
    assert chosen == min(times, key=lambda k: times[k])
    assert used[10:] == [chosen, chosen]
    sub = probs[:8]
    assert api.BatchPlanner.autotune_record(sub, **kw) == ({}, None)
    bp.solve(sub, lanes_per_problem="auto", **kw)
    assert bp.last_lanes == 4
    api.BatchPlanner.autotune_reset()
    assert api.BatchPlanner.autotune_record(probs, **kw) == ({}, None)
