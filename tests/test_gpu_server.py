"""Continuous-batching server: every FK+collision result is identical alone and in the
mix, plan results are valid, the HBM budget admits requests as memory frees up, and
waits time out without losing the request."""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def resident():
    robots = [W.serial_arm(60 + i, dof=6 + i, n_spheres=40 + 20 * i, prismatic_torso=i >= 2, resolution=0.01)
              for i in range(4)]
    envs = [W.random_env(70 + k, 40 + 30 * k, 10 + 5 * k, 2 + k, oriented=True) for k in range(4)]
    R = [api.Robot(r) for r in robots]
    E = [api.Env(e) for e in envs]
    return robots, envs, R, E


def alone(R, E, q):
    v = torch.zeros(q.shape[0], dtype=torch.uint8, device="cuda")
    api.check_states(R, E, torch.from_numpy(q).cuda(), verdict=v)
    torch.cuda.synchronize()
    return v.cpu().numpy()


def test_results_same_alone_and_in_mix(resident):
    robots, envs, R, E = resident
    srv = api.Server(num_streams=4, hbm_budget_bytes=64 << 20, max_batch_states=200_000, plan_workers=1,
                     plan_batch=8, plan_lanes=16)
    rid = [srv.add_robot(r) for r in R]
    eid = [srv.add_env(e) for e in E]
    srv.start()
    rng = np.random.default_rng(0)
    reqs = []
    for k in range(150):
        i, j = int(rng.integers(4)), int(rng.integers(4))
        n = int(np.exp(rng.uniform(0, np.log(20000))))
        q = robots[i].sample_full(rng, n)
        v = np.zeros(n, np.uint8)
        reqs.append(("check", i, j, q, v, srv.submit_check(rid[i], eid[j], q, v)))
        if k % 25 == 0:
            m = O.OracleModel(robots[i], envs[j])
            free = None
            for _ in range(20):
                qs = robots[i].sample_full(rng, 512)
                ok = m.check_states(qs)[1] == 0
                if ok.sum() >= 2:
                    free = qs[ok]
                    break
            if free is not None:
                path = np.zeros((4096, robots[i].num_links), np.float32)
                reqs.append(("plan", i, j, (free[0], free[1], m), path,
                             srv.submit_plan(rid[i], eid[j], free[0], free[1], 7 + k, path)))
    for kind, i, j, data, out, t in reqs:
        info = srv.wait(t, 60.0)
        assert info is not None
        if kind == "check":
            assert info["status"] == 0
            np.testing.assert_array_equal(out, alone(R[i], E[j], data))
        else:
            s0, g0, m = data
            if info["solved"]:
                path = out[: info["path_len"]]
                np.testing.assert_array_equal(path[0], s0)
                np.testing.assert_array_equal(path[-1], g0)
                ok, fh, ns, ln = m.check_motions(path[:-1], path[1:], 0.01, _lib.STEP_LINF)
                for e in np.nonzero(~ok)[0]:
                    st = m.edge_states(path[e], path[e + 1], 0.01, _lib.STEP_LINF)
                    assert np.any(np.abs(m.clearance(st[: fh[e] + 1])) <= 1e-4)
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["budget_in_use"] == 0
    assert st["batches"] < 150            # requests were batched
    srv.close()


def test_budget_admission_and_oversize(resident):
    robots, envs, R, E = resident
    L = robots[0].num_links
    one = 4096 * (L * 4 + 1) + 64
    srv = api.Server(num_streams=2, hbm_budget_bytes=2 * one, max_batch_states=1 << 20, plan_workers=0)
    srv.add_robot(R[0])
    srv.add_env(E[0])
    srv.start()
    rng = np.random.default_rng(1)
    qs = [robots[0].sample_full(rng, 4096) for _ in range(12)]
    vs = [np.zeros(4096, np.uint8) for _ in range(12)]
    ts = [srv.submit_check(0, 0, q, v) for q, v in zip(qs, vs)]
    big = robots[0].sample_full(rng, 50_000)
    vb = np.zeros(50_000, np.uint8)
    tb = srv.submit_check(0, 0, big, vb)
    for q, v, t in zip(qs, vs, ts):
        info = srv.wait(t, 60.0)
        assert info["status"] == 0
        np.testing.assert_array_equal(v, alone(R[0], E[0], q))
    info = srv.wait(tb, 60.0)
    assert info["status"] == 5             # larger than the whole budget: capacity error
    assert srv.stats()["budget_in_use"] == 0
    srv.close()


def test_wait_timeout_keeps_ticket(resident):
    robots, envs, R, E = resident
    srv = api.Server(num_streams=1, hbm_budget_bytes=1 << 30, plan_workers=0)
    srv.add_robot(R[3])
    srv.add_env(E[3])
    srv.start()
    q = robots[3].sample_full(np.random.default_rng(2), 400_000)
    v = np.zeros(q.shape[0], np.uint8)
    t = srv.submit_check(0, 0, q, v)
    first = srv.wait(t, 1e-6)
    info = srv.wait(t, 120.0)
    assert info is not None and info["status"] == 0
    assert first is None or first["status"] == 0
    srv.close()


def test_plans_alone_and_in_the_mix_agree_statistically():
    """Plan requests are solved by parallel lanes, so a result is not reproducible to the
    bit; the same 30 shelf problems served one at a time and served inside a stream of
    check requests must agree statistically: success counts within a two-proportion
    |z| < 3, path lengths with a two-sided Mann-Whitney p > 0.01 and a median per-problem
    ratio within [0.85, 1.15].  Every solved path starts and ends at its problem's start
    and goal."""
    scipy_stats = pytest.importorskip("scipy.stats")
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7", resolution=0.01)
    shelves = [W.shelf_env(k) for k in range(3)]
    R = api.Robot(robot)
    E = [api.Env(e) for e in shelves]
    probs = []
    for seed in range(30):
        m = O.OracleModel(robot, shelves[seed % 3])
        _, _, fs = W.planning_workload(seed, lambda q, m=m: m.check_states(q)[1] == 0, robot=robot,
                                       env=shelves[seed % 3])
        s0, g0 = W.pick_problem(fs, lambda a, b, m=m: bool(m.check_motions(a[None], b[None], 0.01, 1)[0][0]),
                                seed)
        probs.append((seed % 3, s0, g0, 100 + seed))

    def serve(mix):
        srv = api.Server(num_streams=4, hbm_budget_bytes=1 << 30, max_batch_states=1 << 20, plan_workers=1,
                         plan_batch=8, plan_lanes=64, planner_max_nodes=65536, plan_path_cap=4096)
        srv.add_robot(R)
        for e in E:
            srv.add_env(e)
        srv.start()
        rng = np.random.default_rng(9)
        out, keep = [], []
        for k, s0, g0, seed in probs:
            path = np.zeros((4096, robot.num_links), np.float32)
            t = srv.submit_plan(0, k, s0, g0, seed, path)
            if mix:   # check traffic around every plan
                for _ in range(10):
                    q = robot.sample_full(rng, int(rng.integers(1, 20000)))
                    v = np.zeros(q.shape[0], np.uint8)
                    keep.append((q, v, srv.submit_check(0, int(rng.integers(3)), q, v)))
            info = srv.wait(t, 60.0)
            assert info is not None
            if info["solved"]:
                np.testing.assert_array_equal(path[0], s0)
                np.testing.assert_array_equal(path[info["path_len"] - 1], g0)
            out.append((bool(info["solved"]), float(info["cost"])))
        for q, v, t in keep:
            assert srv.wait(t, 60.0)["status"] == 0
        srv.close()
        return out

    a, b = serve(False), serve(True)
    sa, sb = np.array([s for s, _ in a]), np.array([s for s, _ in b])
    p = (sa.sum() + sb.sum()) / (2 * len(sa))
    z = 0.0 if p in (0.0, 1.0) else (sa.mean() - sb.mean()) / np.sqrt(p * (1 - p) * 2 / len(sa))
    assert abs(z) < 3.0
    ca = np.array([c for s, c in a if s])
    cb = np.array([c for s, c in b if s])
    assert scipy_stats.mannwhitneyu(ca, cb, alternative="two-sided").pvalue > 0.01
    both = sa & sb
    ratio = np.median(np.array([c for _, c in a])[both] / np.array([c for _, c in b])[both])
    assert 0.85 <= ratio <= 1.15, ratio
