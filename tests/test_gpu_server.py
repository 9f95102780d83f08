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
