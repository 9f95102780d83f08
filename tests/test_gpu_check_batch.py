"""Batched state checks of several (robot, scene) requests in one launch
(gbmp_check_batch_run): every request's verdicts, costs, poses and sphere centres are
bit-identical to a gbmp_check_states_fk call of its own, whatever the mix of robots (6 to
9 links, 30 to 110 spheres, a branching tree), scenes and request sizes (including empty
and single-state requests), in verdict and cost mode; the verdicts also match the oracle
outside the clearance band."""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BAND = 1e-4


@pytest.fixture(scope="module")
def mix():
    robots = [W.serial_arm(1, dof=7, n_spheres=59, name="arm7"),
              W.serial_arm(2, dof=8, n_spheres=110, prismatic_torso=True, name="arm8"),
              W.serial_arm(5, dof=5, n_spheres=30, name="arm5"),
              W.tree_robot(3)]
    envs = [W.random_env(11, 32, 8, 0, oriented=False), W.random_env(12, 256, 64, 16, oriented=True),
            W.random_env(13, 0, 0, 6, oriented=True), W.shelf_env(0)]
    R = [api.Robot(r) for r in robots]
    E = [api.Env(e) for e in envs]
    rng = np.random.default_rng(9)
    sizes = [0, 1, 7, 64, 333, 4096, 2500, 1, 900, 31, 12000, 257, 5, 1500]
    reqs = []
    for i, n in enumerate(sizes):
        ri, ei = int(rng.integers(len(robots))), int(rng.integers(len(envs)))
        q = robots[ri].sample_full(rng, max(n, 1))[:n]
        reqs.append((ri, ei, q))
    return robots, envs, R, E, reqs


def _outputs(robots, R, reqs, mode, with_fk):
    outs = []
    for ri, ei, q in reqs:
        n, L, S = len(q), robots[ri].num_links, robots[ri].num_spheres
        o = {"q": torch.from_numpy(np.ascontiguousarray(q, np.float32).reshape(n, L)).cuda(),
             "verdict": torch.full((n,), 7, dtype=torch.uint8, device="cuda")}
        if mode == _lib.CHECK_COST:
            o["costs"] = torch.full((4, n), float("nan"), device="cuda")
            o["total"] = torch.full((n,), float("nan"), device="cuda")
        if with_fk:
            o["poses"] = torch.full((n, L, 16), float("nan"), device="cuda")
            o["centers"] = torch.full((n, S, 3), float("nan"), device="cuda")
        outs.append(o)
    return outs


@pytest.mark.parametrize("mode,with_fk", [(_lib.CHECK_VERDICT, False), (_lib.CHECK_VERDICT, True),
                                          (_lib.CHECK_COST, False), (_lib.CHECK_COST, True)])
def test_batch_equals_one_call_per_request(mix, mode, with_fk):
    robots, envs, R, E, reqs = mix
    batched = _outputs(robots, R, reqs, mode, with_fk)
    single = _outputs(robots, R, reqs, mode, with_fk)
    cb = api.CheckBatch(max_requests=32)
    cb.run([dict(robot=R[ri], env=E[ei], **o) for (ri, ei, _), o in zip(reqs, batched)], mode=mode)
    for (ri, ei, _), o in zip(reqs, single):
        if o["q"].shape[0]:
            api.check_states(R[ri], E[ei], o["q"], verdict=o["verdict"], costs=o.get("costs"),
                             total=o.get("total"), mode=mode, poses=o.get("poses"), centers=o.get("centers"))
    torch.cuda.synchronize()
    for a, b in zip(batched, single):
        for k in a:
            assert torch.equal(a[k], b[k]) or (a[k].numel() == 0), k
    cb.close()


def test_batch_verdicts_match_the_oracle(mix):
    robots, envs, R, E, reqs = mix
    outs = _outputs(robots, R, reqs, _lib.CHECK_VERDICT, False)
    cb = api.CheckBatch(max_requests=len(reqs))
    cb.run([dict(robot=R[ri], env=E[ei], **o) for (ri, ei, _), o in zip(reqs, outs)])
    torch.cuda.synchronize()
    models = {}
    for (ri, ei, q), o in zip(reqs, outs):
        if len(q) == 0:
            continue
        m = models.setdefault((ri, ei), O.OracleModel(robots[ri], envs[ei]))
        qs = q[:512]
        cl = m.clearance(qs)
        clear = np.abs(cl) > BAND
        v = o["verdict"].cpu().numpy()[:512].astype(bool)
        np.testing.assert_array_equal(v[clear], (cl < 0)[clear])


def test_batch_rejects_bad_requests(mix):
    robots, envs, R, E, reqs = mix
    cb = api.CheckBatch(max_requests=2)
    q = torch.zeros((4, robots[0].num_links), device="cuda")
    v = torch.zeros(4, dtype=torch.uint8, device="cuda")
    three = [dict(robot=R[0], env=E[0], q=q, verdict=v)] * 3
    with pytest.raises(_lib.GbmpError):
        cb.run(three)
    with pytest.raises(_lib.GbmpError):
        cb.run([dict(robot=R[0], env=E[0], q=q, verdict=v)], mode=5)
    cb.run([])                                   # nothing to do
    cb.run([dict(robot=R[0], env=E[0], q=q, verdict=v)] * 2)
    torch.cuda.synchronize()
    cb.close()
