"""The GPU kernels against golden vectors of the reference's own kernels
(tests/golden/reference_outputs.npz, see tests/golden/make_golden.py): FK poses and
sphere centres, per-constraint collision costs and verdicts, edge step counts and
lengths, edge first hits, nearest-neighbour indices and steered states of the benchmark
robot and scene."""
import os

import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_outputs.npz"))
BAND = 1e-4


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_gpu_matches_reference_golden():
    robot, env, _, _ = W.edge_workload(n_edges=1)
    R, E = api.Robot(robot), api.Env(env)
    m = O.OracleModel(robot, env)
    L, S = robot.num_links, robot.num_spheres
    q = G["fk_q"]
    n = len(q)
    # FK and sphere centres (both sides within 1e-5 of FP64)
    poses = torch.zeros((n, L, 16), device="cuda")
    cen = torch.zeros((n, S, 3), device="cuda")
    api.fk(R, dev(q), poses, cen)
    torch.cuda.synchronize()
    p = poses.cpu().numpy()
    for k in ("fk_generated", "fk_table"):
        assert np.abs(p[:, :, :12] - G[k][:, :, :12]).max() < 2e-5, k
    assert np.abs(cen.cpu().numpy() - G["sphere_centers"]).max() < 3e-5
    # per-constraint costs and verdicts
    costs = torch.zeros((4, n), device="cuda")
    v = torch.zeros(n, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, dev(q), verdict=v, costs=costs, mode=1)
    torch.cuda.synchronize()
    gc = G["costs"]
    np.testing.assert_allclose(costs.cpu().numpy(), gc, rtol=2e-4, atol=4e-5)
    differ = v.cpu().numpy().astype(bool) != (gc.sum(axis=0) > 0)
    assert np.all(np.abs(m.clearance(q[differ])) <= BAND)
    # edge step counts and lengths (the reference's L2 rule)
    qf, qt = G["edge_from"], G["edge_to"]
    ne = len(qf)
    ok = torch.zeros(ne, dtype=torch.uint8, device="cuda")
    ln = torch.zeros(ne, device="cuda")
    ns = torch.zeros(ne, dtype=torch.int32, device="cuda")
    api.check_edges(R, E, dev(qf), dev(qt), float(G["edge_res"]), _lib.STEP_L2, ok, None, ln, ns)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ns.cpu().numpy(), G["edge_steps"])
    np.testing.assert_array_equal(ln.cpu().numpy(), G["edge_length"])
    # nearest neighbour over a candidate group, and steering
    out = torch.zeros(len(G["nn_queries"]), dtype=torch.int32, device="cuda")
    api.nearest(R, dev(G["nn_tree"]), dev(G["nn_queries"]), out, cand=dev(G["nn_candidates"]))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), G["nn_index"])
    to = dev(G["steer_to"])
    api.steer(R, dev(G["nn_tree"][:64]), to, float(G["steer_max"]))
    torch.cuda.synchronize()
    assert np.abs(to.cpu().numpy() - G["steer_out"]).max() <= 1e-6


def test_gpu_edge_first_hits_match_reference_golden():
    """128 more states in cost mode and 40 short edges whose first colliding state comes
    from the reference's own kernels: costs within FP32 tolerance, verdicts and first hits
    equal outside the clearance band, on both edge forms."""
    robot, env, _, _ = W.edge_workload(n_edges=1)
    R, E = api.Robot(robot), api.Env(env)
    m = O.OracleModel(robot, env)
    q2, gc = G["state2_q"], G["state2_costs"]
    n = len(q2)
    costs = torch.zeros((4, n), device="cuda")
    v = torch.zeros(n, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, dev(q2), verdict=v, costs=costs, mode=1)
    torch.cuda.synchronize()
    np.testing.assert_allclose(costs.cpu().numpy(), gc, rtol=2e-4, atol=4e-5)
    differ = v.cpu().numpy().astype(bool) != (gc.sum(axis=0) > 0)
    assert np.all(np.abs(m.clearance(q2[differ])) <= BAND)
    ef, et, res = G["edge2_from"], G["edge2_to"], float(G["edge2_res"])
    gfh = G["edge2_first_hit"]
    ne = len(ef)
    for form in (1, 0):
        R.set_edge_form(form)
        ok = torch.zeros(ne, dtype=torch.uint8, device="cuda")
        fh = torch.zeros(ne, dtype=torch.int32, device="cuda")
        ns = torch.zeros(ne, dtype=torch.int32, device="cuda")
        api.check_edges(R, E, dev(ef), dev(et), res, _lib.STEP_L2, ok, fh, None, ns)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ns.cpu().numpy(), G["edge2_steps"])
        f = fh.cpu().numpy()
        for k in np.nonzero(f != gfh)[0]:
            st = m.edge_states(ef[k], et[k], res, O.STEP_L2)
            upto = max(f[k], gfh[k]) if min(f[k], gfh[k]) >= 0 else len(st) - 1
            assert np.any(np.abs(m.clearance(st[: upto + 1])) <= BAND), (form, k, f[k], gfh[k])
    R.set_edge_form(0)
