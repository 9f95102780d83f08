"""The oracle against golden vectors of the reference's own kernels
(tests/golden/reference_outputs.npz, made by tests/golden/make_golden.py from the
reference's generated and table FK, sphere transform, collision-cost, step /
interpolation, nearest-neighbour, steer and projection kernels compiled for the host).
Runs without the reference tree; bars as in the pinning tests."""
import os

import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import workloads as W

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_outputs.npz"))
BAND = 1e-4


@pytest.fixture(scope="module")
def edge():
    robot, env, _, _ = W.edge_workload(n_edges=1)
    return robot, env, O.OracleModel(robot, env)


def test_fk_and_sphere_transform(edge):
    robot, env, m = edge
    q = G["fk_q"]
    p32, p64 = m.fk(q), m.fk(q.astype(np.float64), f64=True)
    for k in ("fk_generated", "fk_table"):
        assert np.abs(G[k][:, :, :12] - p64[:, :, :12]).max() < 1e-5, k
        assert np.abs(G[k][:, :, :12] - p32[:, :, :12]).max() < 1e-5, k
    cen = m.sphere_centers(G["fk_table"])
    assert np.abs(cen - G["sphere_centers"]).max() <= 2.5e-7
    assert np.mean(cen == G["sphere_centers"]) > 0.9


def test_collision_costs(edge):
    robot, env, m = edge
    q = G["fk_q"]
    oc, ot = m.check_states(q)
    gc = G["costs"]
    np.testing.assert_allclose(oc, gc, rtol=1e-4, atol=2e-5)
    differ = (ot > 0) != (gc.sum(axis=0) > 0)
    assert np.all(np.abs(m.clearance(q[differ])) <= BAND)
    assert 0 < (gc.sum(axis=0) > 0).sum() < len(q)


def test_edge_steps_and_interpolation(edge):
    robot, env, m = edge
    qf, qt, res = G["edge_from"], G["edge_to"], float(G["edge_res"])
    for k in range(len(qf)):
        n, d = m.edge_steps(qf[k], qt[k], res, O.STEP_L2)
        assert n == G["edge_steps"][k]
        np.testing.assert_array_equal(d, G["edge_dir"][k])
    kk, pos = int(G["edge_interp_count"]), 0
    for k in range(kk):
        st = m.edge_states(qf[k], qt[k], res, O.STEP_L2)
        np.testing.assert_allclose(st, G["edge_interp"][pos:pos + len(st)], rtol=0, atol=2.5e-7)
        pos += len(st)


def test_nearest_and_steer(edge):
    robot, env, m = edge
    nn = O.nearest(G["nn_tree"], G["nn_queries"], active=robot.active, cand=G["nn_candidates"])
    np.testing.assert_array_equal(nn, G["nn_index"])
    st = O.steer(G["nn_tree"][:64], G["steer_to"], float(G["steer_max"]))
    assert np.abs(st - G["steer_out"]).max() <= 1e-6


def test_projection():
    arm = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    m = O.OracleModel(arm)
    La, act = arm.num_links, arm.active.astype(bool)
    # joint-limit pull: to the bit
    q, b = m.project(G["limit_q"], O.projection(task_link=-1, use_boundary=True, iterations=1))[::2]
    np.testing.assert_array_equal(q, G["limit_q1"])
    np.testing.assert_array_equal(b, G["limit_bound_cost"])
    # one task-space iteration, on the states whose step is insensitive to rounding
    kw = dict(task_link=La - 1, offset=G["proj_offset"], reference=[float(x) for x in G["proj_target"]],
              tolerance=[float(x) for x in G["proj_tolerance"]], use_boundary=True, iterations=1)
    qp = G["proj_q"]
    q1 = m.project(qp, O.projection(**kw))[0]
    qu = qp.copy()
    qu[:, act] = np.nextafter(qp[:, act], np.float32(np.inf))
    stable = np.abs(m.project(qu, O.projection(**kw))[0] - q1).max(axis=1) < 1e-5
    assert stable.mean() > 0.75
    assert np.abs(q1[stable] - G["proj_q1"][stable]).max() < 1e-4


def _first_hits_agree(m, qf, qt, res, fh, gfh):
    """First hits equal, or differing only where a state up to the later one lies inside
    the clearance band."""
    for k in np.nonzero(fh != gfh)[0]:
        st = m.edge_states(qf[k], qt[k], res, O.STEP_L2)
        upto = max(fh[k], gfh[k]) if min(fh[k], gfh[k]) >= 0 else len(st) - 1
        assert np.any(np.abs(m.clearance(st[: upto + 1])) <= BAND), (k, fh[k], gfh[k])


def test_wider_states_and_edge_first_hits(edge):
    """128 more states (per-constraint costs) and 40 short edges from collision-free
    starts whose first colliding state the reference's own step, interpolation, FK and
    cost kernels give (7 of them collide part-way)."""
    robot, env, m = edge
    q2, gc = G["state2_q"], G["state2_costs"]
    oc, ot = m.check_states(q2)
    np.testing.assert_allclose(oc, gc, rtol=1e-4, atol=2e-5)
    differ = (ot > 0) != (gc.sum(axis=0) > 0)
    assert np.all(np.abs(m.clearance(q2[differ])) <= BAND)
    ef, et, res = G["edge2_from"], G["edge2_to"], float(G["edge2_res"])
    ok, fh, ns, _ = m.check_motions(ef, et, res, O.STEP_L2)
    np.testing.assert_array_equal(ns, G["edge2_steps"])
    gfh = G["edge2_first_hit"]
    assert (gfh > 0).sum() >= 5 and (gfh < 0).sum() >= 5
    _first_hits_agree(m, ef, et, res, fh, gfh)
    np.testing.assert_array_equal(ok, fh < 0)
