"""Golden vectors of the reference's own kernels (test fixtures).

Run where the reference tree is present:  python tests/golden/make_golden.py
It builds, through oracle/ref_build.py, the reference's generated FK / step /
interpolation kernels (KernelGenerator.h), its table FK and sphere transform, the four
collision-cost kernels, the nearest-neighbour and steer kernels and the projection
kernels for the host, runs them on seeded inputs of the benchmark robots and scenes, and
writes tests/golden/reference_outputs.npz (inputs and outputs).  Robots and scenes are
re-created from their seeds by isaac_sim_ros2_humble_gb300.workloads, so only arrays
are stored."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import ref_build  # noqa: E402
from isaac_sim_ros2_humble_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "reference_outputs.npz")


def f32(a):
    return np.ascontiguousarray(a, np.float32).reshape(-1)


def i32(a):
    return np.ascontiguousarray(a, np.int32).reshape(-1)


def main():
    if not (ref_build.available() and ref_build.cost_available() and ref_build.project_available()):
        raise SystemExit("the reference tree is not present")
    robot, env, _, _ = W.edge_workload(n_edges=1)   # 8-DOF torso arm, 110 spheres, 336 obstacles
    L, S = robot.num_links, robot.num_spheres
    rng = np.random.default_rng(2024)
    g = {}

    # forward kinematics: generated kernel and table kernel, then the sphere transform
    q = robot.sample_full(rng, 64)
    gen = ref_build.robot_kernels(robot)
    fk_gen = np.zeros((64, L, 16), np.float32)
    gen.ref_fk(np.ascontiguousarray(q), 64, fk_gen)
    prj = ref_build.project_kernels()
    fk_tab = np.zeros((64, L, 16), np.float32)
    prj.ref_table_fk(64, L, i32(robot.joint_types), f32(robot.joint_poses), f32(robot.joint_axes), i32(robot.parent),
                     f32(q), fk_tab.reshape(-1))
    cen = np.zeros((64, S, 3), np.float32)
    mgr = ref_build.manager_kernels()
    mgr.ref_sphere_centers(64, L, S, i32(robot.sphere_link), f32(robot.sphere_pos), fk_tab.reshape(-1).copy(), cen)
    g.update(fk_q=q, fk_generated=fk_gen, fk_table=fk_tab, sphere_centers=cen)

    # collision costs of those states, from the reference's own centres
    cst = ref_build.cost_kernels()
    r = f32(robot.sphere_r)
    costs = np.zeros((4, 64), np.float32)
    c = np.ascontiguousarray(cen.reshape(-1))
    cst.ref_cost_self(c, i32(robot.sphere_link), r, np.ascontiguousarray(robot.enables, np.uint8).reshape(-1), S, L,
                      64, costs[0])
    ns, nb, nc = env.counts
    cst.ref_cost_sphere(c, r, S, 64, f32(env.sphere_pos), f32(env.sphere_r), ns, costs[1])
    cst.ref_cost_cuboid(c, r, S, 64, f32(env.box_pos), f32(env.box_rot), f32(env.box_min), f32(env.box_max), nb,
                        costs[2])
    cst.ref_cost_cylinder(c, r, S, 64, f32(env.cyl_pos), f32(env.cyl_rot), f32(env.cyl_radius),
                          f32(env.cyl_height), nc, costs[3])
    g.update(costs=costs)

    # edge steps (L2 rule) and the interpolated states of a few edges
    qf, qt = robot.sample_full(rng, 64), robot.sample_full(rng, 64)
    qt[:2] = qf[:2]
    res = np.float32(0.05)
    nsteps = np.zeros(64, np.int32)
    d = np.zeros((64, L), np.float32)
    dist = np.zeros(64, np.float32)
    gen.ref_step(qf.copy(), qt.copy(), 64, res, nsteps, d, dist)
    k = 4
    start = np.concatenate([[0], np.cumsum(nsteps[:k])[:-1]]).astype(np.int32)
    interp = np.zeros((int(nsteps[:k].sum()), L), np.float32)
    gen.ref_interp(np.ascontiguousarray(qf[:k]), np.ascontiguousarray(qt[:k]), k, start, nsteps[:k].copy(),
                   np.ascontiguousarray(d[:k]), interp)
    g.update(edge_from=qf, edge_to=qt, edge_res=np.float32(res), edge_steps=nsteps, edge_dir=d, edge_length=dist,
             edge_interp=interp, edge_interp_count=np.int32(k))

    # nearest neighbour over a candidate group, and steering
    tree, queries = robot.sample_full(rng, 500), robot.sample_full(rng, 32)
    cand = np.sort(rng.choice(500, 300, replace=False)).astype(np.int32)
    nn = np.zeros(32, np.int32)
    mgr.ref_nearest(queries, 32, tree, cand, len(cand), L, i32(robot.active), nn)
    to = robot.sample_full(rng, 64)
    steered = to.copy()
    mgr.ref_steer(steered, 64, tree, L, np.arange(64, dtype=np.int32), 0.5)
    g.update(nn_tree=tree, nn_queries=queries, nn_candidates=cand, nn_index=nn, steer_to=to, steer_out=steered,
             steer_max=np.float32(0.5))

    # projection onto a task-space region (7-DOF arm), one iteration, and the joint-limit pull
    arm = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    La = arm.num_links
    q0 = arm.sample_full(np.random.default_rng(3), 1)
    T = W.fk_numpy(arm, q0)[0][La - 1]
    off = np.eye(4, dtype=np.float32)
    off[:3, :3] = T[:3, :3].T
    target = np.array([T[0, 3], T[1, 3], T[2, 3], 0, 0, 0], np.float32)
    tol = np.array([1e-3] * 3 + [1e-2] * 3, np.float32)
    qp = (q0 + 0.1 * rng.standard_normal((64, La)) * arm.active).astype(np.float32)

    def project(qin, task_link, use_boundary, iterations, tolerance):
        qq = np.ascontiguousarray(qin, np.float32).copy()
        tc, bc = np.zeros(len(qq), np.float32), np.zeros(len(qq), np.float32)
        prj.ref_project(len(qq), La, i32(arm.joint_types), f32(arm.joint_poses), f32(arm.joint_axes), i32(arm.parent),
                        i32(arm.active), f32(arm.lower), f32(arm.upper), task_link, f32(off), f32(target),
                        f32(tolerance), use_boundary, iterations, qq.reshape(-1), tc, bc)
        return qq, tc, bc

    p1 = project(qp, La - 1, 1, 1, tol)
    ql = arm.sample_full(rng, 64)
    act = arm.active.astype(bool)
    ql[:, act] += rng.uniform(-1.0, 1.0, size=(64, act.sum())).astype(np.float32)
    pl = project(ql, -1, 1, 1, np.zeros(6, np.float32))
    g.update(proj_offset=off, proj_target=target, proj_tolerance=tol, proj_q=qp, proj_q1=p1[0], proj_task_cost=p1[1],
             proj_bound_cost=p1[2], limit_q=ql, limit_q1=pl[0], limit_bound_cost=pl[2])

    # wider coverage from a second seed (the arrays above stay as they were):
    # per-constraint costs of 128 more states, and the first colliding state of 40 short
    # edges (reference step rule, interpolation, generated FK, sphere transform and cost
    # kernels; an edge is feasible when every state's total cost is 0, and its first hit
    # is the first state with a positive total).  The reference's kernels run here one
    # thread at a time, about 0.1 s per state, so the edges are kept short (joint moves
    # of at most 0.6, about 25 states each)
    rng2 = np.random.default_rng(2025)

    def ref_costs(qs):
        k2 = len(qs)
        fk = np.zeros((k2, L, 16), np.float32)
        gen.ref_fk(np.ascontiguousarray(qs, np.float32), k2, fk)
        c2 = np.zeros((k2, S, 3), np.float32)
        mgr.ref_sphere_centers(k2, L, S, i32(robot.sphere_link), f32(robot.sphere_pos), fk.reshape(-1).copy(), c2)
        out = np.zeros((4, k2), np.float32)
        cc = np.ascontiguousarray(c2.reshape(-1))
        cst.ref_cost_self(cc, i32(robot.sphere_link), r, np.ascontiguousarray(robot.enables, np.uint8).reshape(-1),
                          S, L, k2, out[0])
        cst.ref_cost_sphere(cc, r, S, k2, f32(env.sphere_pos), f32(env.sphere_r), ns, out[1])
        cst.ref_cost_cuboid(cc, r, S, k2, f32(env.box_pos), f32(env.box_rot), f32(env.box_min), f32(env.box_max), nb,
                            out[2])
        cst.ref_cost_cylinder(cc, r, S, k2, f32(env.cyl_pos), f32(env.cyl_rot), f32(env.cyl_radius),
                              f32(env.cyl_height), nc, out[3])
        return out

    q2 = robot.sample_full(rng2, 128)
    g.update(state2_q=q2, state2_costs=ref_costs(q2))
    # edges from collision-free starts (picked with the oracle, which only selects inputs
    # here) so that first hits fall inside the edges, not at their first state
    import oracle as O
    om = O.OracleModel(robot, env)
    cand = robot.sample_full(rng2, 400)
    ne2 = 40
    ef = cand[om.check_states(cand)[1] == 0][:ne2]
    assert len(ef) == ne2
    et = np.clip(ef + rng2.uniform(-0.6, 0.6, ef.shape).astype(np.float32) * robot.active,
                 robot.lower, robot.upper).astype(np.float32)
    res2 = np.float32(0.05)
    st2 = np.zeros(ne2, np.int32)
    d2 = np.zeros((ne2, L), np.float32)
    dist2 = np.zeros(ne2, np.float32)
    gen.ref_step(ef.copy(), et.copy(), ne2, res2, st2, d2, dist2)
    start2 = np.concatenate([[0], np.cumsum(st2)[:-1]]).astype(np.int32)
    states2 = np.zeros((int(st2.sum()), L), np.float32)
    gen.ref_interp(np.ascontiguousarray(ef), np.ascontiguousarray(et), ne2, start2, st2.copy(), np.ascontiguousarray(d2),
                   states2)
    tot2 = ref_costs(states2).sum(axis=0)
    fh2 = np.full(ne2, -1, np.int32)
    for e in range(ne2):
        hits = np.nonzero(tot2[start2[e]:start2[e] + st2[e]] > 0)[0]
        if len(hits):
            fh2[e] = hits[0]
    g.update(edge2_from=ef, edge2_to=et, edge2_res=res2, edge2_steps=st2, edge2_first_hit=fh2)

    np.savez_compressed(OUT, **g)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
