"""Pins the oracle to the reference's own code: the FK, edge-step and interpolation
kernels that cudampl/CUDAMPLib/include/spaces/KernelGenerator.h generates for a robot,
and the four collision-cost kernels of cudampl/CUDAMPLib/src/constraints/ with the
self-collision pair list of SelfCollisionConstraint's constructor, are compiled for the
CPU (oracle/ref_build.py) and compared with the oracle's restatement.  Skipped where
the reference tree is absent."""
import numpy as np
import pytest

import oracle as O
import ref_build
from isaac_sim_ros2_humble_gb300 import workloads as W

pytestmark = pytest.mark.skipif(not ref_build.available(), reason="reference tree not present")


def robots():
    return [W.plain_check_workload(n=1)[0], W.edge_workload(n_edges=1)[0], W.tree_robot(3)]


@pytest.mark.parametrize("idx", [0, 1, 2])
def test_fk_matches_reference_generated_kernel(idx):
    robot = robots()[idx]
    ref = ref_build.robot_kernels(robot)
    q = robot.sample_full(np.random.default_rng(idx), 2000)
    out = np.zeros((q.shape[0], robot.num_links, 16), np.float32)
    ref.ref_fk(np.ascontiguousarray(q), q.shape[0], out)
    m = O.OracleModel(robot)
    p32 = m.fk(q)
    p64 = m.fk(q.astype(np.float64), f64=True)
    # The generated kernel bakes the joint poses and axes into the source with
    # std::to_string, i.e. rounded to 6 decimals (KernelGenerator.h:229-249), so it
    # differs from the exact-table FK by a few 1e-6; both are within 1e-5 of FP64.
    assert np.abs(out - p64).max() < 1e-5
    assert np.abs(out - p32).max() < 1e-5
    np.testing.assert_array_equal(out[:, :, 12:], p32[:, :, 12:])


@pytest.mark.parametrize("idx", [0, 1, 2])
def test_step_and_interpolation_match_reference(idx):
    robot = robots()[idx]
    ref = ref_build.robot_kernels(robot)
    rng = np.random.default_rng(10 + idx)
    n = 300
    qf = robot.sample_full(rng, n)
    qt = robot.sample_full(rng, n)
    qt[:5] = qf[:5]                                   # zero-length edges: one state each
    res = np.float32(0.02)
    ns = np.zeros(n, np.int32)
    d = np.zeros((n, robot.num_links), np.float32)
    dist = np.zeros(n, np.float32)
    ref.ref_step(qf.copy(), qt.copy(), n, res, ns, d, dist)
    m = O.OracleModel(robot)
    for k in range(n):
        n_o, d_o = m.edge_steps(qf[k], qt[k], res, O.STEP_L2)
        assert n_o == ns[k], (k, n_o, ns[k], dist[k] / res)
        np.testing.assert_array_equal(d_o, d[k])
    start = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32)
    out = np.zeros((int(ns.sum()), robot.num_links), np.float32)
    ref.ref_interp(qf, qt, n, start, ns, d, out)
    # The generated interpolation `from + dir * i` (KernelGenerator.h:497-499) is one FMA
    # under NVRTC's default contraction, as in the oracle; the host compiler keeps it as
    # a multiply and an add, hence one rounding of the O(1) joint value (<= 2.4e-7 for
    # |q| < 2) here.  Step counts and directions above are bit-exact.
    for k in range(0, n, 7):
        st = m.edge_states(qf[k], qt[k], res, O.STEP_L2)
        np.testing.assert_allclose(st, out[start[k]:start[k] + ns[k]], rtol=0, atol=2.5e-7)
        np.testing.assert_array_equal(st[-1], qt[k])


def _cost_case(which):
    if which == "plain":
        robot, env, q = W.plain_check_workload(n=48)
    else:
        robot, env, q, _ = W.edge_workload(n_edges=48)
    return robot, env, q


@pytest.mark.skipif(not ref_build.cost_available(), reason="reference constraint sources not present")
@pytest.mark.parametrize("which", ["plain", "edge"])
def test_collision_costs_match_reference_kernels(which):
    """Per-configuration self, sphere, cuboid and cylinder costs of the reference's kernels
    (one 256-thread block per configuration and its shared-memory reduction, run on the
    host) against the oracle's, on the sphere centres of the oracle's FP32 FK (FK itself
    is pinned above).  Same bar as the GPU tests: 1e-4 relative, 2e-5 absolute."""
    robot, env, q = _cost_case(which)
    ref = ref_build.cost_kernels()
    m = O.OracleModel(robot, env)
    oc, ot = m.check_states(q)
    cen = np.ascontiguousarray(m.sphere_centers(m.fk(q)), np.float32)
    n, S, L = q.shape[0], robot.num_spheres, robot.num_links
    r = np.ascontiguousarray(robot.sphere_r, np.float32)
    ns, nb, nc = env.counts
    f = lambda a: np.ascontiguousarray(a, np.float32)
    got = np.zeros((4, n), np.float32)
    npairs = ref.ref_cost_self(cen, np.ascontiguousarray(robot.sphere_link, np.int32), r,
                               np.ascontiguousarray(robot.enables, np.uint8), S, L, n, got[0])
    assert npairs == m.npairs                      # the constructor's pair list, counted
    ref.ref_cost_sphere(cen, r, S, n, f(env.sphere_pos), f(env.sphere_r), ns, got[1])
    ref.ref_cost_cuboid(cen, r, S, n, f(env.box_pos), f(env.box_rot), f(env.box_min), f(env.box_max), nb, got[2])
    ref.ref_cost_cylinder(cen, r, S, n, f(env.cyl_pos), f(env.cyl_rot), f(env.cyl_radius), f(env.cyl_height), nc,
                          got[3])
    for k in range(4):
        if k == 3 and nc == 0:
            assert np.all(got[3] == 0)
            continue
        assert (oc[k] > 0).any(), f"no configuration with cost in slot {k}"
        np.testing.assert_allclose(got[k], oc[k], rtol=1e-4, atol=2e-5, err_msg=f"cost slot {k}")
        np.testing.assert_array_equal(got[k] > 0, oc[k] > 0)


@pytest.mark.skipif(not ref_build.manager_available(), reason="reference state sources not present")
def test_nearest_and_steer_match_reference_kernels():
    """SingleArmStateManager's nearest-neighbour kernel (block per query, shared-memory
    argmin over sqrtf distances of the active joints) and its steer kernel, run on the
    host, against the oracle's restatement: the same nearest index for every query, and
    steered states within 1e-6 and nearly all of them equal to the bit (the host
    compiler fuses the interpolation's multiply-add but not the squared-distance sum,
    where nvcc, the oracle and the GPU kernel fuse both; a one-ulp change of the
    distance moves a state by at most about |to - from| x 1e-7)."""
    robot = W.edge_workload(n_edges=1)[0]
    L = robot.num_links
    rng = np.random.default_rng(5)
    tree = robot.sample_full(rng, 3000)
    queries = robot.sample_full(rng, 128)
    cand = np.sort(rng.choice(3000, 1700, replace=False)).astype(np.int32)
    ref = ref_build.manager_kernels()
    out = np.zeros(128, np.int32)
    ref.ref_nearest(queries, 128, tree, cand, len(cand), L, np.ascontiguousarray(robot.active, np.int32), out)
    np.testing.assert_array_equal(out, O.nearest(tree, queries, active=robot.active, cand=cand))

    to = robot.sample_full(rng, 500)
    steered = to.copy()
    ref.ref_steer(steered, 500, tree, L, np.arange(500, dtype=np.int32), 0.5)
    o = O.steer(tree[:500], to, 0.5)
    assert not np.array_equal(o, to)                # the limit binds on these pairs
    assert np.abs(steered - o).max() <= 1e-6
    assert np.mean(steered == o) > 0.95


@pytest.mark.skipif(not ref_build.manager_available(), reason="reference state sources not present")
@pytest.mark.parametrize("idx", [0, 1, 2])
def test_sphere_transform_matches_reference_kernel(idx):
    """update_self_collision_spheres_kernel (SingleArmStates.cu:340-393) on the oracle's
    FP32 link poses: sphere centres within one rounding of the oracle's and mostly equal
    to the bit (which two products of m0 x + m1 y + m2 z + m3 a compiler fuses first is
    its own choice), both within 1e-6 of the FP64 centres."""
    robot = robots()[idx]
    m = O.OracleModel(robot)
    q = robot.sample_full(np.random.default_rng(20 + idx), 500)
    poses = np.ascontiguousarray(m.fk(q), np.float32)
    n, L, S = q.shape[0], robot.num_links, robot.num_spheres
    out = np.zeros((n, S, 3), np.float32)
    ref_build.manager_kernels().ref_sphere_centers(n, L, S, np.ascontiguousarray(robot.sphere_link, np.int32),
                                                   np.ascontiguousarray(robot.sphere_pos, np.float32), poses, out)
    o = m.sphere_centers(poses)
    assert np.abs(out - o).max() <= 2.5e-7
    assert np.mean(out == o) > 0.9
    p64 = m.sphere_centers(m.fk(q.astype(np.float64), f64=True))
    assert np.abs(out - p64).max() < 1e-6


@pytest.mark.skipif(not ref_build.project_available(), reason="reference projection sources not present")
def test_projection_matches_reference_kernels():
    """SingleArmSpace::projectStates from the reference's own kernels (table FK, the
    task-space and boundary gradients, their sum, update_with_grad, then the two cost
    kernels), run on the host, against the oracle's restatement.  The step solves a
    damped 6x6 system whose conditioning (up to ~1e4) amplifies last-bit differences of
    compiled arithmetic, so: the joint-limit pull alone is compared to the bit; costs
    with no iteration within 1e-5; one iteration on the states whose oracle step moves
    less than 1e-5 when the joints move by one ulp, within 1e-4; ten iterations on
    position targets reach the region on the same states but for at most 6 %."""
    import math
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    m = O.OracleModel(robot)
    ref = ref_build.project_kernels()
    L = robot.num_links
    tip = L - 1
    q0 = robot.sample_full(np.random.default_rng(3), 1)
    T = W.fk_numpy(robot, q0)[0][tip]
    off = np.eye(4, dtype=np.float32)
    off[:3, :3] = T[:3, :3].T
    target = [float(T[0, 3]), float(T[1, 3]), float(T[2, 3]), 0.0, 0.0, 0.0]
    f32 = lambda a: np.ascontiguousarray(a, np.float32).reshape(-1)
    i32 = lambda a: np.ascontiguousarray(a, np.int32).reshape(-1)

    def run_ref(q, task_link, tol, use_boundary, iterations):
        qq = np.ascontiguousarray(q, np.float32).copy()
        tc, bc = np.zeros(len(q), np.float32), np.zeros(len(q), np.float32)
        ref.ref_project(len(q), L, i32(robot.joint_types), f32(robot.joint_poses), f32(robot.joint_axes),
                        i32(robot.parent), i32(robot.active), f32(robot.lower), f32(robot.upper), task_link,
                        f32(off), f32(target), f32(tol), int(use_boundary), iterations, qq.reshape(-1), tc, bc)
        return qq, tc, bc

    def run_oracle(q, task_link, tol, use_boundary, iterations):
        return m.project(q, O.projection(task_link=task_link, offset=off, reference=target, tolerance=tol,
                                         use_boundary=use_boundary, iterations=iterations))

    rng = np.random.default_rng(8)
    act = robot.active.astype(bool)
    # joint-limit pull alone: to the bit
    q = robot.sample_full(rng, 400)
    q[:, act] += rng.uniform(-1.0, 1.0, size=(400, act.sum())).astype(np.float32)
    zero_tol = (0.0,) * 6
    a, b = run_ref(q, -1, zero_tol, True, 1), run_oracle(q, -1, zero_tol, True, 1)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[2], b[2])
    # costs with no iteration
    q = (q0 + 0.1 * rng.standard_normal((600, L)) * robot.active).astype(np.float32)
    tol = (1e-3,) * 3 + (1e-2,) * 3
    a, b = run_ref(q, tip, tol, True, 0), run_oracle(q, tip, tol, True, 0)
    np.testing.assert_allclose(a[1], b[1], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(a[2], b[2], rtol=1e-4, atol=1e-5)
    # one iteration, on the states whose oracle step is insensitive to rounding
    a, b = run_ref(q, tip, tol, True, 1), run_oracle(q, tip, tol, True, 1)
    q_ulp = q.copy()
    q_ulp[:, act] = np.nextafter(q[:, act], np.float32(np.inf))
    bu = run_oracle(q_ulp, tip, tol, True, 1)
    stable = np.abs(bu[0] - b[0]).max(axis=1) < 1e-5
    assert stable.mean() > 0.8
    assert np.abs(a[0][stable] - b[0][stable]).max() < 1e-4
    # ten iterations on a position target: the same states reach the region
    tol = (1e-3,) * 3 + (2 * math.pi,) * 3
    q = (q0 + 0.15 * rng.standard_normal((600, L)) * robot.active).astype(np.float32)
    a, b = run_ref(q, tip, tol, False, 10), run_oracle(q, tip, tol, False, 10)
    reached_a, reached_b = a[1] == 0, b[1] == 0
    assert reached_b.mean() > 0.5
    assert np.mean(reached_a != reached_b) <= 0.06


@pytest.mark.skipif(not ref_build.project_available(), reason="reference state sources not present")
@pytest.mark.parametrize("idx", [0, 1, 2])
def test_table_fk_matches_reference_kernel(idx):
    """The reference's table-driven FK kernel (SingleArmStates.cu:11-221, used by
    calculateForwardKinematics and the projection) against the oracle: within 1e-5 of
    FP64 like the oracle's own FP32 FK, and within 1e-5 of it."""
    robot = robots()[idx]
    q = robot.sample_full(np.random.default_rng(40 + idx), 2000)
    out = np.zeros((q.shape[0], robot.num_links, 16), np.float32)
    f32 = lambda a: np.ascontiguousarray(a, np.float32).reshape(-1)
    i32 = lambda a: np.ascontiguousarray(a, np.int32).reshape(-1)
    ref_build.project_kernels().ref_table_fk(q.shape[0], robot.num_links, i32(robot.joint_types),
                                             f32(robot.joint_poses), f32(robot.joint_axes), i32(robot.parent),
                                             f32(q), out.reshape(-1))
    m = O.OracleModel(robot)
    p64 = m.fk(q.astype(np.float64), f64=True)
    assert np.abs(out[:, :, :12] - p64[:, :, :12]).max() < 1e-5
    assert np.abs(out[:, :, :12] - m.fk(q)[:, :, :12]).max() < 1e-5
