"""Parity of the CUDA kernels (through the C-ABI) with the CPU oracle.

Bars: FK link poses within 1e-5 of the FP64 oracle; collision verdicts identical for
every state whose signed clearance exceeds 1e-4 m; costs within FP32 summation
tolerance; step counts, lengths, interpolation, nearest-neighbour indices and
samples bit-exact; edge first-hit indices identical wherever no state up to the
hit lies inside the 1e-4 m clearance band.
"""
import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BAND = 1e-4
FK_TOL = 1e-5


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def plain():
    robot, env, q = W.plain_check_workload(n=4096)
    return robot, env, q, O.OracleModel(robot, env), api.Robot(robot), api.Env(env)


@pytest.fixture(scope="module")
def edge():
    robot, env, qf, qt = W.edge_workload(n_edges=512)
    return robot, env, qf, qt, O.OracleModel(robot, env), api.Robot(robot), api.Env(env)


def test_fk_poses_and_centers(plain, edge):
    for robot, q, m, R in ((plain[0], plain[2], plain[3], plain[4]), (edge[0], edge[2], edge[4], edge[5])):
        n = q.shape[0]
        poses = torch.zeros((n, robot.num_links, 16), device="cuda")
        cen = torch.zeros((n, robot.num_spheres, 3), device="cuda")
        api.fk(R, dev(q), poses, cen)
        torch.cuda.synchronize()
        p64 = m.fk(q.astype(np.float64), f64=True)
        assert np.abs(poses.cpu().numpy() - p64).max() < FK_TOL
        c64 = m.sphere_centers(p64)
        assert np.abs(cen.cpu().numpy() - c64).max() < FK_TOL
        # FP32 mirror: identical operation order, only sin/cos may differ in the last bit
        assert np.abs(poses.cpu().numpy() - m.fk(q)).max() < 2e-6


def test_fk_sizes_and_unaligned_outputs(edge):
    """gbmp_fk by chunks of consecutive states: partial last chunks, a single state, one
    output alone, and pose / centre buffers that are not 16-byte aligned (written word by
    word) all give the poses and centres of one full aligned call, bit for bit."""
    robot, q = edge[0], edge[2]
    R = edge[5]
    L, S = robot.num_links, robot.num_spheres
    n0 = q.shape[0]
    p_ref = torch.zeros((n0, L, 16), device="cuda")
    c_ref = torch.zeros((n0, S, 3), device="cuda")
    api.fk(R, dev(q), p_ref, c_ref)
    for n in (1, 9, 10, 11, 257):
        flat_p = torch.full((n * L * 16 + 1,), float("nan"), device="cuda")
        flat_c = torch.full((n * S * 3 + 1,), float("nan"), device="cuda")
        poses, cen = flat_p[1:].view(n, L, 16), flat_c[1:].view(n, S, 3)   # 4-byte offset
        assert poses.data_ptr() % 16 != 0
        api.fk(R, dev(q[:n]), poses, cen)
        only_p = torch.zeros((n, L, 16), device="cuda")
        api.fk(R, dev(q[:n]), only_p, None)
        only_c = torch.zeros((n, S, 3), device="cuda")
        api.fk(R, dev(q[:n]), None, only_c)
        torch.cuda.synchronize()
        assert torch.equal(poses, p_ref[:n]) and torch.equal(cen, c_ref[:n])
        assert torch.equal(only_p, p_ref[:n]) and torch.equal(only_c, c_ref[:n])
        assert torch.isnan(flat_p[0]) and torch.isnan(flat_c[0])


def test_fk_branching_tree():
    """Parent map that is not a chain, fixed and prismatic joints, un-normalised axes."""
    robot = W.tree_robot(3)
    env = W.random_env(9, 40, 10, 4, oriented=True, center=(0.3, 0.0, 0.3))
    R, E = api.Robot(robot), api.Env(env)
    m = O.OracleModel(robot, env)
    q = robot.sample_full(np.random.default_rng(4), 2048)
    poses = torch.zeros((2048, robot.num_links, 16), device="cuda")
    api.fk(R, dev(q), poses)
    v = torch.zeros(2048, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, dev(q), verdict=v)
    torch.cuda.synchronize()
    assert np.abs(poses.cpu().numpy() - m.fk(q.astype(np.float64), f64=True)).max() < FK_TOL
    _verdict_parity(m, q, v.cpu().numpy().astype(bool))


def _verdict_parity(m, q, verdict):
    cl = m.clearance(q)
    clear = np.abs(cl) > BAND
    assert clear.mean() > 0.95
    np.testing.assert_array_equal(verdict[clear], (cl < 0)[clear])


def test_check_states_verdict(plain, edge):
    for robot, q, m, R, E in ((plain[0], plain[2], plain[3], plain[4], plain[5]),
                              (edge[0], edge[2], edge[4], edge[5], edge[6])):
        v = torch.zeros(q.shape[0], dtype=torch.uint8, device="cuda")
        api.check_states(R, E, dev(q), verdict=v)
        torch.cuda.synchronize()
        _verdict_parity(m, q, v.cpu().numpy().astype(bool))


def test_check_states_costs(plain, edge):
    for robot, q, m, R, E in ((plain[0], plain[2], plain[3], plain[4], plain[5]),
                              (edge[0], edge[2], edge[4], edge[5], edge[6])):
        n = q.shape[0]
        costs = torch.zeros((4, n), device="cuda")
        total = torch.zeros(n, device="cuda")
        v = torch.zeros(n, dtype=torch.uint8, device="cuda")
        api.check_states(R, E, dev(q), verdict=v, costs=costs, total=total, mode=1)
        torch.cuda.synchronize()
        oc, ot = m.check_states(q)
        np.testing.assert_allclose(costs.cpu().numpy(), oc, rtol=1e-4, atol=2e-5)
        np.testing.assert_allclose(total.cpu().numpy(), ot, rtol=1e-4, atol=2e-5)
        cl = m.clearance(q)
        clear = np.abs(cl) > BAND
        np.testing.assert_array_equal(v.cpu().numpy().astype(bool)[clear], (ot > 0)[clear])


def test_check_states_fk_is_one_fk_for_both_outputs(plain, edge):
    """gbmp_check_states_fk (the reference's update() + checkStates() as one launch):
    poses and sphere centres bit-identical to gbmp_fk's, verdicts and costs identical to
    gbmp_check_states', on the 4,096-configuration plain workload and the edge arm."""
    for robot, q, R, E in ((plain[0], plain[2], plain[4], plain[5]), (edge[0], edge[2], edge[5], edge[6])):
        n, L, S = q.shape[0], robot.num_links, robot.num_spheres
        p_ref = torch.zeros((n, L, 16), device="cuda")
        c_ref = torch.zeros((n, S, 3), device="cuda")
        api.fk(R, dev(q), p_ref, c_ref)
        for mode in (_lib.CHECK_VERDICT, _lib.CHECK_COST):
            v_ref = torch.zeros(n, dtype=torch.uint8, device="cuda")
            t_ref = torch.zeros(n, device="cuda")
            api.check_states(R, E, dev(q), verdict=v_ref, total=t_ref if mode else None, mode=mode)
            poses = torch.full((n, L, 16), float("nan"), device="cuda")
            cen = torch.full((n, S, 3), float("nan"), device="cuda")
            v = torch.zeros(n, dtype=torch.uint8, device="cuda")
            t = torch.zeros(n, device="cuda")
            api.check_states(R, E, dev(q), verdict=v, total=t if mode else None, mode=mode, poses=poses, centers=cen)
            torch.cuda.synchronize()
            assert torch.equal(poses, p_ref) and torch.equal(cen, c_ref)
            assert torch.equal(v, v_ref) and torch.equal(t, t_ref)
        # one output alone
        poses = torch.zeros((n, L, 16), device="cuda")
        v = torch.zeros(n, dtype=torch.uint8, device="cuda")
        api.check_states(R, E, dev(q), verdict=v, poses=poses)
        torch.cuda.synchronize()
        assert torch.equal(poses, p_ref)


def _edge_parity(m, qf, qt, res, rule, ok, fh, ln, ns):
    o_ok, o_fh, o_ns, o_ln = m.check_motions(qf, qt, res, rule, early_exit=True)
    np.testing.assert_array_equal(ns, o_ns)
    np.testing.assert_array_equal(ln, o_ln)
    bad = np.nonzero(fh != o_fh)[0]
    for k in bad:
        # a disagreement is only allowed if a state up to the earlier hit is in the band
        states = m.edge_states(qf[k], qt[k], res, rule)
        upto = len(states) - 1 if min(fh[k], o_fh[k]) < 0 else max(fh[k], o_fh[k])
        cl = m.clearance(states[: upto + 1])
        assert np.any(np.abs(cl) <= BAND), (k, fh[k], o_fh[k])
    assert len(bad) <= max(2, len(qf) // 100)
    np.testing.assert_array_equal(ok[fh == o_fh], o_ok[fh == o_fh])
    np.testing.assert_array_equal(ok, fh < 0)


@pytest.mark.parametrize("rule", [0, 1])
def test_check_edges(edge, rule):
    robot, env, qf, qt, m, R, E = edge
    res = 0.05 if rule == 0 else 0.02
    n = qf.shape[0]
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    fh = torch.zeros(n, dtype=torch.int32, device="cuda")
    ln = torch.zeros(n, device="cuda")
    ns = torch.zeros(n, dtype=torch.int32, device="cuda")
    api.check_edges(R, E, dev(qf), dev(qt), res, rule, ok, fh, ln, ns)
    torch.cuda.synchronize()
    _edge_parity(m, qf, qt, res, rule, ok.cpu().numpy().astype(bool), fh.cpu().numpy(), ln.cpu().numpy(),
                 ns.cpu().numpy())
    assert ok.sum().item() > 0 and ok.sum().item() < n
    # the verdict-only call (states coarse to fine) gives the same verdicts
    ok2 = torch.zeros(n, dtype=torch.uint8, device="cuda")
    api.check_edges(R, E, dev(qf), dev(qt), res, rule, ok2)
    torch.cuda.synchronize()
    assert torch.equal(ok2, ok)


def test_check_edges_count_rule(edge):
    """pRRTC's granularity as an edge rule: G + 1 states at k / G of every edge, whatever
    its length, with the same first hits as the oracle; a count outside [1, 1e6] is an
    argument error."""
    robot, env, qf, qt, m, R, E = edge
    n = 256
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    fh = torch.zeros(n, dtype=torch.int32, device="cuda")
    ln = torch.zeros(n, device="cuda")
    ns = torch.zeros(n, dtype=torch.int32, device="cuda")
    api.check_edges(R, E, dev(qf[:n]), dev(qt[:n]), 7, _lib.STEP_COUNT, ok, fh, ln, ns)
    torch.cuda.synchronize()
    ok2 = torch.zeros(n, dtype=torch.uint8, device="cuda")
    api.check_edges(R, E, dev(qf[:n]), dev(qt[:n]), 7, _lib.STEP_COUNT, ok2)
    torch.cuda.synchronize()
    assert torch.equal(ok2, ok)
    nsn = ns.cpu().numpy()
    assert np.all(nsn == 8)
    _edge_parity(m, qf[:n], qt[:n], 7, O.STEP_COUNT, ok.cpu().numpy().astype(bool), fh.cpu().numpy(),
                 ln.cpu().numpy(), nsn)
    st = m.edge_states(qf[0], qt[0], 7, O.STEP_COUNT)
    np.testing.assert_allclose(st[3], qf[0] + 3 * (qt[0] - qf[0]) / 7, atol=1e-6)   # k / G
    with pytest.raises(_lib.GbmpError):
        api.check_edges(R, E, dev(qf[:4]), dev(qt[:4]), 0.5, _lib.STEP_COUNT, ok[:4])


def test_check_edges_plain_robot_reference_rule(plain):
    robot, env, q, m, R, E = plain
    qf, qt = q[:256], q[256:512]
    n = 256
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    fh = torch.zeros(n, dtype=torch.int32, device="cuda")
    ln = torch.zeros(n, device="cuda")
    ns = torch.zeros(n, dtype=torch.int32, device="cuda")
    api.check_edges(R, E, dev(qf), dev(qt), 0.02, 0, ok, fh, ln, ns)
    torch.cuda.synchronize()
    _edge_parity(m, qf, qt, 0.02, 0, ok.cpu().numpy().astype(bool), fh.cpu().numpy(), ln.cpu().numpy(),
                 ns.cpu().numpy())


def test_edges_edge_cases(edge):
    robot, env, qf, qt, m, R, E = edge
    # zero-length edge (n = 1, only the goal is checked) and repeated calls reuse scratch
    same = qf[:8].copy()
    ok = torch.zeros(8, dtype=torch.uint8, device="cuda")
    fh = torch.zeros(8, dtype=torch.int32, device="cuda")
    ns = torch.zeros(8, dtype=torch.int32, device="cuda")
    api.check_edges(R, E, dev(same), dev(same), 0.01, 0, ok, fh, None, ns)
    torch.cuda.synchronize()
    assert np.all(ns.cpu().numpy() == 1)
    _, tot = m.check_states(same)
    np.testing.assert_array_equal(ok.cpu().numpy().astype(bool), tot == 0)
    # empty batch is a no-op
    api.check_edges(R, E, dev(qf[:0]), dev(qt[:0]), 0.01, 0)
    # empty environment: only self-collision remains
    E0 = api.Env(W.Environment.empty())
    v = torch.zeros(64, dtype=torch.uint8, device="cuda")
    api.check_states(R, E0, dev(qf[:64]), verdict=v)
    torch.cuda.synchronize()
    m0 = O.OracleModel(robot, W.Environment.empty())
    _verdict_parity(m0, qf[:64], v.cpu().numpy().astype(bool))


def test_nearest_bit_exact(edge):
    robot, env, qf, qt, m, R, E = edge
    tree = np.concatenate([qf, qt])
    qs = robot.sample_full(np.random.default_rng(9), 300)
    out = torch.zeros(300, dtype=torch.int32, device="cuda")
    api.nearest(R, dev(tree), dev(qs), out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), O.nearest(tree, qs, active=robot.active))
    cand = np.random.default_rng(3).choice(len(tree), 77, replace=False).astype(np.int32)
    api.nearest(R, dev(tree), dev(qs), out, cand=dev(cand))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), O.nearest(tree, qs, active=robot.active, cand=cand))


def test_steer_bit_exact(edge):
    robot, env, qf, qt, m, R, E = edge
    to = dev(qt)
    api.steer(R, dev(qf), to, 0.5)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(to.cpu().numpy(), O.steer(qf, qt, 0.5))


def test_gather_states_exact(edge):
    """SingleArmStateManager::get_states as one gather launch: rows copied bit for bit,
    repeated and unordered indices included; an index outside the rows gives a NaN row
    and raises the flag without touching memory outside the source."""
    robot, env, qf, qt, m, R, E = edge
    M = len(qf)
    src = dev(qf)
    rng = np.random.default_rng(3)
    idx = rng.integers(0, M, size=777).astype(np.int32)
    idx[:5] = [M - 1, 0, 0, 17, M - 1]
    out = torch.zeros((777, robot.num_links), device="cuda")
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    api.gather_states(src, torch.from_numpy(idx).cuda(), out, bad)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), qf[idx])
    assert int(bad.item()) == 0
    idx2 = np.array([3, -1, M, 2], np.int32)
    out2 = torch.zeros((4, robot.num_links), device="cuda")
    api.gather_states(src, torch.from_numpy(idx2).cuda(), out2, bad)
    torch.cuda.synchronize()
    o = out2.cpu().numpy()
    np.testing.assert_array_equal(o[[0, 3]], qf[[3, 2]])
    assert np.isnan(o[1]).all() and np.isnan(o[2]).all()
    assert int(bad.item()) == 1
    api.gather_states(src, torch.from_numpy(idx2[:0]).cuda(), out2[:0])   # nothing to do


def test_sample_bit_exact(edge):
    robot, env, qf, qt, m, R, E = edge
    out = torch.zeros((1000, robot.num_links), device="cuda")
    api.sample(R, 77, 5, out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), O.sample(robot, 77, 5, 1000))


def test_many_links_uses_full_path():
    """More than 32 sphere-carrying links: the broad phase is off and every pair is
    tested; verdicts still match the oracle."""
    robot = W.serial_arm(4, dof=40, n_spheres=80, offset_range=(0.03, 0.06), radius_range=(0.01, 0.02))
    env = W.random_env(8, 24, 6, 4, oriented=True)
    R, E = api.Robot(robot), api.Env(env)
    m = O.OracleModel(robot, env)
    q = robot.sample_full(np.random.default_rng(1), 512)
    v = torch.zeros(512, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, dev(q), verdict=v)
    torch.cuda.synchronize()
    _verdict_parity(m, q, v.cpu().numpy().astype(bool))
    qf, qt = q[:64], q[64:128]
    ok = torch.zeros(64, dtype=torch.uint8, device="cuda")
    fh = torch.zeros(64, dtype=torch.int32, device="cuda")
    ln = torch.zeros(64, device="cuda")
    ns = torch.zeros(64, dtype=torch.int32, device="cuda")
    api.check_edges(R, E, dev(qf), dev(qt), 0.05, 1, ok, fh, ln, ns)
    torch.cuda.synchronize()
    _edge_parity(m, qf, qt, 0.05, 1, ok.cpu().numpy().astype(bool), fh.cpu().numpy(), ln.cpu().numpy(),
                 ns.cpu().numpy())


def _run_edges(R, E, qf, qt, res, rule, first_hit=True):
    """Outputs of one gbmp_check_edges call; without first hits (the verdict-only call,
    which walks each edge coarse to fine) the returned first hits are all 99."""
    n = qf.shape[0]
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    fh = torch.full((n,), 99, dtype=torch.int32, device="cuda")
    ln = torch.zeros(n, device="cuda")
    ns = torch.zeros(n, dtype=torch.int32, device="cuda")
    api.check_edges(R, E, dev(qf), dev(qt), res, rule, ok, fh if first_hit else None, ln, ns)
    torch.cuda.synchronize()
    return ok.cpu().numpy().astype(bool), fh.cpu().numpy(), ln.cpu().numpy(), ns.cpu().numpy()


@pytest.mark.parametrize("kinds", [(0, 0, 0), (48, 0, 0), (0, 24, 0), (0, 0, 12), (40, 0, 9), (0, 20, 6)])
def test_check_edges_obstacle_type_mixes(edge, kinds):
    """The chunked edge kernel's broad phase walks the obstacle runs of every type in one
    pass; scenes with some types absent (or none at all) take the same pass."""
    robot, _, qf, qt, _, R, _ = edge
    ns_, nb_, nc_ = kinds
    env = W.Environment.empty() if not any(kinds) else W.random_env(40 + sum(kinds), ns_, nb_, nc_, oriented=True)
    m = O.OracleModel(robot, env)
    E = api.Env(env)
    ok, fh, ln, ns = _run_edges(R, E, qf[:256], qt[:256], 0.02, 1)
    _edge_parity(m, qf[:256], qt[:256], 0.02, 1, ok, fh, ln, ns)


def test_check_edges_full_size_sampled_parity():
    """The benchmark call itself (65,536 edges, at most 0.01 rad per joint between states):
    state counts and lengths match the oracle on every edge of a seeded sample of 384,
    first hits match outside the clearance band, and the verdict is the first-hit flag."""
    robot, env, qf, qt = W.edge_workload()
    R, E = api.Robot(robot), api.Env(env)
    ok, fh, ln, ns = _run_edges(R, E, qf, qt, 0.01, 1)
    assert len(ok) == 65536
    np.testing.assert_array_equal(ok, fh < 0)
    assert 0 < ok.sum() < len(ok)
    pick = np.sort(np.random.default_rng(11).choice(len(qf), size=2048, replace=False))
    m = O.OracleModel(robot, env)
    _edge_parity(m, qf[pick], qt[pick], 0.01, 1, ok[pick], fh[pick], ln[pick], ns[pick])


def test_edge_forms_agree_on_every_edge_of_the_benchmark_call():
    """All 65,536 edges of the benchmark call validated state by state (k_edge_states) and
    by chunks of 4 and 10 states (k_edge_chunk): identical verdicts, first hits, state
    counts and lengths on every edge (the chunk form's narrow tests are the per-state
    tests); the verdict-only calls of every form (coarse-to-fine state orders) give the
    same verdicts, counts and lengths."""
    robot, env, qf, qt = W.edge_workload()
    R, E = api.Robot(robot), api.Env(env)
    out = {}
    for form in (1, 4, 10):
        R.set_edge_form(form)
        out[form] = _run_edges(R, E, qf, qt, 0.01, 1)
        # verdict only: states walked coarse to fine, the same verdicts
        out[-form] = _run_edges(R, E, qf, qt, 0.01, 1, first_hit=False)
    R.set_edge_form(0)
    for form in (4, 10):
        for a, b in zip(out[form], out[1]):
            np.testing.assert_array_equal(a, b)
    for form in (1, 4, 10):
        vo = out[-form]
        np.testing.assert_array_equal(vo[0], out[1][0])
        np.testing.assert_array_equal(vo[2], out[1][2])
        np.testing.assert_array_equal(vo[3], out[1][3])
        assert np.all(vo[1] == 99)
    for bad in (3, 8):
        with pytest.raises(_lib.GbmpError):
            R.set_edge_form(bad)


@pytest.mark.parametrize("dof,n_spheres", [(4, 100), (3, 120), (6, 70)])
def test_edge_forms_agree_for_large_sphere_groups(dof, n_spheres):
    """Robots whose links carry many spheres: the per-state form groups spheres by link
    (groups of 14-40 spheres, so its self-pair tests take both the sphere-against-group
    path and the pair list), the chunk form by pieces of links (groups of 8-10 spheres):
    the same first hits on every edge, and the oracle's outside the clearance band."""
    robot = W.serial_arm(30 + dof, dof=dof, n_spheres=n_spheres, offset_range=(0.1, 0.3),
                         radius_range=(0.02, 0.05))
    env = W.random_env(31, 40, 12, 4, oriented=True)
    R, E = api.Robot(robot), api.Env(env)
    rng = np.random.default_rng(dof)
    qf, qt = robot.sample_full(rng, 1024), robot.sample_full(rng, 1024)
    out = {}
    for form in (1, 10):
        R.set_edge_form(form)
        out[form] = _run_edges(R, E, qf, qt, 0.02, 1)
    out[-10] = _run_edges(R, E, qf, qt, 0.02, 1, first_hit=False)
    R.set_edge_form(0)
    for a, b in zip(out[10], out[1]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[-10][0], out[1][0])
    ok, fh, ln, ns = out[10]
    assert 0 < ok.sum() < len(ok)
    m = O.OracleModel(robot, env)
    _edge_parity(m, qf[:192], qt[:192], 0.02, 1, ok[:192], fh[:192], ln[:192], ns[:192])


def test_staging_wait_that_gives_up_is_reported_and_the_context_stays_usable(plain):
    """The bounded staging wait's give-up path, forced on a fresh handle (a wait of zero
    polls; no fault, no hang): the launch returns, the handle reports GBMP_ERR_TIMEOUT
    (and keeps reporting it), and another handle's next check on the same context gives
    the oracle's verdicts."""
    robot, env, q, m, R0, E = plain
    R = api.Robot(robot)
    assert R.device_status() == _lib.OK
    R.set_stage_wait(0)
    v = torch.zeros(256, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, dev(q[:256]), verdict=v)
    torch.cuda.synchronize()
    assert R.device_status() == 6   # GBMP_ERR_TIMEOUT
    R.set_stage_wait(-1)
    assert R.device_status() == 6   # sticky for the handle's life
    with pytest.raises(_lib.GbmpError):
        R.set_stage_wait(-2)
    v2 = torch.zeros(256, dtype=torch.uint8, device="cuda")
    api.check_states(R0, E, dev(q[:256]), verdict=v2)
    torch.cuda.synchronize()
    _verdict_parity(m, q[:256], v2.cpu().numpy().astype(bool))
    assert R0.device_status() == _lib.OK


def test_device_status_is_clean_after_every_kernel_family(plain, edge):
    """Every kernel stages its tables with bulk asynchronous copies and a bounded wait;
    none of the launches above gave up that wait (gbmp_robot_device_status)."""
    import ctypes as C
    lib = _lib.load()
    for R in (plain[4], edge[5]):
        st = C.c_int32(-1)
        _lib.check(lib.gbmp_robot_device_status(R.handle, C.byref(st)))
        assert st.value == _lib.OK


def test_edges_too_long_to_validate_are_reported_not_checked(edge):
    """An edge of more than 4,194,304 interpolated states is not validated: first hit -2,
    not free, its state count reported; the other edges of the call are validated as
    usual."""
    robot, env, qf, qt, m, R, E = edge
    j = int(np.nonzero(robot.active)[0][-1])
    res = float((robot.upper[j] - robot.lower[j]) / 5.0e6)
    f = qf[:3].copy()
    t = f.copy()
    t[0, j] = f[0, j] + 20.5 * res          # 21 states
    f[2, j], t[2, j] = robot.lower[j], robot.upper[j]   # a joint across its range: 5e6 states
    ok, fh, ln, ns = _run_edges(R, E, f, t, res, 1)
    assert fh[2] == -2 and not ok[2] and ns[2] == 4194305
    o_ok, o_fh, o_ns, _ = m.check_motions(f[:2], t[:2], res, 1, early_exit=True)
    np.testing.assert_array_equal(ns[:2], o_ns)
    np.testing.assert_array_equal(fh[:2], o_fh)
    assert ns[1] == 1


def test_slab_contact_just_outside_the_band_is_a_collision():
    """A 7-DOF configuration whose sphere reaches 1.03e-4 m into a shelf slab (outside the
    1e-4 m band): the state check, the cost check and a two-state edge ending there all
    report the collision."""
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    env = W.shelf_env(0)
    q = np.array([[0., -0.55056757, -0.4444837, -0.50623834, 1.2990656, -0.17087601, -1.0629332, 0.05316496]],
                 np.float32)
    m = O.OracleModel(robot, env)
    assert m.clearance(q)[0] < -1e-4
    R, E = api.Robot(robot), api.Env(env)
    v = torch.zeros(1, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, dev(q), verdict=v)
    costs = torch.zeros((4, 1), device="cuda")
    vc = torch.zeros(1, dtype=torch.uint8, device="cuda")
    api.check_states(R, E, dev(q), verdict=vc, costs=costs, mode=1)
    torch.cuda.synchronize()
    oc, _ = m.check_states(q)
    np.testing.assert_allclose(costs.cpu().numpy(), oc, rtol=1e-3, atol=2e-6)
    assert int(vc.item()) == 1
    assert int(v.item()) == 1, "verdict-mode check misses a 0.1 mm slab contact"
    prev = np.array([[0., -0.5432064, -0.43647614, -0.49676698, 1.2924869, -0.1640834, -1.0549506, 0.05819874]],
                    np.float32)
    ok, fh, _, ns = _run_edges(R, E, prev, q, 0.01, 1)
    o_ok, o_fh, o_ns, _ = m.check_motions(prev, q, 0.01, 1)
    assert ns[0] == o_ns[0] and fh[0] == o_fh[0] and not ok[0]


def test_space_jacobian_matches_the_oracle(plain, edge):
    """gbmp_space_jacobian (SingleArmStates::calculateSpaceJacobian): every link's 6 x L
    space Jacobian within 2e-5 of the FP64 oracle restatement of the reference kernel, on
    the 7-DOF revolute arm, the prismatic-torso arm and a branching tree with fixed and
    prismatic joints; the columns the reference leaves zero are exactly zero."""
    cases = [(plain[0], plain[2][:512], plain[4]), (edge[0], edge[2][:512], edge[5])]
    tree = W.tree_robot(3)
    cases.append((tree, tree.sample_full(np.random.default_rng(5), 256), api.Robot(tree)))
    for robot, q, R in cases:
        n, L = q.shape[0], robot.num_links
        jac = torch.full((n, L, L, 6), float("nan"), device="cuda")
        api.space_jacobian(R, dev(q), jac)
        torch.cuda.synchronize()
        g = jac.cpu().numpy()
        o = O.OracleModel(robot).space_jacobian(q)
        assert np.abs(g - o).max() < 2e-5, np.abs(g - o).max()
        zero = o == 0
        assert np.all(g[zero] == 0)
        assert np.abs(g).max() > 0.1
