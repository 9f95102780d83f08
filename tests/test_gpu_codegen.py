"""Runtime-generated robot kernels (NVRTC, sm_103a): the generated FK gives the
table-driven kernels' poses and sphere centres bit for bit (and stays within 1e-5 of
the FP64 oracle), the generated edge set-up gives identical edge results, and the
cubin cache is keyed by the generated source (same robot: hit; other robot: miss;
GBMP_CODEGEN_CACHE directory: read back by a fresh process)."""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def fk_both(R, robot, q):
    out = []
    for cg in (False, True):
        R.use_codegen(cg)
        poses = torch.full((len(q), robot.num_links, 16), np.nan, device="cuda")
        cen = torch.full((len(q), robot.num_spheres, 3), np.nan, device="cuda")
        api.fk(R, dev(q), poses, cen)
        torch.cuda.synchronize()
        out.append((poses.cpu().numpy(), cen.cpu().numpy()))
    return out


@pytest.mark.parametrize("which", ["arm8_torso", "tree"])
def test_generated_fk_is_bit_identical(which):
    if which == "tree":
        robot = W.tree_robot(3)          # branching tree, fixed + prismatic joints, raw axes
    else:
        robot = W.edge_workload(n_edges=1)[0]
    R = api.Robot(robot, codegen=True)
    info = R.codegen_info()
    assert "gbmp_gen_fk" in info["source"] and info["hash"] != 0
    q = robot.sample_full(np.random.default_rng(7), 3000)
    (p0, c0), (p1, c1) = fk_both(R, robot, q)
    np.testing.assert_array_equal(p1, p0)
    np.testing.assert_array_equal(c1, c0)
    m = O.OracleModel(robot)
    p64 = m.fk(q.astype(np.float64), f64=True)
    assert np.abs(p1 - p64).max() < 1e-5
    assert np.abs(c1 - m.sphere_centers(p64)).max() < 1e-5


@pytest.mark.parametrize("rule", [_lib.STEP_L2, _lib.STEP_LINF])
def test_generated_edge_setup_gives_identical_edges(rule):
    robot, env, qf, qt = W.edge_workload(n_edges=2000)
    R, E = api.Robot(robot, codegen=True), api.Env(env)
    res = []
    for cg in (False, True):
        R.use_codegen(cg)
        n = len(qf)
        outs = (torch.zeros(n, dtype=torch.uint8, device="cuda"), torch.zeros(n, dtype=torch.int32, device="cuda"),
                torch.zeros(n, device="cuda"), torch.zeros(n, dtype=torch.int32, device="cuda"))
        api.check_edges(R, E, dev(qf), dev(qt), 0.02, rule, *outs)
        torch.cuda.synchronize()
        res.append([o.cpu().numpy() for o in outs])
    for a, b in zip(*res):
        np.testing.assert_array_equal(a, b)
    assert res[0][0].any() and not res[0][0].all()


def test_cache_is_keyed_by_the_generated_source():
    a = W.serial_arm(31, dof=6, n_spheres=20)
    b = W.serial_arm(32, dof=6, n_spheres=20)
    Ra = api.Robot(a, codegen=True)
    ia = Ra.codegen_info()
    Ra2 = api.Robot(a, codegen=True)
    ia2 = Ra2.codegen_info()
    assert ia2["hash"] == ia["hash"] and ia2["cache"] == 1 and ia2["compile_ms"] == 0.0
    Rb = api.Robot(b, codegen=True)
    assert Rb.codegen_info()["hash"] != ia["hash"]


def test_disk_cache_is_read_by_a_fresh_process(tmp_path):
    script = textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {ROOT!r})
        from isaac_sim_ros2_humble_gb300 import api, workloads as W
        R = api.Robot(W.serial_arm(41, dof=5, n_spheres=12), codegen=True)
        i = R.codegen_info()
        print(i["cache"], i["hash"])
    """)
    env = dict(os.environ, GBMP_CODEGEN_CACHE=str(tmp_path))
    runs = [subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env, timeout=300)
            for _ in range(2)]
    for r in runs:
        assert r.returncode == 0, r.stderr
    (c0, h0), (c1, h1) = (r.stdout.split() for r in runs)
    assert (c0, c1) == ("0", "2") and h0 == h1
    assert any(f.endswith(".cubin") for f in os.listdir(tmp_path))


def test_codegen_info_requires_a_codegen_robot():
    R = api.Robot(W.serial_arm(5, dof=4, n_spheres=8))
    with pytest.raises(_lib.GbmpError):
        R.codegen_info()
    with pytest.raises(_lib.GbmpError):
        R.use_codegen(True)
