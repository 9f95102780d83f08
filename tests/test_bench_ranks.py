"""The N > 1 path of bench.py on CPU: two gloo ranks reduce their timings and check
counts the way the GPU ranks do (max of times, sum of checks), every rank validates
its own shard of edges for the same robot and scene, and the reference arm prints from
rank 0 only."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from isaac_sim_ros2_humble_gb300 import workloads as W

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        res = bench.reduce_over_ranks(dist, ws, "cpu", timed_s=1.0 + rank, checks=100 * (rank + 1),
                                      e2e_s=2.0 + 0.5 * rank)
        dist.barrier()
    finally:
        dist.destroy_process_group()
    out.put((rank, res))


def test_two_gloo_ranks_reduce_like_the_gpu_run():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert got[r] == (2.0, 300.0, 2.5)


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(None, 1, "cpu", 1.5, 7, 2.5) == (1.5, 7.0, 2.5)


def test_shards_share_robot_and_scene_but_not_edges():
    r0, e0, f0, t0 = W.edge_workload(n_edges=64, shard=0)
    r1, e1, f1, t1 = W.edge_workload(n_edges=64, shard=1)
    np.testing.assert_array_equal(r0.joint_poses, r1.joint_poses)
    np.testing.assert_array_equal(r0.sphere_pos, r1.sphere_pos)
    np.testing.assert_array_equal(e0.sphere_pos, e1.sphere_pos)
    np.testing.assert_array_equal(e0.box_pos, e1.box_pos)
    assert not np.any(np.all(f0 == f1, axis=1))
    assert not np.any(np.all(t0 == t1, axis=1))


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_line_has_the_contract_keys():
    """The reference arm (one process) prints one JSON line with the benchmark's metric,
    unit and direction, a cpu_baseline describing the run, and an e2e entry with no
    host-device copies."""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--edges", "4096"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "FK+collision checks/s" and d["unit"] == "checks/s"
    assert d["higher_is_better"] is True and d["value"] > 0 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "checks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
