#!/usr/bin/env python
"""Benchmark of the motion-planning hot path on one GB300.

Headline (`value`, `e2e`): interpolated-edge validation (FK + sphere collision).
65,536 random edges of an 8-DOF arm (prismatic torso 0-0.4 m + 7 revolute joints, 110
link spheres) in a scene of 256 spheres, 64 oriented boxes and 16 cylinders,
interpolated at 0.01 rad maximum joint step; output per edge: collision flag and
first-collision state index.  Synthetic, seeded inputs (no dataset).

Metric: FK+collision checks/s, where the checks of a batch are the interpolated states
the reference's checkMotions validates for it (every state of every edge).  `value` is
measured on device-resident inputs; `e2e` goes through the same C-ABI call with host
buffers (H2D of the edge endpoints and D2H of the results inside the timed region).

The same line carries `secondary`: the other four workloads of the benchmark set, each
with its own clock record taken during its timed region:
  plain_fk_collision  4,096 configurations of a 7-DOF arm (59 spheres) against 32
                      spheres + 8 boxes: one collision flag and the link poses per
                      configuration, from one launch;
  plan                single-problem parallel RRT-Connect on 100 seeded shelf problems:
                      time to solution p50 / p99;
  uneven_batch        256 heterogeneous planning problems in one persistent launch
                      against 256 sequential single-problem solves;
  serving             a Poisson request stream over 4 resident robots and 16 resident
                      scenes against the per-request path.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbmp|reference]
                  [--workload all|edges|plain|plan|batch|serve]

N > 1 runs under torchrun: every rank validates its own 65,536 edges (weak scaling, no
collective on the data path); the step time is the max over ranks.  The secondary
workloads run on rank 0 at N = 1 only.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "FK+collision checks/s"
UNIT = "checks/s"
WORKLOAD = "edge_validation_8dof_65536_edges"
STEP = 0.01
RULE = 1              # L-infinity: at most 0.01 rad per joint between consecutive states
CPU_SAMPLE_EDGES = 1536
PLAN_RES = 0.01
PLAN_RANGE = 0.1
L2_FLUSH_BYTES = 384 * 1024 * 1024   # > L2 (126 MB)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbmp", choices=["gbmp", "reference"])
    ap.add_argument("--edges", type=int, default=65536)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="all", choices=["all", "edges", "plain", "fk", "checkbatch", "plan", "batch", "serve"],
                    help="all: the headline edge line with every secondary workload; otherwise one workload's "
                         "own line")
    ap.add_argument("--plan-seeds", type=int, default=100)
    ap.add_argument("--lanes", default="1024,2048,4096,8192")
    ap.add_argument("--fk-states", type=int, default=1 << 20, help="fk: states per launch")
    ap.add_argument("--rates", default="200,1000,2000", help="serve: Poisson arrival rates (req/s)")
    ap.add_argument("--duration", type=float, default=2.0, help="serve: seconds of arrivals per rate")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_over_ranks(dist, ws, device, timed_s, checks, e2e_s):
    """Job totals of a weak-scaling run: every rank validates its own shard of edges,
    so the job's time is the slowest rank's (max) and its checks are the sum.  One
    collective for the times and one for the counts, in the same order on every rank."""
    if ws == 1:
        return timed_s, float(checks), e2e_s
    import torch
    t = torch.tensor([timed_s, e2e_s], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(checks)], dtype=torch.float64, device=device)
    dist.all_reduce(c)
    return float(t[0].item()), float(c[0].item()), float(t[1].item())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region:
    sampling starts (and its first sample is awaited) before the region, every sample
    carries its time stamp, and only the samples inside the region are summarised (all
    of them if none fell inside)."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        self.t_begin = self.t_end = None
        return self

    def mark_begin(self):
        self.t_begin = time.time()

    def mark_end(self):
        self.t_end = time.time()

    @staticmethod
    def _stamp(text):
        try:
            return datetime.datetime.strptime(text.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 10:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        inside, in_region = rows, False
        if self.t_begin is not None and self.t_end is not None:
            # a sample stamped up to one period after the region still describes it
            sel = [r for r in rows if (lambda t: t is not None and self.t_begin <= t <= self.t_end + 0.05)(
                self._stamp(r[0]))]
            if sel:
                inside, in_region = sel, True
        sm = [float(r[2]) for r in inside if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in inside if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i in range(4) if r[6 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(inside), "samples_in_region": in_region,
                "reasons": reasons}


def run_reference(args):
    """CPU arm: the reference algorithm (every interpolated state, every pair, cost mode)
    restated by the oracle, on all host cores, over a bounded sample per step."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle as O
    from isaac_sim_ros2_humble_gb300 import workloads as W
    robot, env, qf, qt = W.edge_workload(n_edges=args.edges)
    m = O.OracleModel(robot, env)
    per = 256
    cores = O.num_threads()
    times, checks = [], []
    for it in range(args.warmup + args.steps):
        lo = (it * per) % (len(qf) - per)
        t0 = time.perf_counter()
        ok, fh, ns, ln = m.check_motions(qf[lo:lo + per], qt[lo:lo + per], STEP, RULE, early_exit=False)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
            checks.append(int(ns.sum()))
    value = sum(checks) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "edges_per_step": per, "step_rule": "linf", "resolution": STEP,
                       "l2_flush": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per} edges per step of the 65,536-edge batch, reference algorithm "
                                       f"(all states, all pairs, cost mode), OpenMP"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline(robot, env, qf, qt):
    import oracle as O
    m = O.OracleModel(robot, env)
    n = CPU_SAMPLE_EDGES
    m.check_motions(qf[:4], qt[:4], STEP, RULE, early_exit=False)
    t0 = time.perf_counter()
    ok, fh, ns, ln = m.check_motions(qf[:n], qt[:n], STEP, RULE, early_exit=False)
    dt = time.perf_counter() - t0
    return {"value": float(ns.sum()) / dt, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"first {n} of the 65,536 edges ({int(ns.sum())} states), reference algorithm "
                      f"(all states, all pairs, cost mode), OpenMP, {dt:.1f} s"}


def _pct(v, p):
    return float(np.percentile(v, p)) if len(v) else None


# ---------------------------------------------------------------------------------------
# Secondary workloads (rank 0, one GPU).  Each returns a dict with its own metric, unit,
# direction, config and clock record.
# ---------------------------------------------------------------------------------------
def bench_plain(args, flush, fp32_peak):
    """Plain batched FK + collision: 4,096 configurations of a 7-DOF revolute arm (59
    spheres, all-pairs self mask without adjacent links) against 32 obstacle spheres and
    8 axis-aligned boxes; one collision flag plus the link poses per configuration, both
    from one launch (gbmp_check_states_fk)."""
    import torch
    import oracle as O
    from isaac_sim_ros2_humble_gb300 import _lib, api, roofline, workloads as W
    robot, env, q = W.plain_check_workload(n=4096)
    R, E = api.Robot(robot), api.Env(env)
    n, L = q.shape
    d_q = torch.from_numpy(q).cuda()
    verdict = torch.zeros(n, dtype=torch.uint8, device="cuda")
    poses = torch.zeros((n, L, 16), device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        api.check_states(R, E, d_q, verdict=verdict, poses=poses)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    # The kernel takes tens of microseconds, less than the host needs to issue a step, so
    # steps are timed in blocks of 100 issued behind a 20 ms device sleep: the host is
    # ahead when the block starts and no step waits for its launch.
    block = 100
    steps = max(2000, args.steps) // block * block
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    clk = ClockSampler(torch.cuda.current_device()).start()
    _lib.profile_reset()
    launches0 = _lib.launch_count()
    torch.cuda.synchronize()
    clk.mark_begin()
    _lib.profile_enable(True)
    for b0 in range(0, steps, block):
        torch.cuda._sleep(int(0.02 * 2.0e9))   # ~20 ms at ~2 GHz
        for i in range(b0, b0 + block):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    clk.mark_end()
    _lib.profile_enable(False)
    clocks = clk.stop()
    launches = _lib.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    k_ms, k_launches = _lib.profile_read(_lib.PROF_CHECK_STATES)
    k_ms_per = k_ms / max(k_launches, 1)
    _lib.work_counting(True)
    step()
    torch.cuda.synchronize()
    exec_flops, exec_states = _lib.work_read()
    _lib.work_counting(False)
    flops_state = roofline.flops_per_state(robot, env, R.P)
    # end to end: configurations from pinned host memory, flags and poses back
    h_q = torch.from_numpy(q).pin_memory()
    h_v = torch.empty(n, dtype=torch.uint8).pin_memory()
    h_p = torch.empty((n, L, 16), dtype=torch.float32).pin_memory()
    e2e_ms = []
    for i in range(3 + min(steps, 200)):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_q.copy_(h_q, non_blocking=True)
        step()
        h_v.copy_(verdict, non_blocking=True)
        h_p.copy_(poses, non_blocking=True)
        torch.cuda.synchronize()
        if i >= 3:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    ms = float(np.median(step_ms))
    out = {"metric": "FK+collision checks/s", "value": n / (ms / 1e3), "unit": "configs/s",
           "higher_is_better": True, "ms_per_step": ms, "steps": steps,
           "config": {"workload": "plain_fk_collision_7dof_4096", "configs": n, "dof": robot.dim, "links": L,
                      "robot_spheres": robot.num_spheres, "self_pairs": R.P,
                      "obstacles": {"spheres": env.counts[0], "boxes": env.counts[1]},
                      "outputs": "collision flag + 4x4 link poses per configuration, one launch",
                      "colliding": int(verdict.sum().item()), "l2_flush": "384 MB buffer written between steps",
                      "timing": "CUDA events around each launch, steps issued in blocks of 100 behind a 20 ms "
                                "device sleep so that no step waits for the host"},
           "e2e": {"value": n / (float(np.median(e2e_ms)) / 1e3), "unit": "configs/s",
                   "h2d_bytes_per_step": int(n * L * 4), "d2h_bytes_per_step": int(n + n * L * 64),
                   "ms_per_step": float(np.median(e2e_ms))},
           "roofline": {"bound": "fp32", "kernel": "k_check_states", "unit": "TFLOP/s", "peak": fp32_peak,
                        "achieved": exec_flops / (k_ms_per / 1e3) / 1e12 if k_ms_per > 0 else None,
                        "achieved_is": "flops executed by k_check_states (counted in-kernel in an untimed step) / "
                                       "its device time",
                        "effective": n * flops_state / (k_ms_per / 1e3) / 1e12 if k_ms_per > 0 else None,
                        "effective_is": "reference-equivalent work (all pairs of every configuration) / its device "
                                        "time",
                        "flops_per_config": flops_state, "executed_flops_per_launch": exec_flops,
                        "kernel_ms": k_ms_per, "hbm_bytes_algorithmic": int(n * (L * 4 + L * 64 + 1))},
           "gpu_launches": int(launches), "clocks": clocks}
    rf = out["roofline"]
    rf["frac"] = rf["achieved"] / fp32_peak if rf["achieved"] and fp32_peak else None
    rf["effective_frac"] = rf["effective"] / fp32_peak if rf["effective"] and fp32_peak else None
    if not args.no_cpu_baseline:
        m = O.OracleModel(robot, env)
        m.check_states(q[:64])
        t0 = time.perf_counter()
        m.check_states(q)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "configs/s", "cores": O.num_threads(), "kind": "port",
                               "sample": f"all {n} configurations, reference algorithm (FK, every pair, cost mode), "
                                         f"OpenMP, {dt * 1e3:.1f} ms"}
    return out


def gpu_problem_set(n_seeds, R, robot, api, W, torch):
    """Seeded shelf problems with collision-free start/goal whose direct edge collides,
    selected with the GPU checker (product path)."""
    envs, problems = {}, []
    for seed in range(n_seeds):
        sc = seed % 10
        if sc not in envs:
            env = W.shelf_env(sc)
            envs[sc] = (env, api.Env(env))
        env, E = envs[sc]

        def checker(q, E=E):
            v = torch.zeros(q.shape[0], dtype=torch.uint8, device="cuda")
            api.check_states(R, E, torch.from_numpy(q).cuda(), verdict=v)
            return v.cpu().numpy() == 0

        def edge_free(a, b, E=E):
            ok = torch.zeros(1, dtype=torch.uint8, device="cuda")
            api.check_edges(R, E, torch.from_numpy(a[None].copy()).cuda(), torch.from_numpy(b[None].copy()).cuda(),
                            PLAN_RES, RULE, ok)
            return bool(ok.item())

        _, _, free = W.planning_workload(seed, checker, robot=robot, env=env)
        start, goal = W.pick_problem(free, edge_free, seed)
        problems.append((seed, sc, start, goal))
    return envs, problems


def bench_fk(args, flush):
    """Forward kinematics alone (the reference's generated FK kernel): 1,048,576 states of
    the 8-DOF benchmark arm, 4x4 link poses and sphere centres written out.  Timed twice
    on the same inputs: the table-driven kernel (tables staged in shared memory) and the
    kernel generated for this robot at run time (NVRTC, every
    constant a literal, one thread per state).  Both write the same bytes; the bound is
    HBM.  The table-driven kernel takes chunks of 10 consecutive states per warp (the
    chunk FK of edge validation) and writes each chunk's poses as one contiguous block."""
    import torch
    from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W
    robot, _, _, _ = W.edge_workload(n_edges=16)
    n = args.fk_states
    q = torch.from_numpy(robot.sample_full(np.random.default_rng(7), n)).cuda()
    L, S = robot.num_links, robot.num_spheres
    poses = torch.empty((n, L, 16), device="cuda")
    centers = torch.empty((n, S, 3), device="cuda")
    nbytes = n * (4 * L + 64 * L + 12 * S)
    peak = _hbm_peak()
    out = {}
    for name, cg in (("table", False), ("generated", True)):
        R = api.Robot(robot, codegen=cg)
        info = R.codegen_info() if cg else None
        for _ in range(max(3, args.warmup)):
            api.fk(R, q, poses, centers)
        torch.cuda.synchronize()
        ms = []
        clk = ClockSampler(torch.cuda.current_device()).start()
        clk.mark_begin()
        for i in range(max(10, min(args.steps, 50))):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            api.fk(R, q, poses, centers)
            b.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        clk.mark_end()
        t = float(np.median(ms))
        out[name] = {"ms": t, "states_per_s": n / (t / 1e3), "hbm_gbs": nbytes / (t / 1e3) / 1e9,
                     "frac_of_measured_hbm": nbytes / (t / 1e3) / 1e9 / peak if peak else None,
                     "clocks": clk.stop()}
        if info:
            out[name]["nvrtc_ms"] = info.get("compile_ms")
            out[name]["cache"] = info.get("cache")
        torch.cuda.synchronize()
    best = min(out, key=lambda k: out[k]["ms"])
    return {"metric": "FK states/s", "value": out["table"]["states_per_s"], "unit": "states/s",
            "higher_is_better": True, "ms_per_step": out["table"]["ms"],
            "config": {"workload": f"fk_8dof_110spheres_{n}_states", "states": n, "links": L, "spheres": S,
                       "bytes_per_state": nbytes // n, "l2_flush": "384 MB buffer written between steps",
                       "faster": best, "per_kernel": out},
            "roofline": {"bound": "hbm", "achieved": out["table"]["hbm_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": out["table"]["frac_of_measured_hbm"],
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)"},
            "clocks": out["table"]["clocks"]}


def _hbm_peak():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except Exception:
        return 6800.0   # the recipe's fallback figure


def bench_check_batch(args, flush):
    """Uneven checking instances: 256 state-check requests over 4 robots (6-9 DOF, 40-115
    spheres) and 16 scenes (50-500 obstacles), sizes log-uniform in 1..65,536 states (the
    serving mix's check requests).  One batched launch (gbmp_check_batch_run: a
    descriptor per request, blocks staging their own request's tables) against the plain
    path, one gbmp_check_states launch per request back to back on the same stream.  Both
    are device-timed with CUDA events around the whole set; outputs are compared."""
    import torch
    from isaac_sim_ros2_humble_gb300 import api, workloads as W
    robots = [W.serial_arm(80 + i, dof=6 + i, n_spheres=40 + 25 * i, prismatic_torso=i >= 2, resolution=0.01)
              for i in range(4)]
    envs = [W.random_env(90 + k, *(lambda O: (O - round(O * 80 / 336), round(O * 64 / 336), round(O * 16 / 336)))
                         (50 + 30 * k), oriented=True) for k in range(16)]
    R = [api.Robot(r) for r in robots]
    E = [api.Env(e) for e in envs]
    g = np.random.default_rng(17)
    reqs, total = [], 0
    for _ in range(256):
        i, k = int(g.integers(4)), int(g.integers(16))
        n = int(min(65536, np.exp(g.uniform(0, np.log(65536)))))
        q = torch.from_numpy(robots[i].sample_full(g, n)).cuda()
        reqs.append(dict(robot=R[i], env=E[k], q=q, verdict=torch.zeros(n, dtype=torch.uint8, device="cuda")))
        total += n
    plain_v = [torch.zeros_like(r["verdict"]) for r in reqs]
    cb = api.CheckBatch(max_requests=len(reqs))

    def batched():
        cb.run(reqs)

    def plain():
        for r, v in zip(reqs, plain_v):
            api.check_states(r["robot"], r["env"], r["q"], verdict=v)

    out = {}
    clk = ClockSampler(torch.cuda.current_device()).start()
    clk.mark_begin()
    for name, fn in (("batched", batched), ("plain", plain)):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        ms = []
        for i in range(max(5, min(args.steps, 20))):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        out[name] = float(np.median(ms))
    clk.mark_end()
    same = all(torch.equal(r["verdict"], v) for r, v in zip(reqs, plain_v))
    cb.close()
    return {"metric": "uneven check batch throughput", "value": total / (out["batched"] / 1e3), "unit": "states/s",
            "higher_is_better": True, "ms_per_step": out["batched"], "speedup_vs_plain": out["plain"] / out["batched"],
            "config": {"workload": "check_batch_4robots_16scenes_256_requests", "requests": len(reqs),
                       "states": total, "plain_ms": out["plain"], "verdicts_identical": bool(same),
                       "l2_flush": "384 MB buffer written between steps",
                       "timing": "CUDA events around the whole set of requests"},
            "clocks": clk.stop()}


def bench_plan(args, flush):
    """Single-problem parallel RRT-Connect: time to first solution over seeded shelf
    problems (7-DOF arm, 5 slabs + 40 boxes), for several lane counts."""
    import torch
    import oracle as O
    from isaac_sim_ros2_humble_gb300 import api, workloads as W
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    R = api.Robot(robot)
    envs, problems = gpu_problem_set(args.plan_seeds, R, robot, api, W, torch)
    planner = api.Planner(R, max_nodes=1_000_000, path_cap=65536)
    lanes_list = [int(x) for x in args.lanes.split(",")]
    per_lanes = {}
    clk = ClockSampler(torch.cuda.current_device()).start()
    clk.mark_begin()
    for lanes in lanes_list:
        for seed, sc, start, goal in problems[: max(args.warmup, 3)]:
            planner.solve(envs[sc][1], start, goal, lanes=lanes, range_=PLAN_RANGE, resolution=PLAN_RES, rule=RULE,
                          seed=seed)
        ms, costs, ok, kms = [], [], 0, []
        for seed, sc, start, goal in problems:
            flush.fill_(float(seed))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res, path = planner.solve(envs[sc][1], start, goal, lanes=lanes, range_=PLAN_RANGE, resolution=PLAN_RES,
                                      rule=RULE, seed=seed, time_limit_s=10.0)
            ms.append((time.perf_counter() - t0) * 1e3)
            kms.append(res["kernel_ms"])
            if res["solved"]:
                ok += 1
                costs.append(res["cost"])
        per_lanes[str(lanes)] = {"p50_ms": _pct(ms, 50), "p95_ms": _pct(ms, 95), "p99_ms": _pct(ms, 99),
                                 "mean_ms": float(np.mean(ms)), "kernel_p50_ms": _pct(kms, 50),
                                 "success": ok / len(problems),
                                 "path_length_mean": float(np.mean(costs)) if costs else None,
                                 "path_length_p50": _pct(costs, 50)}
    clk.mark_end()
    clocks = clk.stop()
    best = min(per_lanes, key=lambda k: per_lanes[k]["p50_ms"])
    out = {"metric": "plan time to solution p50", "value": per_lanes[best]["p50_ms"], "unit": "ms",
           "higher_is_better": False, "p99_ms": per_lanes[best]["p99_ms"], "steps": len(problems),
           "config": {"workload": f"rrtc_shelf_7dof_{len(problems)}_seeds", "best_lanes": int(best),
                      "range": PLAN_RANGE, "resolution": PLAN_RES, "step_rule": "linf", "max_nodes": 1_000_000,
                      "timing": "host wall time of each gbmp_rrtc_solve call (reset, launch, path read back); "
                                "L2 flushed before each solve",
                      "per_lanes": per_lanes},
           "clocks": clocks}
    if not args.no_cpu_baseline:
        k = min(10, len(problems))
        t_cpu, c_cpu, s_cpu = [], [], 0
        for seed, sc, start, goal in problems[:k]:
            m = O.OracleModel(robot, envs[sc][0])
            t0 = time.perf_counter()
            r_, p_ = O.rrtc(m, start, goal, range_=PLAN_RANGE, res=PLAN_RES, rule=RULE, seed=seed,
                            max_nodes=200_000, max_iters=200_000)
            t_cpu.append((time.perf_counter() - t0) * 1e3)
            s_cpu += r_["solved"]
            if r_["solved"]:
                c_cpu.append(r_["cost"])
        out["cpu_baseline"] = {"value": _pct(t_cpu, 50), "unit": "ms", "cores": 1, "kind": "port",
                               "sample": f"first {k} problems, sequential RRT-Connect with the same primitives "
                                         f"(oracle), success {s_cpu}/{k}, path length mean "
                                         f"{float(np.mean(c_cpu)) if c_cpu else None}"}
    return out


def bench_batch(args, flush):
    """Uneven batch: 256 heterogeneous planning problems (DOF 6-9, 30-120 spheres,
    10-500 obstacles) in one persistent, graph-captured launch with autotuned lanes per
    problem, against 256 sequential plain single-problem solves on the same GPU."""
    import torch
    from isaac_sim_ros2_humble_gb300 import api, workloads as W
    n = 256

    def feasible(robot, env):
        R_, E_ = api.Robot(robot), api.Env(env)
        q = robot.sample_full(np.random.default_rng(0), 2000)
        v = torch.zeros(q.shape[0], dtype=torch.uint8, device="cuda")
        api.check_states(R_, E_, torch.from_numpy(q).cuda(), verdict=v)
        return float((v == 0).float().mean().item()) >= 0.02

    models = W.uneven_batch_models(0, n=n, feasible=feasible)
    problems = []
    for i, (robot, env) in enumerate(models):
        R, E = api.Robot(robot), api.Env(env)

        def checker(q, R=R, E=E):
            v = torch.zeros(q.shape[0], dtype=torch.uint8, device="cuda")
            api.check_states(R, E, torch.from_numpy(q).cuda(), verdict=v)
            return v.cpu().numpy() == 0

        def edge_free(a, b, R=R, E=E):
            ok = torch.zeros(1, dtype=torch.uint8, device="cuda")
            api.check_edges(R, E, torch.from_numpy(a[None].copy()).cuda(), torch.from_numpy(b[None].copy()).cuda(),
                            PLAN_RES, RULE, ok)
            return bool(ok.item())

        _, _, free = W.planning_workload(i, checker, robot=robot, env=env, max_draws=40000)
        s0, g0 = W.pick_problem(free, edge_free, i)
        problems.append((R, E, s0, g0, 1000 + i))
    kw = dict(range_=PLAN_RANGE, resolution=PLAN_RES, rule=RULE, time_limit_s=10.0)
    bp = api.BatchPlanner(max_problems=n, max_nodes=32768, max_links=16, path_cap=4096)
    # lanes per problem chosen by the library's launch-shape autotuner on the batch itself
    # (gbmp_rrtc_solve_batch_auto: each candidate twice, then the fastest is kept)
    api.BatchPlanner.autotune_reset()
    tune_calls, tune, best = 0, {}, -1
    while tune_calls < 20:
        bp.solve(problems, lanes_per_problem="auto", use_graph=True, **kw)
        tune_calls += 1
        tune, best = api.BatchPlanner.autotune_record(problems, use_graph=True, **kw)
        if best is not None and best >= 0:
            break
    steps = max(3, min(args.steps, 5))
    clk = ClockSampler(torch.cuda.current_device()).start()
    times, solved = [], []
    for rep in range(max(args.warmup, 1) + steps):
        flush.fill_(float(rep))
        torch.cuda.synchronize()
        if rep == max(args.warmup, 1):
            clk.mark_begin()
        t0 = time.perf_counter()
        out = bp.solve(problems, lanes_per_problem="auto", use_graph=True, **kw)
        if rep >= max(args.warmup, 1):
            times.append((time.perf_counter() - t0) * 1e3)
            solved.append(sum(r["solved"] for r, _ in out))
    clk.mark_end()
    clocks = clk.stop()
    batch_ms = float(np.median(times))
    # plain path: sequential single-problem solves
    solved_mask = [bool(r["solved"]) for r, _ in out]
    plain, plain_each = {}, {}
    clk2 = ClockSampler(torch.cuda.current_device()).start()
    clk2.mark_begin()
    for lanes in (1024, 64):
        planners = {}
        s_plain = 0
        each = []
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for (R, E, s0, g0, seed) in problems:
            pl = planners.get(id(R))
            if pl is None:
                pl = planners[id(R)] = api.Planner(R, max_nodes=32768, path_cap=4096)
            t1 = time.perf_counter()
            r, p = pl.solve(E, s0, g0, lanes=lanes, seed=seed, **kw)
            each.append(((time.perf_counter() - t1) * 1e3, bool(r["solved"])))
            s_plain += r["solved"]
        plain[lanes] = ((time.perf_counter() - t0) * 1e3, s_plain)
        plain_each[lanes] = each
        del planners
    clk2.mark_end()
    clocks_plain = clk2.stop()
    plain_best = min(plain, key=lambda k: plain[k][0])
    plain_ms = plain[plain_best][0]
    # Split by outcome.  A problem without a path ends only when its trees are full, on
    # either path, with the same nearest-node scans: those problems set a floor that
    # batching cannot remove.  The batched call is re-timed on the problems it solved so
    # that the batching gain on solvable work is reported beside the whole-batch figure.
    sub = [p for p, ok in zip(problems, solved_mask) if ok]
    bp.solve(sub, lanes_per_problem=best, use_graph=True, **kw)
    t_sub = []
    for rep in range(3):
        flush.fill_(float(rep))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bp.solve(sub, lanes_per_problem=best, use_graph=True, **kw)
        t_sub.append((time.perf_counter() - t0) * 1e3)
    batch_solved_ms = float(np.median(t_sub))
    each = plain_each[plain_best]
    plain_solved_ms = sum(t for (t, _), ok in zip(each, solved_mask) if ok)
    plain_unsolved_ms = sum(t for (t, _), ok in zip(each, solved_mask) if not ok)
    return {"metric": "uneven-batch planning throughput", "value": n / (batch_ms / 1e3), "unit": "problems/s",
            "higher_is_better": True, "ms_per_step": batch_ms, "steps": steps,
            "speedup_vs_plain": plain_ms / batch_ms,
            "config": {"workload": "uneven_batch_256_rrtc", "problems": n, "lanes_per_problem": best,
                       "autotune_ms": {str(k): v for k, v in tune.items()}, "autotune_calls": tune_calls,
                       "autotuner": "gbmp_rrtc_solve_batch_auto (in libgbmp, keyed by the batch shape)",
                       "solved_batched": int(np.median(solved)), "graph": True,
                       "plain_sequential_ms": plain_ms, "plain_lanes": plain_best,
                       "plain_solved": plain[plain_best][1],
                       "plain_all": {str(k): list(v) for k, v in plain.items()},
                       "plain_clocks": clocks_plain,
                       "by_outcome": {"unsolved_in_batch": n - len(sub),
                                      "plain_ms_on_unsolved": plain_unsolved_ms,
                                      "plain_ms_on_solved": plain_solved_ms,
                                      "batched_ms_on_solved": batch_solved_ms,
                                      "speedup_on_solved": plain_solved_ms / batch_solved_ms},
                       "timing": "host wall time of each batched call; plain = the 256 single solves back to back"},
            "clocks": clocks}


def bench_serve(args):
    """Serving: Poisson request stream over 4 resident robots (6-9 DOF) and 16 resident
    scenes (50-500 obstacles); 70 % FK+collision requests of log-uniform 1-65,536 states,
    30 % RRT-Connect plan requests.  The continuous-batching server against the plain
    per-request path (one request at a time, in arrival order)."""
    import torch
    from isaac_sim_ros2_humble_gb300 import api, workloads as W
    robots = [W.serial_arm(80 + i, dof=6 + i, n_spheres=40 + 25 * i, prismatic_torso=i >= 2, resolution=0.01)
              for i in range(4)]
    envs = [W.random_env(90 + k, *(lambda O: (O - round(O * 80 / 336), round(O * 64 / 336), round(O * 16 / 336)))
                         (50 + 30 * k), oriented=True) for k in range(16)]
    R = [api.Robot(r) for r in robots]
    E = [api.Env(e) for e in envs]
    rng = np.random.default_rng(5)
    pools = [r.sample_full(rng, 65536) for r in robots]
    free = {}
    for i in range(4):
        for k in range(16):
            v = torch.zeros(4096, dtype=torch.uint8, device="cuda")
            api.check_states(R[i], E[k], torch.from_numpy(pools[i][:4096]).cuda(), verdict=v)
            f = pools[i][:4096][v.cpu().numpy() == 0]
            free[(i, k)] = f if len(f) >= 2 else None

    def make_stream(rate, seed):
        g = np.random.default_rng(seed)
        t, out = 0.0, []
        while t < args.duration:
            t += g.exponential(1.0 / rate)
            i, k = int(g.integers(4)), int(g.integers(16))
            if g.random() < 0.7 or free[(i, k)] is None:
                n = int(min(65536, np.exp(g.uniform(0, np.log(65536)))))
                off = int(g.integers(0, 65536 - n + 1))
                out.append((t, "check", i, k, (off, n)))
            else:
                f = free[(i, k)]
                a, b = g.choice(len(f), 2, replace=False)
                out.append((t, "plan", i, k, (f[a], f[b], int(g.integers(1 << 30)))))
        return out

    def run_served(stream):
        srv = api.Server(num_streams=4, hbm_budget_bytes=8 << 30, max_batch_states=1 << 21, plan_workers=2,
                         plan_batch=64, plan_lanes=16, planner_max_nodes=32768, plan_path_cap=4096,
                         plan_range=PLAN_RANGE, plan_resolution=PLAN_RES, step_rule=RULE)
        for r in R:
            srv.add_robot(r)
        for e in E:
            srv.add_env(e)
        srv.start()
        tickets = []
        t0 = time.perf_counter()
        for (ta, kind, i, k, d) in stream:
            dt = ta - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            if kind == "check":
                off, n = d
                out = np.zeros(n, np.uint8)
                tickets.append(("check", srv.submit_check(i, k, pools[i][off:off + n], out)))
            else:
                path = np.zeros((4096, robots[i].num_links), np.float32)
                tickets.append(("plan", srv.submit_plan(i, k, d[0], d[1], d[2], path)))
        lat = {"check": [], "plan": []}
        for kind, t in tickets:
            info = srv.wait(t, 120.0)
            lat[kind].append(info["latency_ms"])
        el = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        return lat, el, st

    def run_plain(stream):
        planners = [api.Planner(r, max_nodes=32768, path_cap=4096) for r in R]
        lat = {"check": [], "plan": []}
        t0 = time.perf_counter()
        for (ta, kind, i, k, d) in stream:
            now = time.perf_counter() - t0
            if now < ta:
                time.sleep(ta - now)
            if kind == "check":
                off, n = d
                q = torch.from_numpy(pools[i][off:off + n]).cuda(non_blocking=False)
                v = torch.zeros(n, dtype=torch.uint8, device="cuda")
                api.check_states(R[i], E[k], q, verdict=v)
                v.cpu()
            else:
                planners[i].solve(E[k], d[0], d[1], lanes=1024, range_=PLAN_RANGE, resolution=PLAN_RES, rule=RULE,
                                  seed=d[2])
            lat[kind].append((time.perf_counter() - t0 - ta) * 1e3)
        return lat, time.perf_counter() - t0

    per_rate = {}
    clk = ClockSampler(torch.cuda.current_device()).start()
    run_served(make_stream(200.0, 1)[: 50])          # warm-up
    clk.mark_begin()
    for rate in [float(x) for x in args.rates.split(",")]:
        stream = make_stream(rate, int(rate))
        lat_s, el_s, st = run_served(stream)
        lat_p, el_p = run_plain(stream)
        all_s = lat_s["check"] + lat_s["plan"]
        all_p = lat_p["check"] + lat_p["plan"]
        per_rate[str(int(rate))] = {
            "requests": len(stream), "offered_rps": len(stream) / args.duration,
            "served_throughput_rps": len(stream) / el_s,
            "plain_throughput_rps": len(stream) / el_p,
            "served": {"p50_ms": _pct(all_s, 50), "p95_ms": _pct(all_s, 95), "p99_ms": _pct(all_s, 99),
                       "check_p99_ms": _pct(lat_s["check"], 99), "plan_p99_ms": _pct(lat_s["plan"], 99)},
            "plain": {"p50_ms": _pct(all_p, 50), "p95_ms": _pct(all_p, 95), "p99_ms": _pct(all_p, 99),
                      "check_p99_ms": _pct(lat_p["check"], 99), "plan_p99_ms": _pct(lat_p["plan"], 99)},
            "check_batches": st["batches"], "plan_batches": st["plan_batches"]}
    clk.mark_end()
    clocks = clk.stop()
    top = per_rate[max(per_rate, key=lambda k: float(k))]
    return {"metric": "served p99 latency at the highest rate", "value": top["served"]["p99_ms"], "unit": "ms",
            "higher_is_better": False, "p50_ms": top["served"]["p50_ms"], "p95_ms": top["served"]["p95_ms"],
            "served_throughput_rps": top["served_throughput_rps"],
            "plain_throughput_rps": top["plain_throughput_rps"],
            "throughput_vs_plain": top["served_throughput_rps"] / top["plain_throughput_rps"],
            # a served stream cannot finish faster than it arrives: this is the largest
            # throughput ratio the offered rate allows
            "throughput_vs_plain_cap": top["offered_rps"] / top["plain_throughput_rps"],
            "p99_vs_plain": top["plain"]["p99_ms"] / top["served"]["p99_ms"],
            "steps": sum(v["requests"] for v in per_rate.values()),
            "config": {"workload": "serving_4robots_16scenes_70check_30plan", "duration_s": args.duration,
                       "rates": args.rates, "per_rate": per_rate,
                       "timing": "host wall time from a request's scheduled arrival to its completion; the "
                                 "served and plain paths replay the same stream"},
            "clocks": clocks}


def _standalone_line(d, args):
    """A secondary workload as a line of its own (--workload plain|plan|batch|serve)."""
    line = {"metric": d["metric"], "value": d["value"], "unit": d["unit"], "n_gpus": 1,
            "steps": d.get("steps", args.steps), "warmup": args.warmup, "ms_per_step": d.get("ms_per_step"),
            "higher_is_better": d["higher_is_better"], "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)"}
    line.update({k: v for k, v in d.items() if k not in line})
    return line


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist

    from isaac_sim_ros2_humble_gb300 import _lib, api, roofline, workloads as W

    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    if args.workload in ("plain", "fk", "checkbatch", "plan", "batch", "serve"):
        if rank != 0:
            return 0
        fn = {"plain": lambda: bench_plain(args, flush, _lib.measure_fp32_peak(1.0)),
              "fk": lambda: bench_fk(args, flush),
              "checkbatch": lambda: bench_check_batch(args, flush),
              "plan": lambda: bench_plan(args, flush), "batch": lambda: bench_batch(args, flush),
              "serve": lambda: bench_serve(args)}[args.workload]
        print(json.dumps(_standalone_line(fn(), args)), flush=True)
        return 0

    robot, env, qf, qt = W.edge_workload(n_edges=args.edges, shard=rank)
    R, E = api.Robot(robot), api.Env(env)
    L = robot.num_links
    n = qf.shape[0]
    d_from = torch.from_numpy(qf).to(dev)
    d_to = torch.from_numpy(qt).to(dev)
    ok = torch.zeros(n, dtype=torch.uint8, device=dev)
    fh = torch.zeros(n, dtype=torch.int32, device=dev)
    ln = torch.zeros(n, device=dev)
    ns = torch.zeros(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()

    # The timed call asks for what the reference's checkMotions returns (a verdict and the
    # motion cost per edge), so the edges are walked coarse to fine; the call that also
    # returns each edge's first colliding state walks them in state order and is timed
    # beside it (`with_first_hit`).
    def step():
        api.check_edges(R, E, d_from, d_to, STEP, RULE, ok, None, ln, ns)

    def step_first_hit():
        api.check_edges(R, E, d_from, d_to, STEP, RULE, ok, fh, ln, ns)

    fp32_peak = _lib.measure_fp32_peak(1.0)
    for _ in range(max(args.warmup, 3)):
        step_first_hit()
    torch.cuda.synchronize()
    ok_first_hit = ok.clone()
    checks = int(ns.sum().item())
    units_first_hit = roofline.edge_units(fh.cpu().numpy(), ns.cpu().numpy())
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if not torch.equal(ok, ok_first_hit):
        raise RuntimeError("verdicts of the two chunk orders differ")

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clk = ClockSampler(torch.cuda.current_device())
    _lib.profile_reset()
    launches0 = _lib.launch_count()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clk.start()
    clk.mark_begin()
    _lib.profile_enable(True)
    for i in range(args.steps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    clk.mark_end()
    _lib.profile_enable(False)
    if ws > 1:
        dist.barrier()
    clocks = clk.stop()
    launches = _lib.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    wave_ms, wave_launches = _lib.profile_read(_lib.PROF_EDGE_WAVE)
    # executed work of one step (counted in an extra, untimed step: counting adds work)
    _lib.work_counting(True)
    step()
    torch.cuda.synchronize()
    exec_flops, exec_states = _lib.work_read()
    _lib.work_counting(False)
    units = exec_states
    total_s = sum(step_ms) / 1e3

    # the same edges with first hits (state order), same timing
    fh_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    _lib.profile_reset()
    _lib.profile_enable(True)
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.fill_(float(i))
        fh_ev[i][0].record(stream)
        step_first_hit()
        fh_ev[i][1].record(stream)
    torch.cuda.synchronize()
    _lib.profile_enable(False)
    fh_wave_ms, _ = _lib.profile_read(_lib.PROF_EDGE_WAVE)
    fh_total_s = sum(a.elapsed_time(b) for a, b in fh_ev) / 1e3
    _lib.work_counting(True)
    step_first_hit()
    torch.cuda.synchronize()
    _, fh_exec_states = _lib.work_read()
    _lib.work_counting(False)

    # end-to-end through the same C-ABI call with host buffers
    h_from = torch.from_numpy(qf).pin_memory()
    h_to = torch.from_numpy(qt).pin_memory()
    h_ok = torch.empty(n, dtype=torch.uint8).pin_memory()
    h_ln = torch.empty(n, dtype=torch.float32).pin_memory()
    e2e_ms = []
    for i in range(max(args.warmup, 3) + args.steps):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_from.copy_(h_from, non_blocking=True)
        d_to.copy_(h_to, non_blocking=True)
        step()
        h_ok.copy_(ok, non_blocking=True)
        h_ln.copy_(ln, non_blocking=True)
        torch.cuda.synchronize()
        if i >= max(args.warmup, 3):
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_s = sum(e2e_ms) / 1e3
    total_s, all_checks, e2e_s = reduce_over_ranks(dist, ws, dev, total_s, checks, e2e_s)
    value = all_checks * args.steps / total_s
    e2e_value = all_checks * args.steps / e2e_s

    if rank == 0:
        flops_state = roofline.flops_per_state(robot, env, R.P)
        wave_s_per_step = wave_ms / 1e3 / args.steps
        achieved = exec_flops / wave_s_per_step / 1e12 if wave_s_per_step > 0 else None
        effective = units * flops_state / wave_s_per_step / 1e12 if wave_s_per_step > 0 else None
        traffic = None
        kernel = "k_edge_chunk"
        tp = os.path.join(ROOT, "profiles", f"{kernel}_traffic.json")
        if os.path.exists(tp):
            try:
                traffic = json.load(open(tp)).get("bytes_per_launch")
            except Exception:
                traffic = None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "edges": n, "dof": robot.dim, "links": L,
                       "robot_spheres": robot.num_spheres, "self_pairs": R.P,
                       "obstacles": {"spheres": env.counts[0], "oriented_boxes": env.counts[1],
                                     "cylinders": env.counts[2]},
                       "resolution": STEP, "step_rule": "linf", "states_per_step": checks,
                       "outputs": "verdict + motion cost per edge (checkMotions' outputs); states walked coarse "
                                  "to fine, stopping at any colliding state",
                       "states_evaluated_per_step": exec_states, "edges_free": int(ok.sum().item()),
                       "edges_per_s": n * ws * args.steps / total_s,
                       "l2_flush": "384 MB buffer written between timed steps",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(2 * n * L * 4),
                    "d2h_bytes_per_step": int(n * (1 + 4)), "ms_per_step": 1e3 * e2e_s / args.steps},
            "with_first_hit": {"value": checks * args.steps / fh_total_s, "unit": UNIT,
                               "ms_per_step": 1e3 * fh_total_s / args.steps,
                               "kernel_ms_per_step": fh_wave_ms / args.steps,
                               "states_evaluated_per_step": fh_exec_states,
                               "states_needed_per_step": units_first_hit,
                               "outputs": "verdict, lowest colliding state index and motion cost per edge; "
                                          "states walked in order, stopping at the first colliding one"},
            "roofline": {"bound": "fp32", "kernel": kernel, "achieved": achieved, "peak": fp32_peak,
                         "unit": "TFLOP/s", "frac": (achieved / fp32_peak) if achieved and fp32_peak else None,
                         "traffic": traffic,
                         "peak_source": "measured FP32 FMA throughput (gbmp_measure_fp32_peak) on this GPU; "
                                        "MEASURED_PEAKS.json has no FP32 CUDA-core figure",
                         "nominal_peak": roofline.nominal_fp32_tflops(),
                         "achieved_is": f"flops executed by {kernel} (counted in-kernel in an untimed step) / "
                                        f"{kernel} time",
                         "executed_flops_per_step": exec_flops, "states_evaluated_per_step": exec_states,
                         "effective": effective, "effective_frac": (effective / fp32_peak) if effective else None,
                         "effective_is": "reference-equivalent work (full pair tests of every evaluated state, "
                                         f"flops_per_state x units_per_step) / {kernel} time",
                         "flops_per_state": flops_state, "units_per_step": units,
                         "kernel_ms_per_step": wave_ms / args.steps,
                         "kernel_launches_per_step": wave_launches / args.steps},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(robot, env, qf, qt)
        if args.workload == "all" and ws == 1:
            sec = {}
            for name, fn in (("plain_fk_collision", lambda: bench_plain(args, flush, fp32_peak)),
                             ("fk", lambda: bench_fk(args, flush)),
                             ("check_batch", lambda: bench_check_batch(args, flush)),
                             ("plan", lambda: bench_plan(args, flush)),
                             ("uneven_batch", lambda: bench_batch(args, flush)),
                             ("serving", lambda: bench_serve(args))):
                t0 = time.perf_counter()
                try:
                    sec[name] = fn()
                except Exception as e:   # a failed secondary workload is reported, not hidden
                    sec[name] = {"error": f"{type(e).__name__}: {e}"}
                sec[name]["wall_s"] = time.perf_counter() - t0
            line["secondary"] = sec
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
