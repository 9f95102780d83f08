"""Algorithmic work per checked state (the roofline numerator).

Counting rule: multiply, add, subtract, compare, min, max = 1 flop; fused
multiply-add = 2 flops; sqrt / sin / cos are counted separately as SFU ops.

Per state (the reference's full, no-early-exit work):
  FK        revolute 151 (Rodrigues ~25 + two 3x4 products of 63), prismatic 129
            (3 + 2 x 63), fixed 63, base link 0
  spheres   18 per sphere (3x4 transform of a point)
  self      9 per enabled pair (3 sub, 1 mul + 2 fma, compare)
  env       per (robot sphere, obstacle): sphere 11, cuboid 33, cylinder 34
The unit count of a launch is the number of states that have to be checked to
produce the outputs: for edge validation, the states of every edge up to and
including its first colliding state (all states of a free edge).
"""
from __future__ import annotations

import numpy as np

FK_FLOPS = {1: 151, 2: 129, 5: 63}
SPHERE_XFORM = 18
SELF_PAIR = 9
ENV_PAIR = {"sphere": 11, "cuboid": 33, "cylinder": 34}


def flops_per_state(robot, env, n_self_pairs: int) -> int:
    fk = sum(FK_FLOPS.get(int(t), 0) for t in robot.joint_types[1:])
    ns, nb, nc = env.counts
    S = robot.num_spheres
    env_f = S * (ns * ENV_PAIR["sphere"] + nb * ENV_PAIR["cuboid"] + nc * ENV_PAIR["cylinder"])
    return int(fk + S * SPHERE_XFORM + n_self_pairs * SELF_PAIR + env_f)


def sfu_per_state(robot, env) -> int:
    rev = int(np.sum(robot.joint_types[1:] == 1))
    return 2 * rev + 2 * robot.num_spheres * env.counts[2]


def edge_units(first_hit: np.ndarray, num_steps: np.ndarray) -> int:
    """States needed per edge: up to and including the first hit, else all."""
    fh = np.asarray(first_hit, np.int64)
    ns = np.asarray(num_steps, np.int64)
    return int(np.where(fh >= 0, fh + 1, ns).sum())


def nominal_fp32_tflops(num_sms: int = 152, sm_mhz: float = 2070.0) -> float:
    """128 FP32 lanes per SM, one FMA (2 flops) per lane per clock."""
    return num_sms * 128 * 2 * sm_mhz * 1e6 / 1e12
