"""Pins the oracle to the reference's own code: the FK, edge-step and interpolation
kernels that cudampl/CUDAMPLib/include/spaces/KernelGenerator.h generates for a robot
are compiled for the CPU (oracle/ref_build.py) and compared with the oracle's
restatement.  Skipped where the reference tree is absent."""
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
