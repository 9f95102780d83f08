"""gbmp_check_edges_noalloc, called through the C-ABI, gives the results of
gbmp_check_edges on two calls in a row, takes no device memory, and refuses calls
larger than its fixed scratch.  Collected last so that it also runs after every other
GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

from isaac_sim_ros2_humble_gb300 import _lib, api, workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_EDGES = 65536
MAX_EDGE_LINKS = 1 << 20
CAPACITY = 5   # GBMP_ERR_CAPACITY


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def outputs(n):
    return (torch.zeros(n, dtype=torch.uint8, device="cuda"), torch.zeros(n, dtype=torch.int32, device="cuda"),
            torch.zeros(n, dtype=torch.float32, device="cuda"), torch.zeros(n, dtype=torch.int32, device="cuda"))


def call(fn, R, E, qf, qt, res, rule, outs):
    n = qf.shape[0]
    st = fn(R.handle, E.handle, _lib.ptr(qf), _lib.ptr(qt), n, float(res), rule, *(_lib.ptr(o) for o in outs),
            _lib.stream_handle(None))
    return st


def host(outs):
    return [o.cpu().numpy() for o in outs]


@pytest.fixture(scope="module")
def cases():
    lib = _lib.load()
    robot, env, qf, qt = W.edge_workload(n_edges=6000)
    R, E = api.Robot(robot), api.Env(env)
    # a second robot / scene / size, so that the second call reuses the scratch with
    # different extents
    arm = W.serial_arm(5, dof=7, n_spheres=59)
    shelf = W.shelf_env(6)
    rng = np.random.default_rng(12)
    af, at = arm.sample_full(rng, 1500), arm.sample_full(rng, 1500)
    return lib, [(R, E, dev(qf), dev(qt), 0.01, _lib.STEP_L2), (api.Robot(arm), api.Env(shelf), dev(af), dev(at),
                                                                    0.05, _lib.STEP_LINF)]


def test_noalloc_matches_check_edges_on_two_calls(cases):
    lib, cs = cases
    expect = []
    for R, E, qf, qt, res, rule in cs:
        outs = outputs(qf.shape[0])
        _lib.check(call(lib.gbmp_check_edges, R, E, qf, qt, res, rule, outs))
        expect.append(host(outs))
    torch.cuda.synchronize()
    assert any(not e[0].all() for e in expect) and any(e[0].any() for e in expect)
    # two calls in a row, each against the existing entry point's results (same kernels:
    # bit-exact), then the first case again after the second one changed the scratch
    for k in (0, 1, 0):
        R, E, qf, qt, res, rule = cs[k]
        outs = outputs(qf.shape[0])
        _lib.check(call(lib.gbmp_check_edges_noalloc, R, E, qf, qt, res, rule, outs))
        got = host(outs)
        for g, e in zip(got, expect[k]):
            np.testing.assert_array_equal(g, e)


def test_noalloc_takes_no_device_memory(cases):
    """A robot handle that only ever sees the allocation-free entry point: after the
    per-device set-up call (no edges), neither its first real call nor later ones take
    device memory.  The module fixture already ran gbmp_check_edges with a robot of the
    same tables, so the kernels this call uses are loaded."""
    lib, cs = cases
    _, E, qf, qt, res, rule = cs[0]
    robot, _, _, _ = W.edge_workload(n_edges=8)
    R = api.Robot(robot)
    outs = outputs(qf.shape[0])
    torch.cuda.synchronize()
    assert lib.gbmp_check_edges_noalloc(R.handle, E.handle, None, None, 0, 0.01, rule, None, None, None, None,
                                        None) == _lib.OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _lib.check(call(lib.gbmp_check_edges_noalloc, R, E, qf, qt, res, rule, outs))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "the first call took device memory"
    for _ in range(2):
        _lib.check(call(lib.gbmp_check_edges_noalloc, R, E, qf, qt, res, rule, outs))
    torch.cuda.synchronize()
    free2, _ = torch.cuda.mem_get_info()
    assert free2 == free0, "later calls took device memory"


def test_noalloc_rejects_calls_beyond_its_scratch(cases):
    lib, cs = cases
    R, E = cs[0][0], cs[0][1]
    f = lib.gbmp_check_edges_noalloc
    # edge count beyond the scratch: refused before any pointer is read
    st = f(R.handle, E.handle, None, None, MAX_EDGES + 1, 0.01, 0, None, None, None, None, None)
    assert st == CAPACITY
    assert b"allocation-free scratch" in lib.gbmp_last_error()
    # edges x links beyond the scratch with an edge count that alone would fit
    wide = W.serial_arm(8, dof=20, n_spheres=40)
    Rw = api.Robot(wide)
    n = MAX_EDGE_LINKS // wide.num_links + 1
    assert n <= MAX_EDGES
    st = f(Rw.handle, E.handle, None, None, n, 0.01, 0, None, None, None, None, None)
    assert st == CAPACITY
    # zero edges: only the per-device set-up
    assert f(R.handle, E.handle, None, None, 0, 0.01, 0, None, None, None, None, None) == _lib.OK
