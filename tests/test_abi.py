"""The C-ABI library loads and exports every entry point of include/gbmp.h, and its
argument validation answers without a GPU (no compute calls here)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from isaac_sim_ros2_humble_gb300 import _lib, workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if hdr.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", hdr)).read()
            names += re.findall(r"^GBMP_API\s+[\w\s\*]+?\b(gbmp_\w+)\s*\(", txt, flags=re.M)
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 18
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (gbmp_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_status_strings_and_limits():
    lib = _lib.load()
    assert lib.gbmp_status_string(0) == b"ok"
    assert lib.gbmp_status_string(1) == b"invalid argument"
    lim = _lib.Limits()
    _lib.check(lib.gbmp_get_limits(C.byref(lim)))
    assert lim.max_links >= 16 and lim.max_spheres >= 128


def _desc(model, parent=None):
    keep = [np.ascontiguousarray(model.joint_types, np.int32),
            np.ascontiguousarray(model.joint_poses.reshape(-1, 16), np.float32),
            np.ascontiguousarray(model.joint_axes, np.float32),
            np.ascontiguousarray(model.parent if parent is None else parent, np.int32),
            np.ascontiguousarray(model.sphere_link, np.int32), np.ascontiguousarray(model.sphere_pos, np.float32),
            np.ascontiguousarray(model.sphere_r, np.float32), np.ascontiguousarray(model.active, np.uint8),
            np.ascontiguousarray(model.lower, np.float32), np.ascontiguousarray(model.upper, np.float32),
            np.ascontiguousarray(model.default, np.float32), np.ascontiguousarray(model.enables, np.uint8)]
    d = _lib.RobotDesc(model.num_links, *(k.ctypes.data for k in keep[:4]), model.num_spheres,
                       *(k.ctypes.data for k in keep[4:]), float(model.resolution))
    return d, keep


def test_invalid_parent_map_rejected_like_reference():
    """SingleArmSpace.cu:63-69 throws when parent[i] >= i; the C-ABI returns
    GBMP_ERR_INVALID_ARGUMENT with the same message."""
    lib = _lib.load()
    model = W.serial_arm(1, dof=3, n_spheres=6)
    bad = model.parent.copy()
    bad[2] = 2
    d, keep = _desc(model, bad)
    h = C.c_void_p()
    st = lib.gbmp_robot_create(C.byref(d), 0, C.byref(h))
    assert st == 1
    assert b"Link parent link map is not valid at index 2" in lib.gbmp_last_error()
    assert not h.value
    with pytest.raises(_lib.GbmpError):
        _lib.check(st)


def test_other_invalid_descriptors():
    lib = _lib.load()
    model = W.serial_arm(1, dof=3, n_spheres=6)
    d, keep = _desc(model)
    h = C.c_void_p()
    d.resolution = 0.0
    assert lib.gbmp_robot_create(C.byref(d), 0, C.byref(h)) == 1
    d.resolution = 0.02
    d.num_links = 0
    assert lib.gbmp_robot_create(C.byref(d), 0, C.byref(h)) == 1
    d.num_links = 1000
    assert lib.gbmp_robot_create(C.byref(d), 0, C.byref(h)) == 1
    d.num_links = model.num_links
    sl = keep[4].copy()
    sl[0] = 99
    d.sphere_link = sl.ctypes.data
    assert lib.gbmp_robot_create(C.byref(d), 0, C.byref(h)) == 1
    assert lib.gbmp_robot_create(None, 0, C.byref(h)) == 1
    assert lib.gbmp_env_create(-1, None, None, 0, None, None, None, None, 0, None, None, None, None,
                               C.byref(h)) == 1
    assert lib.gbmp_env_create(1, None, None, 0, None, None, None, None, 0, None, None, None, None,
                               C.byref(h)) == 1
    # NULL handles are rejected, not dereferenced
    assert lib.gbmp_check_states(None, None, None, 1, 0, None, None, None, None) == 1
    assert lib.gbmp_check_edges(None, None, None, None, 1, 0.0, 0, None, None, None, None, None) == 1
    assert lib.gbmp_robot_destroy(None) == 0


def test_struct_layouts_match_ctypes(tmp_path):
    """Every struct of the C-ABI has the size and field offsets the ctypes binding
    declares (gcc compiles a program that prints them from include/gbmp.h)."""
    import shutil
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    pairs = {"gbmp_robot_desc": _lib.RobotDesc, "gbmp_limits": _lib.Limits, "gbmp_projection": _lib.Projection,
             "gbmp_rrtc_settings": _lib.RrtcSettings, "gbmp_rrtc_result": _lib.RrtcResult,
             "gbmp_rrtc_problem": _lib.RrtcProblem, "gbmp_server_config": _lib.ServerConfig,
             "gbmp_request_info": _lib.RequestInfo, "gbmp_server_metrics": _lib.ServerMetrics,
             "gbmp_check_request": _lib.CheckRequest}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gbmp.h"', "int main(void) {"]
    for cname, cls in pairs.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", inc, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (ln.split() for ln in out if ln)}
    for cname, cls in pairs.items():
        assert got[(cname, "sizeof")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_kernel_setup_is_recorded_per_device(tmp_path):
    """The record of kernels whose shared-memory limit was raised is keyed by (device,
    kernel): configuring a kernel on one device does not count for another."""
    exe = tmp_path / "devset_check"
    src = os.path.join(ROOT, "tests", "cpp", "devset_check.cpp")
    inc = os.path.join(ROOT, "isaac_sim_ros2_humble_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", inc, src, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "devset ok" in out.stdout


def test_edge_state_orders_cover_every_state_once(tmp_path):
    """The orders in which edge validation visits an edge's states (csrc/gbmp_order.h,
    compiled here for the host): every state of every edge length up to 6,000 exactly
    once, for both chunk sizes; state order from the start; coarse to fine with the first
    4 states, then the last chunk, then the chunks between pass by pass in bit-reversed
    offset order; the state-by-state form a permutation starting with the first and last
    states."""
    exe = tmp_path / "order_check"
    src = os.path.join(ROOT, "tests", "cpp", "order_check.cpp")
    inc = os.path.join(ROOT, "isaac_sim_ros2_humble_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", inc, src, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "order ok" in out.stdout


def test_sphere_groups_split_links_within_the_group_limit(tmp_path):
    """The robots' sphere groups (csrc/gbmp_groups.h, compiled here for the host): one
    group per link for the per-state kernels; pieces of links for the chunk kernels, each
    within one link, at most M spheres (M the smallest size from the piece up within the
    group limit), following the link's longest extent, in link order."""
    exe = tmp_path / "groups_check"
    src = os.path.join(ROOT, "tests", "cpp", "groups_check.cpp")
    inc = os.path.join(ROOT, "isaac_sim_ros2_humble_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", inc, src, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "groups ok" in out.stdout


def test_batch_autotuner_policy_with_a_fake_timer(tmp_path):
    """The batched planner's launch-shape tuner (csrc/gbmp_autotune.h), driven by a fake
    timer: each allowed candidate tried twice in order, the least time of each kept, the
    fastest chosen and kept per shape key, keys independent, lane limits respected, and
    concurrent callers agreeing on one decision."""
    exe = tmp_path / "autotune_check"
    src = os.path.join(ROOT, "tests", "cpp", "autotune_check.cpp")
    inc = os.path.join(ROOT, "isaac_sim_ros2_humble_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", inc, src, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "autotune ok" in out.stdout
