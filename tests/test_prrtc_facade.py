"""The pRRTC interface include/gbmp_prrtc.hpp (pRRTC::solve<Robot>, pRRTC_settings,
PlannerResult and the ppln::collision shapes over the C-ABI) compiles against gbmp.h and
libgbmp, and a C++ program calling it the way pRRTC's scripts do plans in a scene of
spheres, capsules, z-aligned capsules, oriented cuboids and z-aligned cuboids with
several goals.  The returned path is re-validated here against the original shapes
(segment distance for capsules, axis projections for cuboids), not against the
converted scene the library plans in, so the conversion is checked too."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from isaac_sim_ros2_humble_gb300 import workloads as W
from test_cudampl_facade import ROOT, _cuda_home, _read_results

SRC = os.path.join(ROOT, "tests", "cpp", "prrtc_facade_check.cpp")
GRAN, RANGE = 16, 0.3
BAND = 1e-4


def build_prrtc_check(out_dir):
    from isaac_sim_ros2_humble_gb300 import _lib
    cuda = _cuda_home()
    if cuda is None:
        pytest.skip("no CUDA headers")
    _lib.load()
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = os.path.join(str(out_dir), "prrtc_facade_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), SRC, "-o", exe, "-L", libdir, "-lgbmp",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{libdir}",
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_prrtc_facade_compiles_and_links(tmp_path):
    exe = build_prrtc_check(tmp_path)
    assert os.access(exe, os.X_OK)


def _scene():
    """pRRTC shapes: the shelf's boxes as cuboids (axes = rotation columns, half
    extents), two spheres, two capsules, a z-aligned capsule and a rotated z-aligned
    cuboid beside the shelf."""
    shelf = W.shelf_env(0)
    cub = []
    for p, R, lo, hi in zip(shelf.box_pos, shelf.box_rot, shelf.box_min, shelf.box_max):
        c = p + R @ ((lo + hi) / 2)
        h = (hi - lo) / 2
        cub.append([*c, *R[:, 0], *R[:, 1], *R[:, 2], *h])
    sph = [[0.2, 0.6, 0.9, 0.08], [0.3, -0.6, 0.2, 0.1]]
    cap = [[0.1, 0.55, 0.1, 0.0, 0.0, 0.6, 0.05], [0.25, -0.5, 1.1, 0.2, 0.25, 0.0, 0.04]]
    zcap = [[-0.3, 0.4, 0.0, 0.0, 0.0, 0.9, 0.06]]
    a = 0.5
    zcub = [[-0.35, -0.45, 0.4, np.cos(a), np.sin(a), 0.0, -np.sin(a), np.cos(a), 0.0, 0.0, 0.0, 1.0,
             0.08, 0.05, 0.3]]
    return np.array(sph, np.float32), np.array(cap, np.float32), np.array(zcap, np.float32), \
        np.array(cub, np.float32), np.array(zcub, np.float32)


def _as_env(sph, cap, zcap, cub, zcub):
    """The same scene as libgbmp spheres / boxes / cylinders (used only to draw
    collision-free start and goals; the path check below uses the original shapes)."""
    sp, sr, bp, br, bmn, bmx, cp, cr, crad, ch = [], [], [], [], [], [], [], [], [], []
    for x, y, z, r in sph:
        sp.append([x, y, z]); sr.append(r)
    caps = [c for c in cap] + [[c[0], c[1], c[2], 0.0, 0.0, c[5], c[6]] for c in zcap]
    for x1, y1, z1, xv, yv, zv, r in caps:
        a, v = np.array([x1, y1, z1]), np.array([xv, yv, zv])
        sp += [a, a + v]; sr += [r, r]
        zax = v / np.linalg.norm(v)
        u = np.array([0.0, 1.0, 0.0]) if abs(zax[0]) > 0.9 else np.array([1.0, 0.0, 0.0])
        xax = np.cross(u, zax); xax /= np.linalg.norm(xax)
        cp.append(a + v / 2); cr.append(np.stack([xax, np.cross(zax, xax), zax], 1)); crad.append(r)
        ch.append(np.linalg.norm(v))
    for row in list(cub) + [[*c[:3], c[3], c[4], 0, c[6], c[7], 0, 0, 0, 1, *c[12:]] for c in zcub]:
        bp.append(row[:3]); br.append(np.stack([row[3:6], row[6:9], row[9:12]], 1))
        bmn.append(-np.asarray(row[12:15])); bmx.append(np.asarray(row[12:15]))
    f = lambda a, s: np.asarray(a, np.float32).reshape(s)
    return W.Environment(f(sp, (-1, 3)), f(sr, (-1,)), f(bp, (-1, 3)), f(br, (-1, 3, 3)), f(bmn, (-1, 3)),
                         f(bmx, (-1, 3)), f(cp, (-1, 3)), f(cr, (-1, 3, 3)), f(crad, (-1,)), f(ch, (-1,)))


def _penetration(cen, rad, sph, cap, zcap, cub, zcub):
    """Deepest penetration of any robot sphere into any original shape, per state."""
    c = cen[:, :, None, :]                      # [n, S, 1, 3]
    r = rad[None, :, None]
    worst = np.full(cen.shape[0], -np.inf)
    if len(sph):
        d = np.linalg.norm(c - sph[None, None, :, :3], axis=-1)
        worst = np.maximum(worst, (r + sph[None, None, :, 3] - d).max(axis=(1, 2)))
    caps = np.concatenate([cap, np.c_[zcap[:, :3], np.zeros((len(zcap), 2)), zcap[:, 5:]]]) if len(zcap) else cap
    if len(caps):
        a, v, cr = caps[:, :3], caps[:, 3:6], caps[:, 6]
        t = np.clip(((c - a) * v).sum(-1) / (v * v).sum(-1), 0, 1)
        d = np.linalg.norm(c - (a + t[..., None] * v), axis=-1)
        worst = np.maximum(worst, (r + cr - d).max(axis=(1, 2)))
    zc = np.array([[*z[:3], z[3], z[4], 0, z[6], z[7], 0, 0, 0, 1, *z[12:]] for z in zcub], np.float64)
    boxes = np.concatenate([cub, zc]) if len(zc) else cub
    if len(boxes):
        rel = c - boxes[:, :3]
        e = [np.maximum(0, np.abs((rel * boxes[:, 3 + 3 * k:6 + 3 * k]).sum(-1)) - boxes[:, 12 + k]) for k in range(3)]
        d = np.sqrt(e[0] ** 2 + e[1] ** 2 + e[2] ** 2)
        worst = np.maximum(worst, (r - d).max(axis=(1, 2)))
    return worst


def _write(path, robot, shapes, start, goals, settings):
    f = lambda a: " ".join("%.9g" % v for v in np.asarray(a, np.float64).ravel())
    i = lambda a: " ".join(str(int(v)) for v in np.asarray(a).ravel())
    act = robot.active.astype(bool)
    lines = [f"{robot.num_links} {robot.dim} {robot.num_spheres}", i(robot.joint_types), f(robot.joint_poses),
             f(robot.joint_axes), i(robot.parent), i(robot.sphere_link), f(robot.sphere_pos), f(robot.sphere_r),
             i(robot.active), f(robot.lower), f(robot.upper), f(robot.default), i(robot.enables)]
    for arr in shapes:
        lines.append(str(len(arr)))
        lines += [f(row) for row in arr]
    lines += [f(start[act]), str(len(goals))] + [f(g[act]) for g in goals] + [" ".join(str(x) for x in settings)]
    with open(path, "w") as fp:
        fp.write("\n".join(lines) + "\n")


@pytest.mark.gpu
def test_prrtc_solve_multi_goal_path_is_valid(tmp_path):
    exe = build_prrtc_check(tmp_path)
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    shapes = _scene()
    m = O.OracleModel(robot, _as_env(*shapes))
    checker = lambda q: m.check_states(q)[1] == 0
    edge_free = lambda a, b: bool(m.check_motions(a[None], b[None], 0.01, 1)[0][0])
    _, _, free = W.planning_workload(3, checker, robot=robot, env=_as_env(*shapes))
    start, g0 = W.pick_problem(free, edge_free, 3)
    rng = np.random.default_rng(7)
    goals = [g0] + [free[k] for k in rng.choice(len(free), 2, replace=False)]
    prob, resf = tmp_path / "p.txt", tmp_path / "r.txt"
    _write(prob, robot, shapes, start, goals, (200000, 200000, 512, GRAN, RANGE))
    r = subprocess.run([exe, str(prob), str(resf)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = _read_results(resf)
    assert int(got["solved"][0]) == 1
    act = robot.active.astype(bool)
    path_a = got["path"].astype(np.float32).reshape(-1, robot.dim)
    n_states = int(got["sizes"][2])
    assert len(path_a) == n_states >= 2
    full = np.tile(robot.default.astype(np.float32), (len(path_a), 1))
    full[:, act] = path_a
    np.testing.assert_array_equal(full[0], start.astype(np.float32))
    assert any(np.array_equal(full[-1], g.astype(np.float32)) for g in goals)   # ends at one of the goals
    seg = np.linalg.norm(np.diff(path_a, axis=0), axis=1)
    assert np.all(seg <= RANGE + 1e-5)
    assert got["cost"][0] == pytest.approx(float(seg.sum()), rel=1e-4)
    # every state the planner checked (k / GRAN of each edge, k = 1..GRAN), against the
    # original shapes and the robot's own self pairs
    k = np.arange(1, GRAN + 1, dtype=np.float32)[:, None] / np.float32(GRAN)
    states = np.concatenate([a + k * (b - a) for a, b in zip(full[:-1], full[1:])]).astype(np.float32)
    cen = m.sphere_centers(m.fk(states.astype(np.float64), f64=True))
    pen = _penetration(cen, robot.sphere_r.astype(np.float64), *[s.astype(np.float64) for s in shapes])
    assert pen.max() <= BAND, pen.max()
    self_only = O.OracleModel(robot)
    assert np.all(self_only.clearance(states) > -BAND)


def test_scene_conversion_matches_prrtc_collision(tmp_path):
    """The scene the header builds from a pRRTC environment (gbmp_prrtc_detail::
    scene_arrays, printed by a program without device work) collides, by the oracle,
    with the same robot configurations as pRRTC's own sphere_environment_in_collision
    (pRRTC/src/planning/utils.cuh, compiled for the host over the reference's shape
    types) says, but for configurations within 1e-4 m of contact."""
    import shutil
    import ref_build
    if not ref_build.prrtc_available() or shutil.which("g++") is None:
        pytest.skip("pRRTC sources or g++ not present")
    exe = tmp_path / "dump"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "prrtc_scene_dump.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    shapes = _scene()
    f = lambda a: " ".join("%.9g" % v for v in np.asarray(a, np.float64).ravel())
    lines = []
    for arr in shapes:
        lines.append(str(len(arr)))
        lines += [f(row) for row in arr]
    (tmp_path / "s.txt").write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(exe), str(tmp_path / "s.txt"), str(tmp_path / "o.txt")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = _read_results(tmp_path / "o.txt")
    f32 = lambda k, s: np.asarray(got[k], np.float32).reshape(s)
    env = W.Environment(f32("sph_pos", (-1, 3)), f32("sph_r", (-1,)), f32("box_pos", (-1, 3)),
                        f32("box_rot", (-1, 3, 3)), f32("box_min", (-1, 3)), f32("box_max", (-1, 3)),
                        f32("cyl_pos", (-1, 3)), f32("cyl_rot", (-1, 3, 3)), f32("cyl_r", (-1,)), f32("cyl_h", (-1,)))
    robot = W.serial_arm(1, dof=7, n_spheres=59, name="arm7")
    m = O.OracleModel(robot, env)
    q = robot.sample_full(np.random.default_rng(0), 3000)
    oc, _ = m.check_states(q)
    env_hit = (oc[1] + oc[2] + oc[3]) > 0
    cen = np.ascontiguousarray(m.sphere_centers(m.fk(q)), np.float32)
    rad = np.ascontiguousarray(robot.sphere_r, np.float32)
    c = lambda a: np.ascontiguousarray(a, np.float32).reshape(-1)
    sph, cap, zcap, cub, zcub = shapes
    out = np.zeros(len(q), np.uint8)
    ref_build.prrtc_collision().ref_prrtc_collide(len(q), robot.num_spheres, c(cen), rad, len(sph), c(sph), len(cap),
                                                  c(cap), len(zcap), c(zcap), len(cub), c(cub), len(zcub), c(zcub), out)
    assert 0.1 < env_hit.mean() < 0.9
    bad = (out != 0) != env_hit
    pen = _penetration(cen.astype(np.float64), rad.astype(np.float64), *[s.astype(np.float64) for s in shapes])
    assert np.all(np.abs(pen[bad]) <= BAND), (bad.sum(), np.abs(pen[bad]).max() if bad.any() else 0)
