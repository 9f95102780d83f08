"""Robot models, environments and seeded synthetic workloads.

The tables follow the reference's robot description contract
(src/foliation_planner/include/foliation_planner/robot_info.hpp:13-310, consumed by
cudampl/CUDAMPLib/src/spaces/SingleArmSpace.cu:10-161): one joint per link, joint i
drives link i, parent[i] < i, joint types 1 revolute / 2 prismatic / 5 fixed, joint
origins as row-major 4x4 poses in the parent link frame, collision spheres attached
to links, an active-joint map and per-joint limits and defaults.

Every generator is seeded (numpy PCG64) and deterministic, so the CUDA path, the CPU
oracle and the CPU baseline see identical inputs.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional

import numpy as np

REVOLUTE, PRISMATIC, FIXED = 1, 2, 5


@dataclasses.dataclass
class RobotModel:
    name: str
    joint_types: np.ndarray      # int32 [L]
    joint_poses: np.ndarray      # float32 [L,4,4]
    joint_axes: np.ndarray       # float32 [L,3]
    parent: np.ndarray           # int32 [L]
    sphere_link: np.ndarray      # int32 [S]
    sphere_pos: np.ndarray       # float32 [S,3]
    sphere_r: np.ndarray         # float32 [S]
    active: np.ndarray           # uint8 [L]
    lower: np.ndarray            # float32 [L]
    upper: np.ndarray            # float32 [L]
    default: np.ndarray          # float32 [L]
    enables: np.ndarray          # uint8 [L,L] self-collision link-pair mask
    link_names: List[str]
    resolution: float = 0.02

    @property
    def num_links(self) -> int:
        return int(self.joint_types.shape[0])

    @property
    def num_spheres(self) -> int:
        return int(self.sphere_r.shape[0])

    @property
    def dim(self) -> int:
        return int(self.active.sum())

    def full_from_active(self, q_active: np.ndarray) -> np.ndarray:
        """Expand [N, dim] active-joint vectors to [N, L] full vectors with defaults
        (cudampl/CUDAMPLib/src/spaces/SingleArmSpace.cu:436-497)."""
        q_active = np.asarray(q_active, dtype=np.float32).reshape(-1, self.dim)
        out = np.broadcast_to(self.default, (q_active.shape[0], self.num_links)).copy()
        out[:, self.active.astype(bool)] = q_active
        return out

    def active_from_full(self, q_full: np.ndarray) -> np.ndarray:
        return np.asarray(q_full, dtype=np.float32)[:, self.active.astype(bool)]

    def sample_full(self, rng: np.random.Generator, n: int) -> np.ndarray:
        u = rng.random((n, self.num_links), dtype=np.float32)
        q = self.lower + u * (self.upper - self.lower)
        inactive = ~self.active.astype(bool)
        q[:, inactive] = self.default[inactive]
        return q.astype(np.float32)


@dataclasses.dataclass
class Environment:
    sphere_pos: np.ndarray       # float32 [ns,3]
    sphere_r: np.ndarray         # float32 [ns]
    box_pos: np.ndarray          # float32 [nb,3]
    box_rot: np.ndarray          # float32 [nb,3,3] row-major rotation
    box_min: np.ndarray          # float32 [nb,3] in the box frame
    box_max: np.ndarray          # float32 [nb,3]
    cyl_pos: np.ndarray          # float32 [nc,3]
    cyl_rot: np.ndarray          # float32 [nc,3,3]
    cyl_radius: np.ndarray       # float32 [nc]
    cyl_height: np.ndarray       # float32 [nc] full height along local z

    @property
    def counts(self):
        return (len(self.sphere_r), len(self.box_pos), len(self.cyl_radius))

    @staticmethod
    def empty() -> "Environment":
        z3 = np.zeros((0, 3), np.float32)
        z33 = np.zeros((0, 3, 3), np.float32)
        z = np.zeros((0,), np.float32)
        return Environment(z3, z, z3, z33, z3, z3, z3, z33, z, z)

    def subset(self, ns: int, nb: int, nc: int) -> "Environment":
        return Environment(self.sphere_pos[:ns], self.sphere_r[:ns], self.box_pos[:nb],
                           self.box_rot[:nb], self.box_min[:nb], self.box_max[:nb],
                           self.cyl_pos[:nc], self.cyl_rot[:nc], self.cyl_radius[:nc],
                           self.cyl_height[:nc])


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _unit(rng: np.random.Generator) -> np.ndarray:
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def serial_arm(seed: int, dof: int = 7, n_spheres: int = 59, prismatic_torso: bool = False,
               offset_range=(0.05, 0.35), radius_range=(0.03, 0.08), limit: float = 2.8,
               torso_range=(0.0, 0.4), resolution: float = 0.02, name: Optional[str] = None,
               vertical_base: bool = True) -> RobotModel:
    """A serial arm with random link transforms.

    Link 0 is the fixed base.  Joint i (i >= 1) sits at a random offset of
    |t| in offset_range from the origin of link i-1 with a random orientation, and
    turns about a random unit axis (or slides along one for the prismatic torso).
    Collision spheres are spread over links 1..L-1 along the segment from the link
    origin to the next joint origin, radii in radius_range.  Self-collision is
    enabled for every link pair except a link with itself or its parent.
    """
    rng = np.random.default_rng(seed)
    n_moving = dof
    L = n_moving + 1
    types = np.full(L, REVOLUTE, np.int32)
    types[0] = FIXED
    if prismatic_torso:
        types[1] = PRISMATIC
    poses = np.tile(np.eye(4, dtype=np.float64), (L, 1, 1))
    axes = np.zeros((L, 3), np.float64)
    axes[0] = (0, 0, 1)
    for i in range(1, L):
        if i == 1 and vertical_base:
            R = np.eye(3)
            t = np.array([0.0, 0.0, rng.uniform(*offset_range)])
            ax = np.array([0.0, 0.0, 1.0])
        else:
            R = _random_rotation(rng)
            t = _unit(rng) * rng.uniform(*offset_range)
            ax = _unit(rng)
        poses[i, :3, :3] = R
        poses[i, :3, 3] = t
        axes[i] = ax
    parent = np.arange(-1, L - 1, dtype=np.int32)
    lower = np.full(L, -limit, np.float32)
    upper = np.full(L, limit, np.float32)
    lower[0] = upper[0] = 0.0
    if prismatic_torso:
        lower[1], upper[1] = torso_range
    active = np.ones(L, np.uint8)
    active[0] = 0
    default = np.zeros(L, np.float32)
    if prismatic_torso:
        default[1] = torso_range[0]

    # Segment of link i: from its origin to the next joint origin (expressed in link i);
    # the last link gets a short random tool segment.
    seg_end = np.zeros((L, 3))
    for i in range(1, L):
        if i + 1 < L:
            seg_end[i] = poses[i + 1, :3, 3]
        else:
            seg_end[i] = _unit(rng) * rng.uniform(*offset_range)
    moving = np.arange(1, L)
    counts = np.full(n_moving, n_spheres // n_moving)
    counts[: n_spheres % n_moving] += 1
    s_link, s_pos, s_r = [], [], []
    for li, cnt in zip(moving, counts):
        fr = np.linspace(0.15, 0.85, cnt) if cnt > 1 else np.array([0.5])
        for f in fr:
            s_link.append(li)
            s_pos.append(seg_end[li] * f + rng.normal(scale=0.005, size=3))
            s_r.append(rng.uniform(*radius_range))
    enables = np.ones((L, L), np.uint8)
    for i in range(L):
        enables[i, i] = 0
        if parent[i] >= 0:
            enables[i, parent[i]] = enables[parent[i], i] = 0
    robot = RobotModel(
        name=name or f"arm{dof}_s{seed}", joint_types=types, joint_poses=poses.astype(np.float32),
        joint_axes=axes.astype(np.float32), parent=parent,
        sphere_link=np.asarray(s_link, np.int32), sphere_pos=np.asarray(s_pos, np.float32),
        sphere_r=np.asarray(s_r, np.float32), active=active, lower=lower, upper=upper,
        default=default, enables=enables, link_names=[f"link_{i}" for i in range(L)],
        resolution=resolution)
    disable_default_collisions(robot, np.random.default_rng(seed + 7))
    return robot


def tree_robot(seed: int, n_spheres: int = 40) -> RobotModel:
    """A branching kinematic tree (torso with two 3-joint arms and a fixed head) mixing
    revolute, prismatic and fixed joints, with un-normalised joint axes; used to test
    general parent maps (parent[i] < i but not i - 1)."""
    rng = np.random.default_rng(seed)
    #          0 base, 1 torso(prism), 2 head(fixed), 3-5 left arm, 6-8 right arm, 9 tool(fixed)
    parent = np.array([-1, 0, 1, 1, 3, 4, 1, 6, 7, 5], np.int32)
    types = np.array([FIXED, PRISMATIC, FIXED, REVOLUTE, REVOLUTE, REVOLUTE, REVOLUTE, REVOLUTE,
                      REVOLUTE, FIXED], np.int32)
    L = len(parent)
    poses = np.tile(np.eye(4), (L, 1, 1))
    axes = np.zeros((L, 3))
    for i in range(1, L):
        poses[i, :3, :3] = _random_rotation(rng)
        poses[i, :3, 3] = _unit(rng) * rng.uniform(0.08, 0.3)
        axes[i] = _unit(rng) * rng.uniform(0.5, 2.0)         # not unit length
    lower = np.full(L, -2.8, np.float32)
    upper = np.full(L, 2.8, np.float32)
    lower[1], upper[1] = 0.0, 0.3
    active = (types != FIXED).astype(np.uint8)
    default = np.zeros(L, np.float32)
    lower[~active.astype(bool)] = upper[~active.astype(bool)] = 0.0
    carriers = [1, 2, 3, 4, 5, 6, 7, 8, 9]
    s_link = rng.choice(carriers, n_spheres).astype(np.int32)
    s_pos = rng.normal(scale=0.05, size=(n_spheres, 3))
    s_r = rng.uniform(0.02, 0.05, n_spheres)
    enables = np.ones((L, L), np.uint8)
    for i in range(L):
        enables[i, i] = 0
        if parent[i] >= 0:
            enables[i, parent[i]] = enables[parent[i], i] = 0
    robot = RobotModel(name=f"tree_s{seed}", joint_types=types, joint_poses=poses.astype(np.float32),
                       joint_axes=axes.astype(np.float32), parent=parent, sphere_link=s_link,
                       sphere_pos=s_pos.astype(np.float32), sphere_r=s_r.astype(np.float32), active=active,
                       lower=lower, upper=upper, default=default, enables=enables,
                       link_names=[f"link_{i}" for i in range(L)], resolution=0.02)
    disable_default_collisions(robot, np.random.default_rng(seed + 7))
    return robot


def fk_numpy(robot: RobotModel, q: np.ndarray) -> np.ndarray:
    """Float64 link poses [N, L, 4, 4] (host-side helper for scene generation)."""
    q = np.asarray(q, np.float64).reshape(-1, robot.num_links)
    N, L = q.shape
    P = np.zeros((N, L, 4, 4))
    P[:, 0] = np.eye(4)
    for i in range(1, L):
        J = robot.joint_poses[i].astype(np.float64)
        M = np.tile(np.eye(4), (N, 1, 1))
        if robot.joint_types[i] == REVOLUTE:
            a = robot.joint_axes[i].astype(np.float64)
            a = a / np.linalg.norm(a)                        # revolute axes are normalised
            c, s = np.cos(q[:, i]), np.sin(q[:, i])
            K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
            M[:, :3, :3] = (c[:, None, None] * np.eye(3) + s[:, None, None] * K
                            + (1 - c)[:, None, None] * np.outer(a, a))
        elif robot.joint_types[i] == PRISMATIC:
            M[:, :3, 3] = q[:, i, None] * robot.joint_axes[i].astype(np.float64)
        P[:, i] = P[:, robot.parent[i]] @ J @ M
    return P


def sphere_centers_numpy(robot: RobotModel, q: np.ndarray) -> np.ndarray:
    P = fk_numpy(robot, q)
    T = P[:, robot.sphere_link]                        # [N,S,4,4]
    return np.einsum("nsij,sj->nsi", T[:, :, :3, :3], robot.sphere_pos.astype(np.float64)) + T[:, :, :3, 3]


def disable_default_collisions(robot: RobotModel, rng: np.random.Generator, samples: int = 2000,
                               always: float = 0.25) -> None:
    """Disable self-collision checks between link pairs that collide in the default
    configuration or in at least `always` of random configurations (the way a MoveIt
    SRDF allowed-collision matrix drops "Default" and "Always" pairs; the threshold
    here also drops pairs that collide in a quarter of the joint space)."""
    q = np.concatenate([robot.default[None], robot.sample_full(rng, samples)])
    C = sphere_centers_numpy(robot, q)
    S, L = robot.num_spheres, robot.num_links
    hit = np.zeros((q.shape[0], L, L), bool)
    for i in range(S):
        d = np.linalg.norm(C[:, i, None, :] - C[:, i + 1:, :], axis=-1)
        coll = d < (robot.sphere_r[i] + robot.sphere_r[i + 1:])
        for j_off in range(coll.shape[1]):
            j = i + 1 + j_off
            a, b = robot.sphere_link[i], robot.sphere_link[j]
            if a != b:
                hit[:, a, b] |= coll[:, j_off]
                hit[:, b, a] |= coll[:, j_off]
    frac = hit[1:].mean(0)
    off = hit[0] | (frac >= always)
    robot.enables[off] = 0


SCENE_CENTER = (0.9, 0.0, 0.5)


def random_env(seed: int, n_spheres: int, n_boxes: int, n_cyl: int, center=SCENE_CENTER,
               size: float = 1.2, sphere_r=(0.05, 0.15), box_side=(0.05, 0.4), oriented: bool = False,
               cyl_r=(0.02, 0.1), cyl_h=(0.2, 1.0), keepout: float = 0.3) -> Environment:
    """Obstacles with centres uniform in a cube of edge `size` around `center`.

    The default cube (edge 1.2 m, centred 0.9 m in front of the base) overlaps about
    half of the arm's reach: roughly half of the uniformly drawn configurations of
    the benchmark arms collide, so batches mix free and colliding states.

    Obstacles whose bounding sphere reaches within `keepout` of the robot base
    (the origin) are redrawn, so the base itself is never in collision."""
    rng = np.random.default_rng(seed)
    c = np.asarray(center, np.float64)

    def draw_center(rad):
        while True:
            p = c + (rng.random(3) - 0.5) * size
            if np.linalg.norm(p) - rad > keepout:
                return p

    sp, sr = [], []
    for _ in range(n_spheres):
        r = rng.uniform(*sphere_r)
        sp.append(draw_center(r))
        sr.append(r)
    bp, brot, bmin, bmax = [], [], [], []
    for _ in range(n_boxes):
        half = rng.uniform(*box_side, size=3) * 0.5
        bp.append(draw_center(np.linalg.norm(half)))
        brot.append(_random_rotation(rng) if oriented else np.eye(3))
        bmin.append(-half)
        bmax.append(half)
    cp, crot, cr, ch = [], [], [], []
    for _ in range(n_cyl):
        r = rng.uniform(*cyl_r)
        h = rng.uniform(*cyl_h)
        cp.append(draw_center(np.hypot(r, h / 2)))
        crot.append(_random_rotation(rng))
        cr.append(r)
        ch.append(h)
    f = lambda a, shape: np.asarray(a, np.float32).reshape(shape)
    return Environment(f(sp, (-1, 3)), f(sr, (-1,)), f(bp, (-1, 3)), f(brot, (-1, 3, 3)),
                       f(bmin, (-1, 3)), f(bmax, (-1, 3)), f(cp, (-1, 3)), f(crot, (-1, 3, 3)),
                       f(cr, (-1,)), f(ch, (-1,)))


def shelf_env(seed: int, n_slabs: int = 5, slab=(0.8, 0.3, 0.02), spacing: float = 0.3,
              n_boxes: int = 40, front: float = 0.55, base_z: float = 0.1) -> Environment:
    """Shelf-like scene: n_slabs horizontal slabs spaced `spacing` apart in front of the
    robot plus random small boxes resting inside the shelf cells."""
    rng = np.random.default_rng(seed)
    bp, brot, bmin, bmax = [], [], [], []
    for k in range(n_slabs):
        bp.append([front + slab[1] / 2, 0.0, base_z + k * spacing])
        brot.append(np.eye(3))
        bmin.append([-slab[1] / 2, -slab[0] / 2, -slab[2] / 2])
        bmax.append([slab[1] / 2, slab[0] / 2, slab[2] / 2])
    for _ in range(n_boxes):
        cell = rng.integers(0, n_slabs - 1)
        half = rng.uniform(0.02, 0.06, size=3)
        x = front + rng.uniform(half[0], slab[1] - half[0])
        y = rng.uniform(-slab[0] / 2 + half[1], slab[0] / 2 - half[1])
        z = base_z + cell * spacing + slab[2] / 2 + half[2]
        bp.append([x, y, z])
        brot.append(np.eye(3))
        bmin.append(-half)
        bmax.append(half)
    e = Environment.empty()
    f = lambda a, shape: np.asarray(a, np.float32).reshape(shape)
    return dataclasses.replace(e, box_pos=f(bp, (-1, 3)), box_rot=f(brot, (-1, 3, 3)),
                               box_min=f(bmin, (-1, 3)), box_max=f(bmax, (-1, 3)))


# ---------------------------------------------------------------------------------
# Named workloads (sizes of the benchmark configurations).
# ---------------------------------------------------------------------------------

def plain_check_workload(seed: int = 1, n: int = 4096):
    """Batched FK + collision: 7-DOF revolute arm, 59 spheres, 32 obstacle spheres and
    8 axis-aligned boxes, n configurations uniform in the joint limits."""
    robot = serial_arm(seed, dof=7, n_spheres=59, name="arm7")
    env = random_env(seed + 100, n_spheres=32, n_boxes=8, n_cyl=0, oriented=False)
    q = robot.sample_full(np.random.default_rng(seed + 200), n)
    return robot, env, q


def edge_workload(seed: int = 2, n_edges: int = 65536, step: float = 0.01, shard: int = 0):
    """Edge validation: 8-DOF arm (prismatic torso 0-0.4 m + 7 revolute), 110 spheres,
    256 obstacle spheres, 64 oriented boxes, 16 cylinders; n_edges edges with
    endpoints uniform in the limits, interpolated at `step`.  `shard` selects an
    independent set of edges for the same robot and scene."""
    robot = serial_arm(seed, dof=8, n_spheres=110, prismatic_torso=True, name="arm8_torso",
                       resolution=step)
    env = random_env(seed + 100, n_spheres=256, n_boxes=64, n_cyl=16, oriented=True)
    rng = np.random.default_rng(seed + 200 + 7919 * shard)
    q_from = robot.sample_full(rng, n_edges)
    q_to = robot.sample_full(rng, n_edges)
    return robot, env, q_from, q_to


def planning_workload(seed: int, checker, robot: Optional[RobotModel] = None, env: Optional[Environment] = None,
                      resolution: float = 0.01, max_draws: int = 200000):
    """Single-problem RRT-Connect: the 7-DOF arm of plain_check_workload in the shelf scene
    (5 slabs 0.8 x 0.3 x 0.02 m spaced 0.3 m plus 40 boxes in the cells).  Start and goal
    are collision-free configurations drawn from `seed` whose straight joint-space edge
    collides, so the planner has to go around.  `checker(q_batch) -> bool[n]` (True =
    collision-free) and `edge_checker(a, b) -> bool` come from the caller."""
    robot = robot if robot is not None else serial_arm(1, dof=7, n_spheres=59, name="arm7")
    env = env if env is not None else shelf_env(seed)
    rng = np.random.default_rng(10_000 + seed)
    free_states = []
    drawn = 0
    while len(free_states) < 64 and drawn < max_draws:
        q = robot.sample_full(rng, 4096)
        drawn += 4096
        free_states.extend(q[checker(q)])
    if len(free_states) < 2:
        raise RuntimeError("scene has no collision-free configurations")
    free_states = np.asarray(free_states, np.float32)
    return robot, env, free_states


def pick_problem(free_states: np.ndarray, edge_free, seed: int):
    """First (start, goal) pair of `free_states` (in a seeded order) whose direct edge
    collides; falls back to the first pair."""
    rng = np.random.default_rng(20_000 + seed)
    order = rng.permutation(len(free_states))
    for a in range(0, len(order) - 1, 2):
        s, g = free_states[order[a]], free_states[order[a + 1]]
        if not edge_free(s, g):
            return s.copy(), g.copy()
    return free_states[order[0]].copy(), free_states[order[1]].copy()


def uneven_batch_models(seed: int, n: int = 256, feasible=None):
    """Robots and scenes of the uneven batch: DOF U{6..9} (8 and 9 with a prismatic
    torso), link spheres U[30, 120], obstacles U[10, 500] split 76 / 19 / 5 % into
    spheres / oriented boxes / cylinders (the 256 : 64 : 16 proportions).  The obstacle
    cube grows with the count so that the density stays near that of a 120-obstacle
    scene.  `feasible(robot, env) -> bool`, if given, rejects a scene (for example one
    without collision-free configurations) and the next scene seed of that problem is
    tried, up to 16 times."""
    rng = np.random.default_rng(30_000 + seed)
    out = []
    for i in range(n):
        dof = int(rng.integers(6, 10))
        S = int(rng.integers(30, 121))
        O = int(rng.integers(10, 501))
        nb = int(round(O * 64 / 336))
        nc = int(round(O * 16 / 336))
        ns = O - nb - nc
        robot = serial_arm(40_000 + 7 * seed + i, dof=dof, n_spheres=S, prismatic_torso=dof >= 8,
                           name=f"arm{dof}_b{i}", resolution=0.01)
        size = 1.2 * max(1.0, (O / 120.0) ** (1.0 / 3.0))
        for attempt in range(16):
            k = 50_000 + 7 * seed + i + 100_003 * attempt
            env = random_env(k, ns, nb, nc, oriented=True, size=size,
                             center=(SCENE_CENTER[0] + (size - 1.2) / 2, 0.0, SCENE_CENTER[2]))
            env = prune_blocking_obstacles(robot, env, np.random.default_rng(k + 10_000))
            if feasible is None or feasible(robot, env):
                break
        out.append((robot, env))
    return out


def prune_blocking_obstacles(robot: RobotModel, env: Environment, rng: np.random.Generator,
                             samples: int = 256, always: float = 0.9) -> Environment:
    """Drop obstacles whose bounding sphere meets the robot in at least `always` of
    random configurations (obstacles sitting in the permanently swept volume around the
    base would make every configuration collide)."""
    q = robot.sample_full(rng, samples)
    C = sphere_centers_numpy(robot, q)                                   # [N,S,3]
    r = robot.sphere_r.astype(np.float64)

    def blocked(pos, rad):
        if len(pos) == 0:
            return np.zeros(0, bool)
        d = np.linalg.norm(C[:, :, None, :] - pos[None, None].astype(np.float64), axis=-1)   # [N,S,O]
        hit = (d < (r[None, :, None] + rad[None, None])).any(1)
        return hit.mean(0) >= always

    bs = blocked(env.sphere_pos, env.sphere_r.astype(np.float64))
    bh = np.linalg.norm(np.maximum(np.abs(env.box_min), np.abs(env.box_max)), axis=1) if len(env.box_pos) else np.zeros(0)
    bb = blocked(env.box_pos, bh)
    ch = np.hypot(env.cyl_radius, env.cyl_height / 2) if len(env.cyl_pos) else np.zeros(0)
    bc = blocked(env.cyl_pos, ch)
    return Environment(env.sphere_pos[~bs], env.sphere_r[~bs], env.box_pos[~bb], env.box_rot[~bb],
                       env.box_min[~bb], env.box_max[~bb], env.cyl_pos[~bc], env.cyl_rot[~bc],
                       env.cyl_radius[~bc], env.cyl_height[~bc])
