"""Robot / scene / request loaders (host code): the YAML-subset reader, URDF + SRDF +
collision-sphere tables (link order, joint types, poses, axes, limits, defaults, planning
group, disabled pairs) checked against hand-computed values, MoveIt scene and request
files, an end-to-end GPU check of a loaded robot, and - where the reference tree is
present - the real Fetch description with MotionBenchMaker problems, whose start and goal
configurations must come out collision-free."""
import glob
import math
import os

import numpy as np
import pytest

from isaac_sim_ros2_humble_gb300 import robot_io as RIO, workloads as W

URDF = """<?xml version="1.0"?>
<robot name="tri">
  <link name="base"/>
  <link name="l1"/>
  <link name="l2"/>
  <link name="tool"/>
  <joint name="j3" type="prismatic">
    <parent link="l2"/><child link="tool"/>
    <origin xyz="0.2 0 0"/><axis xyz="1 0 0"/>
    <limit lower="0.1" upper="0.3" effort="1" velocity="1"/>
  </joint>
  <joint name="j1" type="continuous">
    <parent link="base"/><child link="l1"/>
    <origin xyz="0 0 0.3" rpy="0 0 0"/><axis xyz="0 0 2"/>
  </joint>
  <joint name="j2" type="revolute">
    <parent link="l1"/><child link="l2"/>
    <origin xyz="0.4 0 0" rpy="1.5707963267948966 0 0"/><axis xyz="0 0 1"/>
    <limit lower="-1" upper="2" effort="1" velocity="1"/>
  </joint>
</robot>"""

SRDF = """<?xml version="1.0"?>
<robot name="tri">
  <group name="arm"><joint name="j1"/><joint name="j2"/></group>
  <group name="arm_chain"><chain base_link="base" tip_link="l2"/></group>
  <disable_collisions link1="base" link2="l1" reason="Adjacent"/>
  <disable_collisions link1="l1" link2="nowhere" reason="Never"/>
</robot>"""

SPHERES = """# spheres per link
collision_spheres:
  l1:
    - "center": [0.1, 0, 0]
      "radius": 0.05
  ghost_link:
    - center: [0, 0, 0]
      radius: 1.0
  tool:
    - {center: [0.0, 0.0, 0.02], radius: 0.03}
    - center: [0.0, 0.0, -0.02]
      radius: 0.025
"""


def test_yaml_subset():
    doc = RIO.parse_yaml("""
a: 1
b: -2.5e-3   # comment
c: [1, [2, 3], {x: 1, y: "q: z"}]
d:
  - plain text
  - 'quoted # not a comment'
  - k: v
    k2: [true, false, null]
  -
    - nested
e: {m: [0,
        1, 2]}
f:
- same-indent item
g: 'single'
""")
    assert doc["a"] == 1 and doc["b"] == pytest.approx(-2.5e-3)
    assert doc["c"] == [1, [2, 3], {"x": 1, "y": "q: z"}]
    assert doc["d"] == ["plain text", "quoted # not a comment", {"k": "v", "k2": [True, False, None]}, ["nested"]]
    assert doc["e"] == {"m": [0, 1, 2]}
    assert doc["f"] == ["same-indent item"] and doc["g"] == "single"


def test_urdf_tables():
    r = RIO.load_robot(URDF, SRDF, SPHERES, group="arm")
    assert r.link_names == ["base", "l1", "l2", "tool"]
    np.testing.assert_array_equal(r.parent, [-1, 0, 1, 2])
    np.testing.assert_array_equal(r.joint_types, [0, 1, 1, 2])
    np.testing.assert_allclose(r.joint_axes[1], [0, 0, 1])          # normalised
    np.testing.assert_array_equal(r.active, [0, 1, 1, 0])
    np.testing.assert_allclose(r.lower, [0, -math.pi, -1, 0], rtol=1e-6)   # continuous: +-pi
    np.testing.assert_allclose(r.upper, [0, math.pi, 2, 0], rtol=1e-6)
    np.testing.assert_allclose(r.default, [0, 0, 0, 0.2], rtol=1e-6)      # 0 outside [0.1, 0.3]: middle
    assert r.enables[0, 1] == 0 and r.enables[1, 0] == 0 and r.enables[1, 2] == 1
    np.testing.assert_array_equal(r.sphere_link, [1, 3, 3])              # ghost_link skipped
    np.testing.assert_allclose(r.sphere_r, [0.05, 0.03, 0.025])
    assert RIO.joint_names(URDF, r) == [None, "j1", "j2", "j3"]
    chain = RIO.load_robot(URDF, SRDF, SPHERES, group="arm_chain")
    np.testing.assert_array_equal(chain.active, [0, 1, 1, 0])
    every = RIO.load_robot(URDF)
    np.testing.assert_array_equal(every.active, [0, 1, 1, 1])


def test_urdf_forward_kinematics():
    r = RIO.load_robot(URDF, SRDF, SPHERES, group="arm")
    q = np.array([[0.0, math.pi / 2, 0.0, 0.1]], np.float32)
    P = W.fk_numpy(r, q)[0]
    # j1 turns l1 by 90 deg about z at height 0.3; l2 sits 0.4 along l1's x (world y);
    # the tool 0.2 further along l2's x (still world y) plus the 0.1 prismatic travel
    np.testing.assert_allclose(P[2][:3, 3], [0.0, 0.4, 0.3], atol=1e-6)
    np.testing.assert_allclose(P[3][:3, 3], [0.0, 0.7, 0.3], atol=1e-6)
    # l2 is rolled +90 deg about x, so its z axis is l1's -y axis, which j1's quarter turn
    # points along world +x
    np.testing.assert_allclose(P[2][:3, 2], [1.0, 0.0, 0.0], atol=1e-6)


SCENE = """world:
  collision_objects:
    - id: box1
      primitives:
        - type: box
          dimensions: [0.2, 0.4, 0.6]
      primitive_poses:
        - position: [1, 0, 0.5]
          orientation: [0, 0, 0.7071067811865476, 0.7071067811865476]
    - id: obj2
      pose:
        position: [0, 1, 0]
        orientation: [0, 0, 0, 1]
      primitives: [{type: sphere, dimensions: [0.1]}, {type: cylinder, dimensions: [0.5, 0.05]}]
      primitive_poses: [{position: [0, 0, 0.2], orientation: [0, 0, 0, 1]}, {position: [0.1, 0, 0], orientation: [0, 0, 0, 1]}]
"""

REQUEST = """start_state:
  joint_state:
    name: [j1, j2, j3, other]
    position: [0.5, -0.5, 0.25, 9]
goal_constraints:
  - joint_constraints:
      - joint_name: j2
        position: 1.5
      - position: -0.25
        joint_name: j1
group_name: arm
"""


def test_scene_and_request():
    env = RIO.load_scene(SCENE)
    assert env.counts == (1, 1, 1)
    np.testing.assert_allclose(env.box_pos[0], [1, 0, 0.5])
    np.testing.assert_allclose(env.box_rot[0], [[0, -1, 0], [1, 0, 0], [0, 0, 1]], atol=1e-6)
    np.testing.assert_allclose(env.box_max[0], [0.1, 0.2, 0.3])
    np.testing.assert_allclose(env.box_min[0], [-0.1, -0.2, -0.3])
    np.testing.assert_allclose(env.sphere_pos[0], [0, 1, 0.2])
    np.testing.assert_allclose(env.sphere_r, [0.1])
    np.testing.assert_allclose(env.cyl_pos[0], [0.1, 1, 0])
    np.testing.assert_allclose(env.cyl_height, [0.5])
    np.testing.assert_allclose(env.cyl_radius, [0.05])
    r = RIO.load_robot(URDF, SRDF, SPHERES, group="arm")
    start, goal = RIO.load_request(REQUEST, r, RIO.joint_names(URDF, r))
    np.testing.assert_allclose(start, [0, 0.5, -0.5, 0.25])
    np.testing.assert_allclose(goal, [0, -0.25, 1.5, 0.25])
    with pytest.raises(ValueError):
        RIO.load_scene("world:\n  collision_objects:\n    - primitives: [{type: cone, dimensions: [1, 1]}]\n"
                       "      primitive_poses: [{position: [0, 0, 0]}]\n")


@pytest.mark.gpu
def test_loaded_robot_runs_on_the_gpu():
    torch = pytest.importorskip("torch")
    import oracle as O
    from isaac_sim_ros2_humble_gb300 import api
    r = RIO.load_robot(URDF, SRDF, SPHERES, group="arm")
    env = RIO.load_scene(SCENE)
    m = O.OracleModel(r, env)
    q = r.sample_full(np.random.default_rng(3), 4096)
    v = torch.zeros(len(q), dtype=torch.uint8, device="cuda")
    api.check_states(api.Robot(r), api.Env(env), torch.from_numpy(q).cuda(), verdict=v)
    torch.cuda.synchronize()
    clear = np.abs(m.clearance(q)) > 1e-4
    np.testing.assert_array_equal(v.cpu().numpy().astype(bool)[clear], (m.check_states(q)[1] > 0)[clear])


from ref_build import REF_ROOT as REF  # noqa: E402  (oracle/ref_build.py: the reference tree, if present)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "problems")), reason="reference tree not present")
def test_fetch_motionbenchmaker_problems_are_collision_free():
    import oracle as O
    base = os.path.join(REF, "src", "fetch_ros")
    urdf = open(os.path.join(base, "fetch_description", "robots", "fetch.urdf")).read()
    robot = RIO.load_robot(urdf, open(os.path.join(base, "fetch_moveit2_config", "config", "fetch.srdf")).read(),
                           open(os.path.join(base, "fetch_description", "robots",
                                             "fetch.collision_spheres.yaml")).read(), group="arm_with_torso")
    assert (robot.num_links, robot.num_spheres, robot.dim) == (30, 110, 8)
    names = RIO.joint_names(urdf, robot)
    checked = 0
    for fam in ("bookshelf_small_fetch", "box_fetch", "cage_fetch", "table_pick_fetch"):
        for scene in sorted(glob.glob(os.path.join(REF, "problems", fam, "scene*.yaml")))[:3]:
            env = RIO.load_scene(open(scene).read())
            start, goal = RIO.load_request(open(scene.replace("scene", "request")).read(), robot, names)
            cl = O.OracleModel(robot, env).clearance(np.stack([start, goal]))
            assert np.all(cl > 0), (scene, cl)
            checked += 1
    assert checked == 12
