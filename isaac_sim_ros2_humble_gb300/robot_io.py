"""Robot, scene and request loaders for libgbmp (host side, no GPU).

* `load_robot`: a robot model (`workloads.RobotModel`) from a URDF, an optional SRDF and
  a collision-sphere YAML, replacing the MoveIt-based table builder of the reference
  (`src/foliation_planner/include/foliation_planner/robot_info.hpp:13-310`) with the
  same mapping: links in the robot model's depth-first order, each link carrying the
  joint from its parent (MoveIt joint-type numbers: 0 root / unknown, 1 revolute and
  continuous, 2 prismatic, 5 fixed), joint origins as 4x4 poses, unit joint axes,
  self-collision allowed for every link pair except the SRDF's disabled pairs
  (`robot_info.hpp:55-90`), spheres per link in file order (`robot_info.hpp:236-300`),
  active joints = the joints of the planning group, limits of inactive joints 0
  (`robot_info.hpp:180-215`).
* `load_scene`: obstacles of a MoveIt planning-scene YAML (the MotionBenchMaker
  `scene*.yaml` files read by `obstacle_generator.hpp:914` `loadSceneObjects`): boxes,
  spheres and cylinders of `world.collision_objects`.
* `load_request`: start and goal joint vectors of a motion-plan-request YAML
  (`request*.yaml`, `MPM_helper.hpp:10-64`).
* `parse_yaml`: the subset of YAML these files use (block mappings and sequences,
  flow lists and maps that may span lines, quoted keys, comments, plain scalars); no
  YAML library is needed.
"""
from __future__ import annotations

import math
import re
import xml.etree.ElementTree as ET
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .workloads import Environment, RobotModel

# ---------------------------------------------------------------------------------
# YAML subset.
# ---------------------------------------------------------------------------------
_NUM = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?$")


def _strip_comment(line: str) -> str:
    out, q = [], None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _scalar(tok: str):
    t = tok.strip()
    if not t:
        return None
    if t[0] in "'\"" and t[-1] == t[0] and len(t) >= 2:
        return t[1:-1]
    low = t.lower()
    if low in ("true", "yes"):
        return True
    if low in ("false", "no"):
        return False
    if low in ("null", "~"):
        return None
    if _NUM.match(t):
        return float(t) if any(c in t for c in ".eE") else int(t)
    if low in (".inf", "+.inf"):
        return math.inf
    if low == "-.inf":
        return -math.inf
    return t


def _split_top(s: str, sep: str) -> List[str]:
    parts, depth, q, cur = [], 0, None, []
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


def _key_split(s: str) -> Optional[Tuple[str, str]]:
    """Split 'key: rest' at the first top-level ': ' (or trailing ':'); None if no key."""
    depth, q = 0, None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == ":" and depth == 0 and (i + 1 == len(s) or s[i + 1] in " \t"):
            key = s[:i].strip()
            if len(key) >= 2 and key[0] in "'\"" and key[-1] == key[0]:
                key = key[1:-1]
            return key, s[i + 1:].strip()
    return None


def _flow(s: str):
    s = s.strip()
    if s.startswith("["):
        body = s[1:-1].strip()
        return [] if not body else [_flow(p) for p in _split_top(body, ",") if p.strip()]
    if s.startswith("{"):
        body = s[1:-1].strip()
        out = {}
        for p in _split_top(body, ","):
            if p.strip():
                kv = _key_split(p.strip()) or (p.strip(), "")
                out[kv[0]] = _flow(kv[1])
        return out
    return _scalar(s)


def _logical_lines(text: str) -> List[Tuple[int, str]]:
    """(indent, content) per logical line; flow collections spanning lines are joined."""
    lines, buf, ind, depth = [], "", 0, 0
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if not line.strip() or line.strip() in ("---", "..."):
            continue
        if depth == 0:
            ind = len(line) - len(line.lstrip(" "))
            buf = line.strip()
        else:
            buf += " " + line.strip()
        q = None
        depth = 0
        for ch in buf:
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
            elif ch in "[{":
                depth += 1
            elif ch in "]}":
                depth -= 1
        if depth <= 0:
            depth = 0
            lines.append((ind, buf))
    return lines


def parse_yaml(text: str):
    """Parse the YAML subset used by robot sphere files and MoveIt scene / request files."""
    lines = _logical_lines(text)
    pos = 0

    def value_after(rest: str, ind: int):
        nonlocal pos
        if rest:
            return _flow(rest)
        if pos < len(lines) and (lines[pos][0] > ind or (lines[pos][0] == ind and lines[pos][1].startswith("- "))):
            return block(lines[pos][0])
        return None

    def block(ind: int):
        nonlocal pos
        if pos >= len(lines):
            return None
        if lines[pos][1] == "-" or lines[pos][1].startswith("- "):
            seq = []
            while pos < len(lines) and lines[pos][0] == ind and (lines[pos][1] == "-" or lines[pos][1].startswith("- ")):
                item = lines[pos][1][1:].strip()
                pos += 1
                if not item:
                    seq.append(block(lines[pos][0]) if pos < len(lines) and lines[pos][0] > ind else None)
                    continue
                kv = _key_split(item) if not item.startswith(("[", "{")) else None
                if kv is None:
                    seq.append(_flow(item))
                    continue
                # a mapping that starts on the dash line; its other keys follow, indented
                # past the dash
                m = {kv[0]: value_after(kv[1], ind + 2)}
                if pos < len(lines) and lines[pos][0] > ind:
                    rest = block(lines[pos][0])
                    if isinstance(rest, dict):
                        m.update(rest)
                seq.append(m)
            return seq
        out = {}
        while pos < len(lines) and lines[pos][0] == ind and not lines[pos][1].startswith("- "):
            kv = _key_split(lines[pos][1])
            if kv is None:
                raise ValueError(f"cannot parse YAML line: {lines[pos][1]!r}")
            pos += 1
            out[kv[0]] = value_after(kv[1], ind)
        return out

    return block(lines[0][0]) if lines else None


# ---------------------------------------------------------------------------------
# Robot model from URDF + SRDF + collision spheres.
# ---------------------------------------------------------------------------------
REVOLUTE, PRISMATIC, FIXED, UNKNOWN = 1, 2, 5, 0
_TYPES = {"revolute": REVOLUTE, "continuous": REVOLUTE, "prismatic": PRISMATIC, "fixed": FIXED}


def _vec(s: Optional[str], default) -> np.ndarray:
    return np.array([float(x) for x in s.split()], np.float64) if s else np.array(default, np.float64)


def _origin(el) -> np.ndarray:
    """4x4 pose of a URDF <origin xyz rpy>: translation, then R = Rz(yaw) Ry(pitch) Rx(roll)."""
    T = np.eye(4)
    if el is None:
        return T
    x, y, z = _vec(el.get("xyz"), (0, 0, 0))
    r, p, w = _vec(el.get("rpy"), (0, 0, 0))
    cr, sr, cp, sp, cw, sw = math.cos(r), math.sin(r), math.cos(p), math.sin(p), math.cos(w), math.sin(w)
    T[:3, :3] = [[cw * cp, cw * sp * sr - sw * cr, cw * sp * cr + sw * sr],
                 [sw * cp, sw * sp * sr + cw * cr, sw * sp * cr - cw * sr],
                 [-sp, cp * sr, cp * cr]]
    T[:3, 3] = (x, y, z)
    return T


def _srdf_group_joints(srdf: ET.Element, group: str, joints: Dict[str, dict]) -> List[str]:
    """Joint names of an SRDF group: <joint> entries, <chain> base..tip, nested <group>s."""
    for g in srdf.findall("group"):
        if g.get("name") != group:
            continue
        names = [j.get("name") for j in g.findall("joint")]
        for ch in g.findall("chain"):
            base, tip = ch.get("base_link"), ch.get("tip_link")
            by_child = {j["child"]: n for n, j in joints.items()}
            chain, link = [], tip
            while link != base and link in by_child:
                chain.append(by_child[link])
                link = joints[by_child[link]]["parent"]
            names += chain[::-1]
        for sub in g.findall("group"):
            names += _srdf_group_joints(srdf, sub.get("name"), joints)
        return names
    raise ValueError(f"group {group!r} is not in the SRDF")


def load_robot(urdf_text: str, srdf_text: Optional[str] = None, spheres_yaml_text: Optional[str] = None,
               group: Optional[str] = None, active_joints: Optional[Sequence[str]] = None,
               default_values: Optional[Dict[str, float]] = None, resolution: float = 0.02,
               name: Optional[str] = None) -> RobotModel:
    """Robot tables for libgbmp from a URDF (string), optionally an SRDF (planning group,
    disabled collision pairs) and a collision-sphere YAML (`collision_spheres: {link:
    [{center: [x, y, z], radius: r}, ...]}`).

    Links are ordered depth first from the root, children in joint-name order (the
    order the URDF parser of the robot model gives them), so every parent precedes its
    children.  Active joints are `active_joints`, else the SRDF `group`'s, else every
    revolute / prismatic joint.  Mimic joints are not followed: a joint that is not
    active stays at its default value.  Default values: `default_values[joint]`, else 0
    when 0 lies within the limits, else the middle of the limits."""
    root = ET.fromstring(urdf_text)
    links = [l.get("name") for l in root.findall("link")]
    joints: Dict[str, dict] = {}
    for j in root.findall("joint"):
        lim = j.find("limit")
        ax = j.find("axis")
        joints[j.get("name")] = {
            "type": j.get("type"), "parent": j.find("parent").get("link"), "child": j.find("child").get("link"),
            "origin": _origin(j.find("origin")), "axis": _vec(ax.get("xyz") if ax is not None else None, (1, 0, 0)),
            "lower": float(lim.get("lower", 0.0)) if lim is not None else 0.0,
            "upper": float(lim.get("upper", 0.0)) if lim is not None else 0.0,
        }
    child_of = {j["child"]: n for n, j in joints.items()}
    roots = [l for l in links if l not in child_of]
    if len(roots) != 1:
        raise ValueError(f"URDF must have exactly one root link, found {roots}")
    kids: Dict[str, List[str]] = {l: [] for l in links}
    for n in sorted(joints):
        kids[joints[n]["parent"]].append(n)
    order, stack = [], [roots[0]]
    while stack:   # depth-first, children in joint-name order
        l = stack.pop()
        order.append(l)
        stack.extend(joints[n]["child"] for n in reversed(kids[l]))
    index = {l: i for i, l in enumerate(order)}
    L = len(order)

    srdf = ET.fromstring(srdf_text) if srdf_text else None
    if active_joints is None and group is not None:
        if srdf is None:
            raise ValueError("a planning group needs the SRDF")
        active_joints = _srdf_group_joints(srdf, group, joints)
    if active_joints is None:
        active_joints = [n for n, j in joints.items() if _TYPES.get(j["type"]) in (REVOLUTE, PRISMATIC)]
    active_set = set(active_joints)
    unknown = active_set - set(joints)
    if unknown:
        raise ValueError(f"active joints not in the URDF: {sorted(unknown)}")

    types = np.zeros(L, np.int32)
    poses = np.tile(np.eye(4, dtype=np.float32), (L, 1, 1))
    axes = np.zeros((L, 3), np.float32)
    parent = np.full(L, -1, np.int32)
    active = np.zeros(L, np.uint8)
    lower = np.zeros(L, np.float32)
    upper = np.zeros(L, np.float32)
    default = np.zeros(L, np.float32)
    dv = default_values or {}
    for l in order[1:]:
        i, jn = index[l], child_of[l]
        j = joints[jn]
        types[i] = _TYPES.get(j["type"], UNKNOWN)
        poses[i] = j["origin"].astype(np.float32)
        parent[i] = index[j["parent"]]
        if types[i] in (REVOLUTE, PRISMATIC):
            a = j["axis"]
            axes[i] = (a / np.linalg.norm(a)).astype(np.float32)
            lo, hi = (j["lower"], j["upper"]) if j["type"] != "continuous" else (-math.pi, math.pi)
            default[i] = dv.get(jn, 0.0 if lo <= 0.0 <= hi else 0.5 * (lo + hi))
            if jn in active_set:
                active[i] = 1
                lower[i], upper[i] = lo, hi

    sphere_link, sphere_pos, sphere_r = [], [], []
    if spheres_yaml_text:
        spheres = (parse_yaml(spheres_yaml_text) or {}).get("collision_spheres") or {}
        for link_name, items in spheres.items():
            if link_name not in index:
                continue   # the reference skips spheres of unknown links (robot_info.hpp:256-270)
            for it in items or []:
                sphere_link.append(index[link_name])
                sphere_pos.append([float(v) for v in it["center"][:3]])
                sphere_r.append(float(it["radius"]))
    enables = np.ones((L, L), np.uint8)
    if srdf is not None:
        for d in srdf.findall("disable_collisions"):
            a, b = d.get("link1"), d.get("link2")
            if a in index and b in index:
                enables[index[a], index[b]] = enables[index[b], index[a]] = 0
    return RobotModel(name=name or root.get("name", "robot"), joint_types=types, joint_poses=poses,
                      joint_axes=axes, parent=parent, sphere_link=np.asarray(sphere_link, np.int32).reshape(-1),
                      sphere_pos=np.asarray(sphere_pos, np.float32).reshape(-1, 3),
                      sphere_r=np.asarray(sphere_r, np.float32).reshape(-1), active=active, lower=lower,
                      upper=upper, default=default, enables=enables, link_names=order, resolution=resolution)


def joint_names(urdf_text: str, robot: RobotModel) -> List[Optional[str]]:
    """Name of the joint carried by each link of `robot` (None for the root)."""
    root = ET.fromstring(urdf_text)
    child_of = {j.find("child").get("link"): j.get("name") for j in root.findall("joint")}
    return [child_of.get(l) for l in robot.link_names]


# ---------------------------------------------------------------------------------
# MoveIt planning scenes and motion-plan requests (MotionBenchMaker problem files).
# ---------------------------------------------------------------------------------
def _quat_rot(q) -> np.ndarray:
    """Row-major rotation of a unit quaternion given as (x, y, z, w)."""
    x, y, z, w = (float(v) for v in q)
    n = math.sqrt(x * x + y * y + z * z + w * w) or 1.0
    x, y, z, w = x / n, y / n, z / n, w / n
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], np.float64)


def _pose(p) -> np.ndarray:
    T = np.eye(4)
    if p:
        T[:3, :3] = _quat_rot(p.get("orientation", (0, 0, 0, 1)))
        T[:3, 3] = [float(v) for v in p.get("position", (0, 0, 0))]
    return T


def load_scene(yaml_text: str) -> Environment:
    """Obstacles of a planning-scene YAML: every primitive of `world.collision_objects`
    (box dimensions = full edge lengths, sphere = [radius], cylinder = [height, radius],
    MoveIt's shape conventions) at its primitive pose, composed with the object's own
    `pose` when the file gives one.  The robot base is taken to sit at the world origin,
    as in the MotionBenchMaker scenes; other primitive types raise ValueError."""
    doc = parse_yaml(yaml_text) or {}
    objs = ((doc.get("world") or {}).get("collision_objects")) or []
    sp, sr, bp, brot, bmn, bmx, cp, crot, crad, chei = ([] for _ in range(10))
    for ob in objs:
        base = _pose(ob.get("pose"))
        for prim, pp in zip(ob.get("primitives") or [], ob.get("primitive_poses") or []):
            T = base @ _pose(pp)
            kind, dims = str(prim.get("type")).lower(), [float(v) for v in prim.get("dimensions") or []]
            if kind == "box":
                h = 0.5 * np.asarray(dims[:3])
                bp.append(T[:3, 3]); brot.append(T[:3, :3]); bmn.append(-h); bmx.append(h)
            elif kind == "sphere":
                sp.append(T[:3, 3]); sr.append(dims[0])
            elif kind == "cylinder":
                cp.append(T[:3, 3]); crot.append(T[:3, :3]); chei.append(dims[0]); crad.append(dims[1])
            else:
                raise ValueError(f"unsupported primitive {kind!r} in object {ob.get('id')!r}")
    f = lambda a, shape: np.asarray(a, np.float32).reshape(shape)
    return Environment(f(sp, (-1, 3)), f(sr, (-1,)), f(bp, (-1, 3)), f(brot, (-1, 3, 3)), f(bmn, (-1, 3)),
                       f(bmx, (-1, 3)), f(cp, (-1, 3)), f(crot, (-1, 3, 3)), f(crad, (-1,)), f(chei, (-1,)))


def load_request(yaml_text: str, robot: RobotModel, link_joint_names: Sequence[Optional[str]]):
    """(start, goal) full joint vectors [L] of a motion-plan-request YAML: the robot's
    defaults overwritten by `start_state.joint_state` (name / position) for the start
    and additionally by the first goal's `joint_constraints` for the goal.
    `link_joint_names` names the joint carried by each link (`joint_names`)."""
    doc = parse_yaml(yaml_text) or {}
    col = {n: i for i, n in enumerate(link_joint_names) if n}
    start = robot.default.astype(np.float32).copy()
    js = ((doc.get("start_state") or {}).get("joint_state")) or {}
    for n, v in zip(js.get("name") or [], js.get("position") or []):
        if n in col:
            start[col[n]] = float(v)
    goal = start.copy()
    goals = doc.get("goal_constraints") or []
    if not goals:
        raise ValueError("request has no goal_constraints")
    for c in goals[0].get("joint_constraints") or []:
        if c.get("joint_name") in col:
            goal[col[c["joint_name"]]] = float(c["position"])
    return start, goal
