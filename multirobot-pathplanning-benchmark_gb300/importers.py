"""Scene importers: MuJoCo MJCF planar multi-robot scenes to sphere-set scenes.

The reference's MuJoCo planar problems (``mujoco.swap``, ``mujoco.hallway``,
``mujoco.piano``: problems/mujoco_env.py:891-1060, scene files under
assets/models/mujoco/) describe each robot as a body with a slide joint
along x, a slide joint along y and a hinge about z, carrying primitive
geoms, among static axis-aligned boxes in the same plane; the environment
takes its joint limits from the compiled model (``jnt_range``,
mujoco_env.py:194-198: radians; MJCF ranges are in degrees unless the
``<compiler angle="radian">`` says otherwise).

``load_mjcf_planar`` turns such a file into an ``ArmScene`` of planar-base
robots (``base_kind`` 1, no links) whose geoms become spheres in the base
frame, and box obstacles:

* a sphere geom is that sphere;
* a cylinder, or a capsule, along the body's z axis becomes one sphere of
  its radius at its centre.  When every geom's height range contains the
  obstacle plane (a planar scene), the sphere touches exactly the boxes and
  discs the cylinder touches, so verdicts are those of the planar problem;
* a box geom becomes a chain of spheres along its longer horizontal axis
  that covers its horizontal rectangle (radius sqrt(2) times the half width,
  centres at most twice the half width apart): conservative, a covered box
  may report a collision slightly before the box itself touches;
* static box geoms (bodies without joints) become box obstacles; planes
  (the floor) are skipped;
* free bodies (``<freejoint/>``, the movable objects of the manipulation
  scenes) become box obstacles at their initial pose, the scene's first
  mode; ``scene.movable_boxes`` maps each such body to its box indices, the
  pool for per-mode tables (``ArmScene.mode_boxes``).

Rotated geoms or bodies, articulated robots (bodies below a robot body),
robot bodies off the x = y = 0 origin and other geom types raise
``NotImplementedError``: they do not map onto this model.
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

from .scenes import MAX_LINKS, ArmScene

_ROT_ATTRS = ("quat", "euler", "axisangle", "xyaxes", "zaxis")


def _vec(el, name, n, default=0.0):
    s = el.get(name)
    if s is None:
        return np.full(n, default, dtype=np.float64)
    v = np.array([float(x) for x in s.split()], dtype=np.float64)
    if len(v) < n:
        v = np.concatenate([v, np.full(n - len(v), default)])
    return v[:n]


def _check_unrotated(el, what):
    for a in _ROT_ATTRS:
        s = el.get(a)
        if s is None:
            continue
        v = [float(x) for x in s.split()]
        if a == "quat" and np.allclose(v, [1, 0, 0, 0]):
            continue
        raise NotImplementedError(f"{what}: rotated frames ({a}) do not map onto the planar sphere model")


def _box_spheres(pos, half):
    """Spheres covering the horizontal rectangle of a box geom."""
    a, b = float(half[0]), float(half[1])
    long_y = b >= a
    w, l = (a, b) if long_y else (b, a)
    rho = math.sqrt(2.0) * w
    if l <= w:
        centers = [0.0]
    else:
        n = int(math.ceil((l - w) / w - 1e-9)) + 1   # centres at most 2 w apart
        centers = list(np.linspace(-(l - w), l - w, n))
    out = []
    for c in centers:
        off = np.array([0.0, c, 0.0]) if long_y else np.array([c, 0.0, 0.0])
        out.append((pos + off, rho))
    return out


def load_mjcf_planar(source, robots=None) -> ArmScene:
    """ArmScene of a planar MJCF scene (a path or the XML text).  ``robots``
    names the robot bodies in configuration order (default: every body with
    joints, in file order); each contributes (x, y, yaw) to the configuration."""
    text = source if isinstance(source, str) and source.lstrip().startswith("<") else Path(source).read_text()
    root = ET.fromstring(text)
    comp = root.find("compiler")
    radian = comp is not None and comp.get("angle", "degree") == "radian"
    wb = root.find("worldbody")
    if wb is None:
        raise ValueError("no <worldbody>")
    boxes_lo, boxes_hi = [], []
    found = {}
    movable = {}

    def static_geom(g, base):
        _check_unrotated(g, "geom")
        t = g.get("type", "sphere")
        if t == "plane":
            return
        if t != "box":
            raise NotImplementedError(f"static {t} geoms are not box obstacles")
        c = base + _vec(g, "pos", 3)
        h = _vec(g, "size", 3)
        boxes_lo.append(c - h)
        boxes_hi.append(c + h)

    def walk(body, base):
        _check_unrotated(body, f"body {body.get('name')}")
        pos = base + _vec(body, "pos", 3)
        joints = body.findall("joint")
        if body.find("freejoint") is not None or any(j.get("type") == "free" for j in joints):
            first = len(boxes_lo)
            for g in body.findall("geom"):
                static_geom(g, pos)
            movable[body.get("name")] = list(range(first, len(boxes_lo)))
            return
        if joints:
            name = body.get("name")
            if body.findall("body"):
                raise NotImplementedError(f"robot {name}: articulated bodies are not planar robots")
            kinds = [(j.get("type", "hinge"), tuple(_vec(j, "axis", 3, 0.0))) for j in joints]
            want = [("slide", (1.0, 0.0, 0.0)), ("slide", (0.0, 1.0, 0.0)), ("hinge", (0.0, 0.0, 1.0))]
            if kinds != want:
                raise NotImplementedError(f"robot {name}: joints must be slide x, slide y, hinge z")
            if any(np.any(_vec(j, "pos", 3) != 0.0) for j in joints):
                raise NotImplementedError(f"robot {name}: joints must sit at the body origin")
            if pos[0] != 0.0 or pos[1] != 0.0:
                raise NotImplementedError(f"robot {name}: the body must sit at x = y = 0 (its slides are the position)")
            lim = []
            for j, (kind, _) in zip(joints, kinds):
                if j.get("range") is None:
                    raise ValueError(f"robot {name}: joint {j.get('name')} has no range")
                r = _vec(j, "range", 2)
                if kind == "hinge" and not radian:
                    r = np.deg2rad(r)
                lim.append(r)
            spheres = []
            for g in body.findall("geom"):
                _check_unrotated(g, f"geom of {name}")
                t = g.get("type", "sphere")
                gp = _vec(g, "pos", 3)
                sz = _vec(g, "size", 3)
                if t == "sphere":
                    spheres.append((gp, float(sz[0])))
                elif t in ("cylinder", "capsule"):
                    if g.get("fromto") is not None:
                        raise NotImplementedError(f"robot {name}: fromto geoms are not supported")
                    spheres.append((gp, float(sz[0])))
                elif t == "box":
                    spheres.extend(_box_spheres(gp, sz))
                else:
                    raise NotImplementedError(f"robot {name}: {t} geoms are not supported")
            if not spheres:
                raise ValueError(f"robot {name} has no geoms")
            found[name] = (float(pos[2]), np.array(lim).T, spheres)
            return
        for g in body.findall("geom"):
            static_geom(g, pos)
        for b in body.findall("body"):
            walk(b, pos)

    zero = np.zeros(3)
    for g in wb.findall("geom"):
        static_geom(g, zero)
    for b in wb.findall("body"):
        walk(b, zero)
    names = list(found) if robots is None else list(robots)
    missing = [n for n in names if n not in found]
    if missing or not names:
        raise ValueError(f"robots not found: {missing or 'none in the file'}")
    R = len(names)
    base_pose = np.zeros((R, 12))
    lims, s_robot, s_loc, s_rad = [], [], [], []
    for r, n in enumerate(names):
        z, lim, spheres = found[n]
        base_pose[r, :9] = np.eye(3).reshape(-1)
        base_pose[r, 9:] = [0.0, 0.0, z]
        lims.append(lim)
        for p, rad in spheres:
            s_robot.append(r)
            s_loc.append(p)
            s_rad.append(rad)
    S = len(s_rad)
    scene = ArmScene(
        q_offset=np.arange(R, dtype=np.int32) * 3,
        base_kind=np.ones(R, dtype=np.int32),
        base_pose=base_pose,
        n_links=np.zeros(R, dtype=np.int32),
        dh=np.zeros((R, MAX_LINKS, 4)),
        sphere_robot=np.array(s_robot, dtype=np.int32),
        sphere_link=np.zeros(S, dtype=np.int32),
        sphere_local=np.array(s_loc, dtype=np.float64).reshape(-1, 3),
        sphere_radius=np.array(s_rad, dtype=np.float64),
        box_lo=np.array(boxes_lo, dtype=np.float64).reshape(-1, 3),
        box_hi=np.array(boxes_hi, dtype=np.float64).reshape(-1, 3),
        q_dim=3 * R,
        limits=np.concatenate(lims, axis=1),
    )
    scene.movable_boxes = movable
    return scene
