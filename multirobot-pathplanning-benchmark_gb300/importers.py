"""Scene importers: the reference's MuJoCo (MJCF) and pinocchio (URDF) scene
files to sphere-set scenes.

* ``load_mjcf_planar``: planar MJCF scenes (below);
* ``load_mjcf_arms``: MJCF scenes of articulated arms (the four-UR10 scene):
  each robot's chain of hinge joints, with general body frames, is brought
  to the standard DH form of the kernels plus fixed joint-angle offsets
  (``chain_to_dh``), collision capsules covered by spheres;
* ``load_urdf_planar``: the planar pinocchio URDF scenes (prismatic x,
  prismatic y, revolute z robots among boxes).

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


# ---------------------------------------------------------------------------
# Rigid transforms
# ---------------------------------------------------------------------------
def _quat_R(q) -> np.ndarray:
    """Rotation of an MJCF quaternion (w, x, y, z), normalised first."""
    w, x, y, z = np.asarray(q, dtype=np.float64) / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _axis_R(axis, angle: float) -> np.ndarray:
    """Rotation by `angle` about the unit `axis` (Rodrigues)."""
    k = np.asarray(axis, dtype=np.float64)
    k = k / np.linalg.norm(k)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * (K @ K)


def _rpy_R(rpy) -> np.ndarray:
    """URDF fixed-axis roll, pitch, yaw: Rz(yaw) Ry(pitch) Rx(roll)."""
    r, p, y = rpy
    return _axis_R([0, 0, 1], y) @ _axis_R([0, 1, 0], p) @ _axis_R([1, 0, 0], r)


def _hom(R, p) -> np.ndarray:
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = p
    return T


# ---------------------------------------------------------------------------
# Serial chains of revolute joints -> standard DH with joint offsets
# ---------------------------------------------------------------------------
def _unit(v):
    n = np.linalg.norm(v)
    return v / n


def chain_to_dh(origins, axes, base_x=None, eps: float = 1e-12):
    """Standard DH form of a serial chain of revolute joints given, at the
    zero configuration, each joint's axis as a line (a point `origins[j]` and
    a direction `axes[j]`, world frame; joint j turns by +q about +axes[j]).

    Returns (frames, dh, offset): frames[k] (4x4, world, zero configuration)
    of DH frame k = 0..n, each fixed to link k (frame 0 to the base); dh[k]
    = (a, d, alpha) of link k+1, with T_{k+1} = T_k Rz(q + offset[k]) Tz(d)
    Tx(a) Rx(alpha).  Frame k (k < n) has its z axis on joint k+1's axis and
    its x axis on the common normal of axes k and k+1 (through frame k-1's
    origin when they are parallel); the last frame is frame n-1 turned by the
    last joint."""
    n = len(axes)
    z = [_unit(np.asarray(a, dtype=np.float64)) for a in axes]
    o = [np.asarray(p, dtype=np.float64) for p in origins]
    # frame 0: on joint 1's axis; x from the base's x (or y) projected off z
    z0 = z[0]
    cand = np.array([1.0, 0.0, 0.0]) if base_x is None else np.asarray(base_x, dtype=np.float64)
    x0 = cand - (cand @ z0) * z0
    if np.linalg.norm(x0) < 1e-6:
        cand = np.array([0.0, 1.0, 0.0])
        x0 = cand - (cand @ z0) * z0
    x0 = _unit(x0)
    frames = [(x0, np.cross(z0, x0), z0, o[0])]
    dh, off = [], []
    for k in range(1, n + 1):
        xp, yp, zp, op = frames[-1]
        if k == n:
            zk, pk = zp, op          # last frame: the previous one turned by the last joint
        else:
            zk, pk = z[k], o[k]
        c = np.cross(zp, zk)
        if np.linalg.norm(c) > 1e-9:          # skew or intersecting axes
            xk = _unit(c)
            # closest points of op + t zp and pk + s zk
            w0 = op - pk
            b = zp @ zk
            den = 1.0 - b * b
            t = (b * (zk @ w0) - (zp @ w0)) / den
            s_ = ((zk @ w0) - b * (zp @ w0)) / den
            foot = op + t * zp
            ok = pk + s_ * zk
            d = t
            a = (ok - foot) @ xk
        else:                                  # parallel (or one) axes
            w = (pk - op) - ((pk - op) @ zp) * zp
            if np.linalg.norm(w) > eps:
                xk = _unit(w)
                a = np.linalg.norm(w)
            else:
                xk = xp
                a = 0.0
            d = 0.0
            ok = op + w
            zk = zk if k < n else zp
        alpha = math.atan2(np.cross(zp, zk) @ xk, zp @ zk)
        theta0 = math.atan2(np.cross(xp, xk) @ zp, xp @ xk)
        frames.append((xk, np.cross(zk, xk), zk, ok))
        dh.append((a, d, alpha))
        off.append(theta0)
    T = [_hom(np.stack([f[0], f[1], f[2]], 1), f[3]) for f in frames]
    return T, np.array(dh), np.array(off)


def _capsule_spheres(p0, p1, r):
    """Spheres covering the capsule of radius r around segment p0-p1:
    centres on the segment at most r apart, radius sqrt(r^2 + (s/2)^2) for
    spacing s (every capsule point is within that of a centre)."""
    L = float(np.linalg.norm(p1 - p0))
    n = max(1, int(math.ceil(L / r - 1e-9))) + 1 if L > 0 else 1
    if n == 1:
        return [(0.5 * (p0 + p1), r)]
    s = L / (n - 1)
    rr = math.sqrt(r * r + 0.25 * s * s)
    return [(p0 + (p1 - p0) * (i / (n - 1)), rr) for i in range(n)]


def _box_cover_spheres(c, R, half):
    """Spheres covering a box (centre c, rotation R, half extents): a grid of
    cells of edge at most 2 * min(half) ... each cell covered by the sphere
    through its corners."""
    h = np.asarray(half, dtype=np.float64)
    cell = max(float(h.min()) * 2.0, 1e-6)
    n = [max(1, int(math.ceil(2 * hi / cell - 1e-9))) for hi in h]
    e = np.array([2 * h[i] / n[i] for i in range(3)])
    rad = 0.5 * float(np.linalg.norm(e))
    out = []
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                loc = -h + e * (np.array([i, j, k]) + 0.5)
                out.append((c + R @ loc, rad))
    return out


# ---------------------------------------------------------------------------
# MJCF articulated arms
# ---------------------------------------------------------------------------
class _Mjcf:
    """Minimal MJCF reader: nested default classes (joint and geom
    attributes, childclass inheritance), <compiler angle>, and <attach> of a
    model declared in <asset><model file=...>."""

    def __init__(self, path: Path):
        self.path = Path(path)
        self.root = ET.fromstring(self.path.read_text())
        comp = self.root.find("compiler")
        self.radian = comp is not None and comp.get("angle", "degree") == "radian"
        self.classes = {}
        d = self.root.find("default")
        if d is not None:
            self._defaults(d, "main", {})
        self.models = {}
        for a in self.root.findall("asset"):
            for m in a.findall("model"):
                self.models[m.get("name")] = _Mjcf(self.path.parent / m.get("file"))

    def _defaults(self, el, name, inherited):
        mine = {tag: dict(attrs) for tag, attrs in inherited.items()}
        for child in el:
            if child.tag == "default":
                continue
            mine.setdefault(child.tag, {}).update(child.attrib)
        self.classes[name] = mine
        for child in el.findall("default"):
            self._defaults(child, child.get("class", name), mine)

    def attrs(self, el, cls):
        """Attributes of element `el` resolved through class `cls` (its own
        class attribute wins over the inherited childclass)."""
        c = el.get("class", cls)
        a = dict(self.classes.get(c, self.classes.get("main", {})).get(el.tag, {}))
        a.update({k: v for k, v in el.attrib.items() if k != "class"})
        return a

    def angle(self, v: float) -> float:
        return v if self.radian else math.radians(v)

    def frame_R(self, a) -> np.ndarray:
        if "quat" in a:
            return _quat_R([float(x) for x in a["quat"].split()])
        if "euler" in a:
            e = [self.angle(float(x)) for x in a["euler"].split()]   # intrinsic x, y, z
            return _axis_R([1, 0, 0], e[0]) @ _axis_R([0, 1, 0], e[1]) @ _axis_R([0, 0, 1], e[2])
        if "axisangle" in a:
            v = [float(x) for x in a["axisangle"].split()]
            return _axis_R(v[:3], self.angle(v[3]))
        for bad in ("xyaxes", "zaxis"):
            if bad in a:
                raise NotImplementedError(f"{bad} frames are not supported")
        return np.eye(3)


def _vec3(a, key, default=(0.0, 0.0, 0.0)):
    return np.array([float(x) for x in a[key].split()][:3]) if key in a else np.array(default, dtype=np.float64)


def parse_mjcf_arms(source):
    """The articulated robots of an MJCF scene as serial chains: for each
    robot body (a world child whose subtree holds hinge joints) its body
    frames, joints and collision geoms (capsules, spheres, cylinders, boxes,
    with the geom's resolved contype / conaffinity not both 0; planes and
    visual meshes are skipped), and the static / free-body boxes of the scene.
    Returns (robots, boxes_lo, boxes_hi, movable), robots a list of dicts
    with 'name', 'base' (4x4 world pose of the robot body), 'joints' (per
    joint: 'T0' body frame at the zero configuration (world), 'pos' and
    'axis' in that body frame, 'range'), 'geoms' (per geom: joint index it
    rides on, -1 for the base, and a list of (centre in that body frame,
    radius) spheres covering it, with 'body_T0')."""
    mj = _Mjcf(Path(source))
    wb = mj.root.find("worldbody")
    if wb is None:
        raise ValueError("no <worldbody>")
    boxes_lo, boxes_hi, movable, robots = [], [], {}, []

    def static_box(g, T, owner):
        a = owner.attrs(g, "main")
        t = a.get("type", "sphere")
        if t == "plane":
            return
        if t != "box":
            raise NotImplementedError(f"static {t} geoms are not box obstacles")
        Tg = T @ _hom(owner.frame_R(a), _vec3(a, "pos"))
        h = _vec3(a, "size")
        corners = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]) * h
        w = (Tg[:3, :3] @ corners.T).T + Tg[:3, 3]
        if not np.allclose(np.abs(Tg[:3, :3]), np.round(np.abs(Tg[:3, :3])), atol=1e-9):
            raise NotImplementedError("rotated box obstacles do not map onto axis-aligned boxes")
        boxes_lo.append(w.min(0))
        boxes_hi.append(w.max(0))

    def has_joints(body, owner):
        if any(j.tag == "joint" for j in body):
            return True
        for b in body.findall("body"):
            if has_joints(b, owner):
                return True
        for at in body.findall("attach"):
            return True
        return False

    def robot_chain(body, T, owner, cls, name):
        joints, geoms = [], []

        def walk(b, T, owner, cls, ji):
            a = owner.attrs(b, cls)
            cls_here = b.get("childclass", cls)
            Tb = T @ _hom(owner.frame_R(a), _vec3(a, "pos"))
            js = [j for j in b if j.tag == "joint"]
            if len(js) > 1:
                raise NotImplementedError(f"robot {name}: several joints in one body")
            if b.find("freejoint") is not None:
                raise NotImplementedError(f"robot {name}: free joints inside a robot")
            if js:
                ja = owner.attrs(js[0], cls_here)
                if ja.get("type", "hinge") != "hinge":
                    raise NotImplementedError(f"robot {name}: {ja.get('type')} joints (hinges only)")
                rng = [float(x) for x in ja.get("range", "-3.141592653589793 3.141592653589793").split()]
                if not owner.radian:
                    rng = [math.radians(x) for x in rng]
                joints.append(dict(T0=Tb, pos=_vec3(ja, "pos"), axis=_vec3(ja, "axis", (0, 0, 1)), range=rng))
                ji = len(joints) - 1
            for g in b.findall("geom"):
                ga = owner.attrs(g, cls_here)
                if int(ga.get("contype", "1")) == 0 and int(ga.get("conaffinity", "1")) == 0:
                    continue
                t = ga.get("type", "sphere")
                if t == "plane":
                    continue
                gR, gp = owner.frame_R(ga), _vec3(ga, "pos")
                sz = [float(x) for x in ga.get("size", "0").split()]
                if "fromto" in ga:
                    ft = [float(x) for x in ga["fromto"].split()]
                    p0, p1 = np.array(ft[:3]), np.array(ft[3:])
                    if t not in ("capsule", "cylinder"):
                        raise NotImplementedError(f"robot {name}: fromto {t} geoms")
                    sph = _capsule_spheres(p0, p1, sz[0])
                elif t in ("capsule", "cylinder"):
                    ax = gR @ np.array([0.0, 0.0, sz[1]])
                    # a cylinder is covered as the capsule around it (conservative)
                    sph = _capsule_spheres(gp - ax, gp + ax, sz[0])
                elif t == "sphere":
                    sph = [(gp, sz[0])]
                elif t == "box":
                    sph = _box_cover_spheres(gp, gR, sz[:3])
                else:
                    raise NotImplementedError(f"robot {name}: {t} collision geoms")
                geoms.append(dict(joint=ji, body_T0=Tb, spheres=sph))
            for c in b.findall("body"):
                walk(c, Tb, owner, cls_here, ji)
            for at in b.findall("attach"):
                m = owner.models[at.get("model")]
                sub = m.root.find("worldbody")
                tgt = [x for x in sub.iter("body") if x.get("name") == at.get("body")]
                if not tgt:
                    raise ValueError(f"attach: body {at.get('body')} not in model {at.get('model')}")
                walk(tgt[0], Tb, m, "main", ji)

        walk(body, T, owner, cls, -1)
        return joints, geoms

    for b in wb.findall("body"):
        a = mj.attrs(b, "main")
        T = _hom(mj.frame_R(a), _vec3(a, "pos"))
        if b.find("freejoint") is not None or any(j.get("type") == "free" for j in b.findall("joint")):
            first = len(boxes_lo)
            for g in b.findall("geom"):
                static_box(g, T, mj)
            movable[b.get("name")] = list(range(first, len(boxes_lo)))
            continue
        if has_joints(b, mj):
            joints, geoms = robot_chain(b, np.eye(4), mj, "main", b.get("name"))
            if not joints:
                raise NotImplementedError(f"robot {b.get('name')} has no hinge joints")
            robots.append(dict(name=b.get("name"), base=T, joints=joints, geoms=geoms))
            continue
        for g in b.findall("geom"):
            static_box(g, T, mj)
    for g in wb.findall("geom"):
        static_box(g, np.eye(4), mj)
    return robots, boxes_lo, boxes_hi, movable


def _joint_lines(robot):
    """Joint axes of a parsed chain at the zero configuration: world points
    and directions."""
    o, z = [], []
    for j in robot["joints"]:
        T = j["T0"]
        o.append(T[:3, :3] @ j["pos"] + T[:3, 3])
        z.append(T[:3, :3] @ (j["axis"] / np.linalg.norm(j["axis"])))
    return o, z


def load_mjcf_arms(source, robots=None) -> ArmScene:
    """ArmScene of an MJCF scene of articulated arms (such as the reference's
    mujoco_4_ur10_world_closer.xml, envs mujoco_env.py:1160-1210): each robot
    body's chain of hinge joints becomes a fixed-base standard-DH arm with
    fixed joint-angle offsets (``chain_to_dh``), its collision geoms sphere
    sets in the DH link frames (capsules and cylinders covered by spheres
    along the axis, conservatively), static and free-body boxes box
    obstacles (free bodies at their initial pose, ``scene.movable_boxes``).
    The configuration is the robots' joints in order (``robots`` names the
    robot bodies; default: file order).  Self-collision within one robot is
    not modelled (the sphere-set model tests robot-box and robot-robot
    pairs)."""
    parsed, lo, hi, movable = parse_mjcf_arms(source)
    byname = {r["name"]: r for r in parsed}
    names = [r["name"] for r in parsed] if robots is None else list(robots)
    missing = [n for n in names if n not in byname]
    if missing or not names:
        raise ValueError(f"robots not found: {missing or 'none in the file'}")
    R = len(names)
    q_off, n_links, base_pose = [], [], np.zeros((R, 12))
    dh = np.zeros((R, MAX_LINKS, 4))
    offsets, lims = [], []
    s_robot, s_link, s_loc, s_rad = [], [], [], []
    q = 0
    for r, n in enumerate(names):
        rb = byname[n]
        nj = len(rb["joints"])
        if nj > MAX_LINKS:
            raise NotImplementedError(f"robot {n}: {nj} joints (at most {MAX_LINKS})")
        o, z = _joint_lines(rb)
        frames, prm, off = chain_to_dh(o, z, base_x=rb["base"][:3, 0])
        base_pose[r, :9] = frames[0][:3, :3].reshape(-1)
        base_pose[r, 9:] = frames[0][:3, 3]
        for k in range(nj):
            a, d, al = prm[k]
            dh[r, k] = [a, d, math.cos(al), math.sin(al)]
        q_off.append(q)
        n_links.append(nj)
        offsets.extend(off)
        lims.extend([j["range"] for j in rb["joints"]])
        q += nj
        for g in rb["geoms"]:
            k = g["joint"] + 1            # link k rides on joint k (link 0: the base)
            F = frames[k]
            Tb = g["body_T0"]
            for c, rad in g["spheres"]:
                w = Tb[:3, :3] @ np.asarray(c) + Tb[:3, 3]
                s_robot.append(r)
                s_link.append(k)
                s_loc.append(F[:3, :3].T @ (w - F[:3, 3]))
                s_rad.append(rad)
    S = len(s_rad)
    scene = ArmScene(
        q_offset=np.array(q_off, dtype=np.int32), base_kind=np.zeros(R, dtype=np.int32), base_pose=base_pose,
        n_links=np.array(n_links, dtype=np.int32), dh=dh,
        sphere_robot=np.array(s_robot, dtype=np.int32), sphere_link=np.array(s_link, dtype=np.int32),
        sphere_local=np.array(s_loc, dtype=np.float64).reshape(-1, 3),
        sphere_radius=np.array(s_rad, dtype=np.float64),
        box_lo=np.array(lo, dtype=np.float64).reshape(-1, 3), box_hi=np.array(hi, dtype=np.float64).reshape(-1, 3),
        q_dim=q, limits=np.array(lims, dtype=np.float64).T, joint_offset=np.array(offsets, dtype=np.float64))
    scene.movable_boxes = movable
    scene.robot_names = names
    return scene


def mjcf_chain_centers(robot: dict, q) -> np.ndarray:
    """Sphere centres (world) of one parsed robot chain at joint values q,
    composing the MJCF body frames directly (each joint turns its body about
    its axis through its position): the reference construction that
    ``load_mjcf_arms``'s DH form is checked against."""
    joints = robot["joints"]
    # world transform of each joint's body as a function of q: the chain is
    # serial, so body j's frame = fixed part (zero configuration) with the
    # rotations of joints <= j applied about their world axes, innermost first
    o, z = _joint_lines(robot)
    Tj = []
    M = np.eye(4)
    for j in range(len(joints)):
        # rotation about joint j's (moved) axis
        oj = M[:3, :3] @ o[j] + M[:3, 3]
        zj = M[:3, :3] @ z[j]
        Rj = _axis_R(zj, q[j])
        M = _hom(Rj, oj - Rj @ oj) @ M
        Tj.append(M.copy())
    out = []
    for g in robot["geoms"]:
        T = Tj[g["joint"]] if g["joint"] >= 0 else np.eye(4)
        Tb = g["body_T0"]
        for c, _ in g["spheres"]:
            w0 = Tb[:3, :3] @ np.asarray(c) + Tb[:3, 3]
            out.append(T[:3, :3] @ w0 + T[:3, 3])
    return np.array(out)


# ---------------------------------------------------------------------------
# URDF planar multi-robot scenes
# ---------------------------------------------------------------------------
def _origin(el):
    o = el.find("origin") if el is not None else None
    if o is None:
        return np.eye(4)
    xyz = _vec(o, "xyz", 3)
    rpy = _vec(o, "rpy", 3)
    return _hom(_rpy_R(rpy), xyz)


def load_urdf_planar(source, robots=None) -> ArmScene:
    """ArmScene of a planar URDF scene such as the reference's pinocchio
    problems (assets/models/pinocchio/*.urdf; envs pinocchio_env.py:663-900):
    each robot is a link reached from a fixed frame by a prismatic joint along
    x, one along y and a revolute joint about z (the configuration's x, y,
    yaw; limits from the joints' <limit>), carrying collision cylinders (axis
    z), spheres or boxes; the links fixed to the root carry box obstacles.

    * Every robot moves in its own horizontal plane: a cylinder becomes the
      sphere of its radius at its centre, a box a chain of spheres covering
      its rectangle (as ``load_mjcf_planar``); sphere geoms are kept.
    * A static box whose height range misses every robot geom's is skipped
      (a robot never reaches it: the table under the robots); a static box
      must otherwise contain the robots' centre planes in its height range
      (so the sphere touches it exactly when the cylinder does).
    * Static spheres and cylinders become their bounding boxes (conservative).
    Robot frames must sit at x = y = 0 without rotation; rotated obstacles
    other than quarter turns about z raise ``NotImplementedError``."""
    text = source if isinstance(source, str) and source.lstrip().startswith("<") else Path(source).read_text()
    root = ET.fromstring(text)
    links = {l.get("name"): l for l in root.findall("link")}
    joints = root.findall("joint")
    child_of = {j.find("child").get("link"): j for j in joints}
    roots = [n for n in links if n not in child_of]
    if len(roots) != 1:
        raise ValueError(f"a URDF scene needs one root link, found {roots}")
    kids = {}
    for j in joints:
        kids.setdefault(j.find("parent").get("link"), []).append(j)

    def collisions(link):
        out = []
        for c in links[link].findall("collision"):
            g = c.find("geometry")
            out.append((_origin(c), g[0]))
        return out

    static, robot_found = [], {}

    def walk(link, T, movable_chain):
        for j in kids.get(link, []):
            child = j.find("child").get("link")
            Tj = T @ _origin(j)
            t = j.get("type")
            if t == "fixed":
                if movable_chain:
                    raise NotImplementedError(f"link {child}: fixed links below a robot joint")
                for To, g in collisions(child):
                    static.append((Tj @ To, g))
                walk(child, Tj, movable_chain)
            elif t in ("prismatic", "revolute", "continuous"):
                ax = _vec(j.find("axis"), "xyz", 3) if j.find("axis") is not None else np.array([1.0, 0, 0])
                lim = j.find("limit")
                rng = (float(lim.get("lower", "-3.141592653589793")), float(lim.get("upper", "3.141592653589793"))) \
                    if lim is not None else (-math.pi, math.pi)
                if not np.allclose(_origin(j), np.eye(4)):
                    raise NotImplementedError(f"joint {j.get('name')}: robot joints must sit at their parent's origin")
                chain = movable_chain + [("slide" if t == "prismatic" else "hinge", tuple(ax), rng, T)]
                if len(chain) == 3:
                    want = [("slide", (1.0, 0.0, 0.0)), ("slide", (0.0, 1.0, 0.0)), ("hinge", (0.0, 0.0, 1.0))]
                    if [(c[0], c[1]) for c in chain] != want:
                        raise NotImplementedError(f"robot {child}: joints must be prismatic x, prismatic y, "
                                                  "revolute z")
                    F = chain[0][3]
                    if not np.allclose(F[:3, :3], np.eye(3)) or abs(F[0, 3]) > 0 or abs(F[1, 3]) > 0:
                        raise NotImplementedError(f"robot {child}: its frame must sit at x = y = 0 unrotated")
                    geoms = collisions(child)

                    def fixed_below(l, Trel):   # links fixed below the robot body ride with it
                        for jj in kids.get(l, []):
                            if jj.get("type") != "fixed":
                                raise NotImplementedError(f"robot {child}: moving links below a robot body")
                            c2 = jj.find("child").get("link")
                            T2 = Trel @ _origin(jj)
                            geoms.extend((T2 @ To, g) for To, g in collisions(c2))
                            fixed_below(c2, T2)

                    fixed_below(child, np.eye(4))
                    robot_found[child] = (float(F[2, 3]), np.array([c[2] for c in chain]).T, geoms)
                else:
                    walk(child, Tj, chain)
            else:
                raise NotImplementedError(f"joint type {t}")

    walk(roots[0], np.eye(4), [])
    for To, g in collisions(roots[0]):
        static.append((To, g))
    names = list(robot_found) if robots is None else list(robots)
    missing = [n for n in names if n not in robot_found]
    if missing or not names:
        raise ValueError(f"robots not found: {missing or 'none in the file'}")
    R = len(names)
    base_pose = np.zeros((R, 12))
    lims, s_robot, s_loc, s_rad, zr = [], [], [], [], []
    for r, n in enumerate(names):
        z, lim, geoms = robot_found[n]
        base_pose[r, :9] = np.eye(3).reshape(-1)
        base_pose[r, 9:] = [0.0, 0.0, z]
        lims.append(lim)
        for To, g in geoms:
            if not np.allclose(To[:3, :3], np.eye(3)):
                raise NotImplementedError(f"robot {n}: rotated collision geometry")
            p = To[:3, 3]
            if g.tag == "cylinder":
                rad, ln = float(g.get("radius")), float(g.get("length"))
                sph = [(p, rad)]
                zr.append((z + p[2] - ln / 2, z + p[2] + ln / 2, z + p[2]))
            elif g.tag == "sphere":
                rad = float(g.get("radius"))
                sph = [(p, rad)]
                zr.append((z + p[2] - rad, z + p[2] + rad, z + p[2]))
            elif g.tag == "box":
                half = 0.5 * _vec(g, "size", 3)
                sph = _box_spheres(p, half)
                zr.append((z + p[2] - half[2], z + p[2] + half[2], z + p[2]))
            else:
                raise NotImplementedError(f"robot {n}: {g.tag} collision geometry")
            for c, rad in sph:
                s_robot.append(r)
                s_loc.append(c)
                s_rad.append(rad)
    zlo, zhi = min(a for a, _, _ in zr), max(b for _, b, _ in zr)
    centres = [c for _, _, c in zr]
    lo_l, hi_l = [], []
    for T, g in static:
        Rm = T[:3, :3]
        if not np.allclose(np.abs(Rm), np.round(np.abs(Rm)), atol=1e-9):
            raise NotImplementedError("rotated obstacles do not map onto axis-aligned boxes")
        if g.tag == "box":
            h = 0.5 * _vec(g, "size", 3)
        elif g.tag == "sphere":
            h = np.full(3, float(g.get("radius")))
        elif g.tag == "cylinder":
            rr = float(g.get("radius"))
            h = np.array([rr, rr, 0.5 * float(g.get("length"))])
        else:
            raise NotImplementedError(f"static {g.tag} geometry")
        hw = np.abs(Rm) @ h
        lo, hi = T[:3, 3] - hw, T[:3, 3] + hw
        if hi[2] < zlo or lo[2] > zhi:
            continue                       # below or above every robot
        if not all(lo[2] <= c <= hi[2] for c in centres):
            raise NotImplementedError("an obstacle overlaps the robots' height range without containing their "
                                      "centre planes")
        lo_l.append(lo)
        hi_l.append(hi)
    S = len(s_rad)
    return ArmScene(
        q_offset=np.arange(R, dtype=np.int32) * 3, base_kind=np.ones(R, dtype=np.int32), base_pose=base_pose,
        n_links=np.zeros(R, dtype=np.int32), dh=np.zeros((R, MAX_LINKS, 4)),
        sphere_robot=np.array(s_robot, dtype=np.int32), sphere_link=np.zeros(S, dtype=np.int32),
        sphere_local=np.array(s_loc, dtype=np.float64).reshape(-1, 3), sphere_radius=np.array(s_rad, dtype=np.float64),
        box_lo=np.array(lo_l, dtype=np.float64).reshape(-1, 3), box_hi=np.array(hi_l, dtype=np.float64).reshape(-1, 3),
        q_dim=3 * R, limits=np.concatenate(lims, axis=1))
