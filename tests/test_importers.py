"""CPU checks of the MJCF planar-scene importer: the parsed geometry and
limits, exactness of the cylinder-to-sphere mapping against a direct 2-D
restatement of the planar problem (disc against rectangle, disc against
disc), the conservative cover of box robots (never free where the rotated
box touches an obstacle), the reference's own planar scene files (when its
checkout is present), and the refused forms."""
import os
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg

SCENE = """
<mujoco>
  <worldbody>
    <geom name="floor" type="plane" size="0 0 0.05" pos="0 0 -0.05"/>
    <body name="walls" pos="0 0 0.1">
      <geom type="box" pos="0 1.8 0" size="1.7 0.1 0.1"/>
      <geom type="box" pos="0 -1.8 0" size="1.7 0.1 0.1"/>
      <geom type="box" pos="1.8 0 0" size="0.1 1.7 0.1"/>
      <geom type="box" pos="-1.8 0 0" size="0.1 1.7 0.1"/>
      <geom type="box" pos="0.3 -0.2 0" size="0.4 0.3 0.1"/>
    </body>
    <body name="r_disc" pos="0 0 0.1">
      <joint name="d_x" type="slide" axis="1 0 0" range="-1.6 1.6"/>
      <joint name="d_y" type="slide" axis="0 1 0" range="-1.6 1.6"/>
      <joint name="d_t" type="hinge" axis="0 0 1" range="-180 180"/>
      <geom type="cylinder" size="0.12 0.05"/>
    </body>
    <body name="r_bar" pos="0 0 0.1">
      <joint name="b_x" type="slide" axis="1 0 0" range="-1.6 1.6"/>
      <joint name="b_y" type="slide" axis="0 1 0" range="-1.6 1.6"/>
      <joint name="b_t" type="hinge" axis="0 0 1" range="-90 90"/>
      <geom type="box" size="0.06 0.3 0.1"/>
    </body>
    <body name="crate" pos="-0.9 0.9 0.1">
      <freejoint/>
      <geom type="box" size="0.15 0.15 0.1"/>
    </body>
  </worldbody>
</mujoco>
"""


def _load(text=SCENE, robots=None):
    return pkg("importers").load_mjcf_planar(text, robots)


def test_mjcf_geometry_and_limits():
    sc = _load()
    assert sc.n_robots == 2 and sc.q_dim == 6
    assert len(sc.box_lo) == 6 and sc.movable_boxes == {"crate": [5]}
    np.testing.assert_allclose(sc.box_lo[4], [-0.1, -0.5, 0.0])
    np.testing.assert_allclose(sc.box_hi[5], [-0.75, 1.05, 0.2])
    np.testing.assert_allclose(sc.limits[:, 2], [-np.pi, np.pi])          # degrees -> radians
    np.testing.assert_allclose(sc.limits[:, 5], [-np.pi / 2, np.pi / 2])
    r0 = sc.sphere_radius[sc.sphere_robot == 0]
    r1 = sc.sphere_radius[sc.sphere_robot == 1]
    assert r0.tolist() == [0.12]
    assert np.allclose(r1, np.sqrt(2) * 0.06) and len(r1) == 5
    loc = sc.sphere_local[sc.sphere_robot == 1]
    assert np.all(loc[:, 0] == 0) and np.isclose(loc[:, 1].min(), -0.24) and np.isclose(loc[:, 1].max(), 0.24)
    assert np.diff(np.sort(loc[:, 1])).max() <= 2 * 0.06 + 1e-12   # a cover: centres at most 2 w apart
    assert _load(robots=["r_bar"]).n_robots == 1


def _rect_dist2(p, lo, hi):
    c = np.clip(p, lo, hi)
    return ((c - p) ** 2).sum(-1)


def test_cylinder_robots_are_exact(oracle):
    """Two cylinder robots: the oracle's verdicts on the imported scene equal
    the planar problem written directly (discs among rectangles)."""
    text = SCENE.replace('<geom type="box" size="0.06 0.3 0.1"/>', '<geom type="cylinder" size="0.2 0.05"/>')
    sc = _load(text)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(0)
    q = rng.uniform(sc.limits[0], sc.limits[1], (4000, 6))
    got = o.configs_free(q).astype(bool)
    lo, hi = sc.box_lo[:, :2], sc.box_hi[:, :2]
    want = np.ones(len(q), dtype=bool)
    for k, (off, r) in enumerate([(0, 0.12), (3, 0.2)]):
        d2 = _rect_dist2(q[:, None, off:off + 2], lo[None], hi[None])
        want &= ~(d2 <= r * r).any(1)
    want &= ~(np.sqrt(((q[:, 0:2] - q[:, 3:5]) ** 2).sum(1)) < 0.32)
    assert np.array_equal(got, want)
    assert 0.1 < want.mean() < 0.9


def _box_touches_rect(c, th, half, lo, hi):
    """Separating-axis test of a rotated rectangle against axis-aligned ones."""
    u = np.array([np.cos(th), np.sin(th)])
    v = np.array([-np.sin(th), np.cos(th)])
    corners = [c + sx * half[0] * u + sy * half[1] * v for sx in (-1, 1) for sy in (-1, 1)]
    P = np.array(corners)
    for l, h in zip(lo, hi):
        Q = np.array([[l[0], l[1]], [h[0], l[1]], [h[0], h[1]], [l[0], h[1]]])
        sep = False
        for ax in (np.array([1.0, 0.0]), np.array([0.0, 1.0]), u, v):
            a, b = P @ ax, Q @ ax
            if a.max() < b.min() or b.max() < a.min():
                sep = True
                break
        if not sep:
            return True
    return False


def test_box_robot_cover_is_conservative(oracle):
    """A configuration the covered model calls free never has the bar robot's
    true rectangle touching an obstacle."""
    sc = _load()
    keep = sc.sphere_robot == 1
    sc1 = pkg("importers").load_mjcf_planar(SCENE, ["r_bar"])
    o = oracle.OracleScene(sc1)
    rng = np.random.default_rng(1)
    q = rng.uniform(sc1.limits[0], sc1.limits[1], (1500, 3))
    free = o.configs_free(q).astype(bool)
    lo, hi = sc1.box_lo[:, :2], sc1.box_hi[:, :2]
    for i in np.nonzero(free)[0]:
        assert not _box_touches_rect(q[i, :2], q[i, 2], (0.06, 0.3), lo, hi), i
    assert keep.sum() == 5 and 0.05 < free.mean() < 0.95


# the reference checkout, named by MRMG_REFERENCE_ROOT (the test is skipped without it)
_REF_ROOT = os.environ.get("MRMG_REFERENCE_ROOT", "")
REF_MUJOCO = (Path(_REF_ROOT) / "src" / "multi_robot_multi_goal_planning" / "assets" / "models" / "mujoco"
              if _REF_ROOT else None)


@pytest.mark.skipif(REF_MUJOCO is None or not REF_MUJOCO.is_dir(),
                    reason="MRMG_REFERENCE_ROOT does not name a reference checkout")
@pytest.mark.parametrize("name", ["mj_two_dim.xml", "mj_hallway.xml", "mj_manip.xml", "mj_piano.xml"])
def test_reference_mujoco_scenes_import(oracle, name):
    """The reference's planar MuJoCo scene files (envs mujoco_env.py:891-1060)
    import as two planar-base robots a1, a2 (x, y, yaw each).  The limits are
    the compiled model's jnt_range (mujoco_env.py:194-198): slide ranges as
    written, hinge ranges in degrees (these files set no <compiler
    angle="radian">; mj_two_dim.xml's "-3.14 3.14" is therefore 0.0548 rad).
    Free bodies become movable boxes.  The start-free checks run on the
    oracle."""
    import xml.etree.ElementTree as ET

    path = REF_MUJOCO / name
    root = ET.fromstring(path.read_text())
    assert root.find("compiler") is None
    sc = pkg("importers").load_mjcf_planar(path)
    assert sc.n_robots == 2 and sc.q_dim == 6
    want = []
    for body in ("a1", "a2"):
        for j in root.find(".//body[@name='%s']" % body).findall("joint"):
            r = [float(x) for x in j.get("range").split()]
            want.append(np.deg2rad(r) if j.get("type") == "hinge" else r)
    np.testing.assert_allclose(sc.limits, np.array(want).T)
    free = {b.get("name") for b in root.iter("body") if b.find("freejoint") is not None}
    assert set(sc.movable_boxes) == free
    assert np.all(sc.sphere_radius > 0) and np.all(sc.box_hi > sc.box_lo)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(0)
    q = rng.uniform(sc.limits[0], sc.limits[1], (2000, 6))
    free_frac = o.configs_free(q).mean()
    assert 0.0 < free_frac < 1.0


@pytest.mark.parametrize("bad, err", [
    ('<geom type="box" pos="0.3 -0.2 0" size="0.4 0.3 0.1"/>',
     '<geom type="box" pos="0.3 -0.2 0" size="0.4 0.3 0.1" euler="0 0 30"/>'),
    ('<geom type="cylinder" size="0.12 0.05"/>', '<geom type="mesh" mesh="m"/>'),
    ('<body name="r_disc" pos="0 0 0.1">', '<body name="r_disc" pos="0.5 0 0.1">'),
    ('<joint name="d_t" type="hinge" axis="0 0 1" range="-180 180"/>',
     '<joint name="d_t" type="hinge" axis="0 1 0" range="-180 180"/>'),
])
def test_refused_forms(bad, err):
    with pytest.raises(NotImplementedError):
        _load(SCENE.replace(bad, err))


# ---------------------------------------------------------------------------
# articulated MJCF arms (general joint frames -> standard DH + joint offsets)
# ---------------------------------------------------------------------------
MJCF_ARMS = Path(__file__).resolve().parent / "golden" / "mjcf" / "two_arms.xml"


def test_mjcf_arms_dh_form_reproduces_the_body_frames(oracle):
    """Two six-joint arms (nested default classes, childclass, quaternion
    body frames, capsule collision geoms, <attach>, euler in degrees): the
    DH form with joint offsets that load_mjcf_arms builds gives, through the
    oracle's kinematics, the sphere centres of the MJCF body frames composed
    directly (each joint turning its body about its axis), to 1e-12."""
    imp = pkg("importers")
    robots, lo, hi, movable = imp.parse_mjcf_arms(MJCF_ARMS)
    sc = imp.load_mjcf_arms(MJCF_ARMS)
    assert sc.n_robots == 2 and sc.q_dim == 12 and list(sc.n_links) == [6, 6]
    assert len(sc.box_lo) == 2 and movable == {"crate": [0]}      # the free crate and the post
    assert np.allclose(sc.limits[:, 0], [-2.5, 2.5]) and np.allclose(sc.limits[:, 2], [-3.1, 3.1])
    assert np.any(sc.joint_offset != 0.0)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(2)
    for _ in range(40):
        q = rng.uniform(sc.limits[0], sc.limits[1])
        got = o.sphere_centers(q)
        want = np.concatenate([imp.mjcf_chain_centers(rb, q[6 * i:6 * i + 6]) for i, rb in enumerate(robots)])
        assert np.max(np.abs(got - want)) <= 1e-12


def test_capsule_cover_contains_the_capsule():
    """The spheres standing for a capsule cover every point of it."""
    imp = pkg("importers")
    rng = np.random.default_rng(4)
    for _ in range(20):
        p0, p1 = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
        r = rng.uniform(0.02, 0.2)
        sph = imp._capsule_spheres(p0, p1, r)
        t = rng.uniform(0, 1, 500)
        dirs = rng.normal(size=(500, 3))
        dirs /= np.linalg.norm(dirs, axis=1)[:, None]
        pts = p0 + t[:, None] * (p1 - p0) + dirs * (r * rng.uniform(0, 1, 500) ** (1 / 3))[:, None]
        c = np.array([s[0] for s in sph])
        rad = np.array([s[1] for s in sph])
        inside = (np.linalg.norm(pts[:, None] - c[None], axis=-1) <= rad[None] + 1e-12).any(1)
        assert inside.all()


def test_chain_to_dh_parallel_and_intersecting_axes():
    """Parallel, intersecting, anti-parallel and skew joint axes all give DH
    frames whose composition reproduces the frames the conversion reports."""
    imp = pkg("importers")
    cases = [
        ([[0, 0, 0], [0, 0, 0.5], [0.4, 0, 0.5]], [[0, 0, 1], [0, 1, 0], [0, 1, 0]]),   # parallel pair
        ([[0, 0, 0], [0, 0, 0.3], [0, 0, 0.3]], [[0, 0, 1], [1, 0, 0], [0, 1, 0]]),     # intersecting
        ([[0, 0, 0], [0.2, 0, 0], [0.2, 0.1, 0.4]], [[0, 0, 1], [0, 0, -1], [1, 1, 0]]),  # anti-parallel, skew
    ]
    for origins, axes in cases:
        frames, dh, off = imp.chain_to_dh(origins, axes)
        T = frames[0]
        for k, (a, d, al) in enumerate(dh):
            th = off[k]
            c, s, ca, sa = np.cos(th), np.sin(th), np.cos(al), np.sin(al)
            A = np.array([[c, -s * ca, s * sa, a * c], [s, c * ca, -c * sa, a * s], [0, sa, ca, d], [0, 0, 0, 1]])
            T = T @ A
            assert np.allclose(T, frames[k + 1], atol=1e-12), (origins, k)
        for k, (o_, z_) in enumerate(zip(origins, axes)):   # frame k's z lies on joint k+1's axis
            z = np.asarray(z_, float) / np.linalg.norm(z_)
            assert np.allclose(frames[k][:3, 2], z, atol=1e-12)
            w = frames[k][:3, 3] - np.asarray(o_, float)
            assert np.linalg.norm(w - (w @ z) * z) <= 1e-12


REF_MODELS = (Path(_REF_ROOT) / "src" / "multi_robot_multi_goal_planning" / "assets" / "models" if _REF_ROOT else None)


@pytest.mark.skipif(REF_MODELS is None or not REF_MODELS.is_dir(),
                    reason="MRMG_REFERENCE_ROOT does not name a reference checkout")
def test_reference_ur10_scene_imports(oracle):
    """The reference's four-UR10 MuJoCo scene (mujoco_env.py:1160-1210):
    four fixed-base six-joint arms and the free box, the DH form reproducing
    the MJCF body frames to 1e-12."""
    imp = pkg("importers")
    for name in ("mujoco_4_ur10_world_closer.xml", "mujoco_4_ur10_world_closer_movable_obj.xml"):
        p = REF_MODELS / "mujoco" / name
        robots, _, _, movable = imp.parse_mjcf_arms(p)
        sc = imp.load_mjcf_arms(p)
        assert sc.n_robots == 4 and sc.q_dim == 24 and list(sc.n_links) == [6] * 4
        assert set(movable) <= {"obj1", "obj2", "obj3", "obj4"}
        o = oracle.OracleScene(sc)
        rng = np.random.default_rng(5)
        for _ in range(20):
            q = rng.uniform(sc.limits[0], sc.limits[1])
            want = np.concatenate([imp.mjcf_chain_centers(rb, q[6 * i:6 * i + 6]) for i, rb in enumerate(robots)])
            assert np.max(np.abs(o.sphere_centers(q) - want)) <= 1e-12


@pytest.mark.skipif(REF_MODELS is None or not REF_MODELS.is_dir(),
                    reason="MRMG_REFERENCE_ROOT does not name a reference checkout")
def test_reference_pinocchio_urdf_scenes_import(oracle):
    """The reference's planar pinocchio scenes (pinocchio_env.py:663-900)
    import as planar-base robots among boxes; the start configurations the
    reference's envs declare are collision free (middle_obs:
    (0, -0.8, 0), (0, 0.8, 0); other_hallway: (1.5, 0, 0), (-1.5, 0, 0))."""
    imp = pkg("importers")
    for name in ("2d_handover.urdf", "middle_obstacle_two_agents.urdf", "other_hallway.urdf", "piano.urdf",
                 "random_2d.urdf"):
        sc = imp.load_urdf_planar(REF_MODELS / "pinocchio" / name)
        assert sc.n_robots in (2, 3) and sc.q_dim == 3 * sc.n_robots and len(sc.box_lo) > 0
    o = oracle.OracleScene(imp.load_urdf_planar(REF_MODELS / "pinocchio" / "middle_obstacle_two_agents.urdf"))
    assert o.config_free(np.array([0, -0.8, 0, 0, 0.8, 0.0]))
    assert not o.config_free(np.array([0, 0.0, 0, 0, 0.8, 0.0]))    # inside the middle obstacle
    o = oracle.OracleScene(imp.load_urdf_planar(REF_MODELS / "pinocchio" / "other_hallway.urdf"))
    assert o.config_free(np.array([1.5, 0, 0, -1.5, 0, 0.0]))


URDF_SCENE = """<?xml version="1.0"?>
<robot name="planar">
  <link name="table"><collision><geometry><box size="2 2 0.06"/></geometry></collision></link>
  <link name="wall"><collision><geometry><box size="2 0.2 0.06"/></geometry></collision></link>
  <joint name="t_w" type="fixed"><parent link="table"/><child link="wall"/><origin xyz="0 1.1 0.07" rpy="0 0 0"/></joint>
  <link name="post"><collision><geometry><box size="0.2 0.4 0.06"/></geometry></collision></link>
  <joint name="t_p" type="fixed"><parent link="table"/><child link="post"/><origin xyz="0.3 0 0.07" rpy="0 0 1.5707963267948966"/></joint>
  <link name="f1"/><link name="x1"/><link name="y1"/>
  <joint name="t_f1" type="fixed"><parent link="table"/><child link="f1"/><origin xyz="0 0 0.07" rpy="0 0 0"/></joint>
  <joint name="f1_x" type="prismatic"><parent link="f1"/><child link="x1"/><axis xyz="1 0 0"/><limit lower="-1" upper="1"/></joint>
  <joint name="f1_y" type="prismatic"><parent link="x1"/><child link="y1"/><axis xyz="0 1 0"/><limit lower="-1" upper="1"/></joint>
  <joint name="f1_t" type="revolute"><parent link="y1"/><child link="a1"/><axis xyz="0 0 1"/><limit lower="-3.14" upper="3.14"/></joint>
  <link name="a1"><collision><geometry><cylinder radius="0.1" length="0.06"/></geometry></collision></link>
  <link name="a1_tip"><collision><origin xyz="0.15 0 0"/><geometry><sphere radius="0.04"/></geometry></collision></link>
  <joint name="a1_t" type="fixed"><parent link="a1"/><child link="a1_tip"/></joint>
</robot>"""


def test_urdf_planar_scene_parsed_and_exact_in_the_plane(oracle):
    """A planar URDF scene: the table below the robots is dropped, the quarter-
    turned post becomes its rotated box, the fixed tip rides on the robot;
    verdicts equal a direct 2-D restatement (disc and tip disc against the
    wall and post rectangles)."""
    imp = pkg("importers")
    sc = imp.load_urdf_planar(URDF_SCENE)
    assert sc.n_robots == 1 and sc.q_dim == 3 and len(sc.box_lo) == 2
    assert np.allclose(sc.box_lo[1], [0.1, -0.1, 0.04]) and np.allclose(sc.box_hi[1], [0.5, 0.1, 0.10])
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(8)
    q = rng.uniform(sc.limits[0], sc.limits[1], (3000, 3))

    def rect_d2(p, lo, hi):
        c = np.clip(p, lo[:2], hi[:2])
        return ((c - p) ** 2).sum(-1)

    free = o.configs_free(q).astype(bool)
    for i in range(len(q)):
        x, y, t = q[i]
        tip = np.array([x + 0.15 * np.cos(t), y + 0.15 * np.sin(t)])
        hit = False
        for lo, hi in zip(sc.box_lo, sc.box_hi):
            hit |= rect_d2(np.array([x, y]), lo, hi) <= 0.1 ** 2 or rect_d2(tip, lo, hi) <= 0.04 ** 2
        assert free[i] == (not hit), i
