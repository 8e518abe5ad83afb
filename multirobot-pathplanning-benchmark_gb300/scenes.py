"""Scene descriptions and seeded synthetic workloads.

Two scene kinds mirror what the reference's abstract backend and the new
sphere-arm backend describe:

* ``AbstractScene`` -- spherical point agents (each agent's position is its
  slice of the configuration) among boxes (``Rectangle``) and sphere obstacles
  (``Sphere``), problems/abstract_env.py:41-131.
* ``ArmScene`` -- serial DH arms (optionally on a planar x, y, theta base)
  carrying collision spheres, among axis-aligned boxes.

The generators build the benchmark workloads with ``numpy.random.default_rng``
seeds; there is no dataset in the reference for this path, so every workload
is synthetic with the stated shapes and distributions.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

MAX_LINKS = 8


# ---------------------------------------------------------------------------
# Abstract point-agent scenes
# ---------------------------------------------------------------------------
@dataclass
class AbstractScene:
    agent_slices: np.ndarray          # [A, 2] (start, end) into q
    agent_radii: list                 # python floats, as AbstractEnvironment.agent_radii
    box_center: np.ndarray            # [nb, dim]
    box_bounds: np.ndarray            # [nb, dim] full side lengths (Rectangle.bounds)
    sphere_pos: np.ndarray            # [ns, dim]
    sphere_radius: list               # python floats
    q_dim: int

    @property
    def dim(self) -> int:
        return int(self.agent_slices[0, 1] - self.agent_slices[0, 0])

    def tables(self) -> dict:
        """Exact FP64 tables computed with the reference's own expressions."""
        A = len(self.agent_radii)
        dim = self.dim
        if np.shape(self.agent_slices) != (A, 2):
            raise ValueError(f"agent_slices {np.shape(self.agent_slices)} must be [{A}, 2] (one per agent radius)")
        for s, e in self.agent_slices:
            if e - s != dim:
                raise ValueError("all agents must have the obstacle dimension")
        nb = np.size(self.box_center) // max(dim, 1)
        if np.size(self.box_center) != nb * dim or np.size(self.box_bounds) != nb * dim:
            raise ValueError(f"box_center {np.shape(self.box_center)} and box_bounds {np.shape(self.box_bounds)} "
                             f"must both be [nb, {dim}]")
        if np.size(self.sphere_pos) != len(self.sphere_radius) * dim:
            raise ValueError(f"sphere_pos {np.shape(self.sphere_pos)} must be [{len(self.sphere_radius)}, {dim}]")
        # Rectangle.__init__ (abstract_env.py:66-67)
        bc = np.asarray(self.box_center, dtype=np.float64).reshape(-1, dim)
        bb = np.asarray(self.box_bounds, dtype=np.float64).reshape(-1, dim)
        lo = bc - bb / 2
        hi = bc + bb / 2
        pair = np.zeros((A, A))
        for i in range(A):
            for j in range(A):
                pair[i, j] = self.agent_radii[i] + self.agent_radii[j]     # abstract_env.py:266
        r2 = np.array([r ** 2 for r in self.agent_radii], dtype=np.float64)  # radius**2 (:84)
        sthr = np.zeros((len(self.sphere_radius), A))
        for o, ro in enumerate(self.sphere_radius):
            for i in range(A):
                sthr[o, i] = ro + self.agent_radii[i]                       # abstract_env.py:47
        return dict(
            agent_offsets=np.ascontiguousarray(self.agent_slices[:, 0], dtype=np.int64),
            agent_radius=np.asarray(self.agent_radii, dtype=np.float64),
            pair_threshold=np.ascontiguousarray(pair, dtype=np.float64),
            agent_radius_sq=r2,
            box_lo=np.ascontiguousarray(lo, dtype=np.float64).reshape(-1, dim),
            box_hi=np.ascontiguousarray(hi, dtype=np.float64).reshape(-1, dim),
            sphere_pos=np.ascontiguousarray(self.sphere_pos, dtype=np.float64).reshape(-1, dim),
            sphere_radius=np.asarray(self.sphere_radius, dtype=np.float64),
            sphere_threshold=np.ascontiguousarray(sthr, dtype=np.float64),
        )


def make_disc_scene(seed: int = 0, n_boxes: int = 10):
    """Two disc robots (radius 0.1, 2-DoF each, q in [-1, 1]^4) among
    `n_boxes` boxes with centres U[-0.8, 0.8]^2 and half extents U[0.05, 0.2]."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-0.8, 0.8, (n_boxes, 2))
    half = rng.uniform(0.05, 0.2, (n_boxes, 2))
    return AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]], dtype=np.int64),
        agent_radii=[0.1, 0.1],
        box_center=centers,
        box_bounds=2.0 * half,
        sphere_pos=np.zeros((0, 2)),
        sphere_radius=[],
        q_dim=4,
    )


def make_disc_workload(seed: int = 0, n_configs: int = 10_000, n_edges: int = 1_000, n_queries: int = 1_000):
    """Configurations U[-1, 1]^4, edges between U[-1, 1]^4 endpoint pairs
    (checked at resolution 0.01), and distance-matrix queries."""
    rng = np.random.default_rng(seed + 1000)
    return dict(
        configs=rng.uniform(-1, 1, (n_configs, 4)),
        q1=rng.uniform(-1, 1, (n_edges, 4)),
        q2=rng.uniform(-1, 1, (n_edges, 4)),
        queries=rng.uniform(-1, 1, (n_queries, 4)),
        resolution=0.01,
    )


# ---------------------------------------------------------------------------
# Sphere-arm scenes
# ---------------------------------------------------------------------------
@dataclass
class ArmScene:
    q_offset: np.ndarray        # [R] int32
    base_kind: np.ndarray       # [R] int32 (0 fixed, 1 planar x,y,theta)
    base_pose: np.ndarray       # [R, 12] rotation (row-major) + translation
    n_links: np.ndarray         # [R] int32
    dh: np.ndarray              # [R, 8, 4] a, d, cos(alpha), sin(alpha)
    sphere_robot: np.ndarray    # [S] int32
    sphere_link: np.ndarray     # [S] int32 (0 = base frame)
    sphere_local: np.ndarray    # [S, 3]
    sphere_radius: np.ndarray   # [S]
    box_lo: np.ndarray          # [B, 3]
    box_hi: np.ndarray          # [B, 3]
    q_dim: int
    limits: np.ndarray = field(default=None)   # [2, q_dim]
    # per-mode scene tables (optional): the boxes above are the pool; mode m
    # keeps boxes mode_boxes[m] and the attached-object spheres whose
    # sphere_attach id is in mode_attach[m] (sphere_attach -1: robot sphere)
    sphere_attach: np.ndarray = field(default=None)   # [S] int32
    mode_boxes: list = field(default=None)
    mode_attach: list = field(default=None)
    # fixed joint-angle offsets (imported general chains): revolute joint j
    # turns by q[j] + joint_offset[j]
    joint_offset: np.ndarray = field(default=None)    # [q_dim] or None

    @property
    def n_robots(self) -> int:
        return len(self.q_offset)

    @property
    def n_modes(self) -> int:
        return 0 if self.mode_boxes is None else len(self.mode_boxes)

    def _mode_attach(self) -> list:
        """Attached-object ids per mode (none when ``mode_attach`` is None)."""
        if self.mode_attach is None:
            return [[] for _ in range(self.n_modes)]
        if len(self.mode_attach) != self.n_modes:
            raise ValueError(f"mode_attach has {len(self.mode_attach)} entries for {self.n_modes} modes")
        return list(self.mode_attach)

    def for_mode(self, m: int) -> "ArmScene":
        """The scene as mode ``m`` sees it: its boxes and the spheres present."""
        att = np.full(len(self.sphere_radius), -1) if self.sphere_attach is None else np.asarray(self.sphere_attach)
        on = (att < 0) | np.isin(att, np.asarray(self._mode_attach()[m], dtype=np.int64))
        bx = np.asarray(self.mode_boxes[m], dtype=np.int64)
        return ArmScene(
            q_offset=self.q_offset, base_kind=self.base_kind, base_pose=self.base_pose, n_links=self.n_links,
            dh=self.dh, sphere_robot=np.asarray(self.sphere_robot)[on], sphere_link=np.asarray(self.sphere_link)[on],
            sphere_local=np.asarray(self.sphere_local)[on], sphere_radius=np.asarray(self.sphere_radius)[on],
            box_lo=np.asarray(self.box_lo).reshape(-1, 3)[bx], box_hi=np.asarray(self.box_hi).reshape(-1, 3)[bx],
            q_dim=self.q_dim, limits=self.limits, joint_offset=self.joint_offset)

    def mode_tables(self) -> dict:
        """Flat arrays for the library: attachment ids and per-mode lists."""
        S = len(self.sphere_radius)
        att = np.full(S, -1, dtype=np.int32) if self.sphere_attach is None else np.asarray(self.sphere_attach, np.int32)
        if att.shape != (S,):
            raise ValueError(f"sphere_attach {att.shape} must hold one id per sphere ({S})")
        attach = self._mode_attach()
        bl = [np.asarray(b, dtype=np.int32).reshape(-1) for b in self.mode_boxes]
        al = [np.asarray(a, dtype=np.int32).reshape(-1) for a in attach]
        off = lambda ls: np.concatenate([[0], np.cumsum([len(x) for x in ls])]).astype(np.int64)
        cat = lambda ls: np.ascontiguousarray(np.concatenate(ls) if ls else np.zeros(0), dtype=np.int32)
        return dict(sphere_attach=np.ascontiguousarray(att), box_off=off(bl), boxes=cat(bl), attach_off=off(al),
                    attach=cat(al))

    def robot_dofs(self) -> list:
        return [int(self.n_links[r] + (3 if self.base_kind[r] == 1 else 0)) for r in range(self.n_robots)]

    def agent_slices(self) -> np.ndarray:
        return np.array([[o, o + d] for o, d in zip(self.q_offset, self.robot_dofs())], dtype=np.int64)

    def arrays(self) -> dict:
        """Flat arrays for the library, their shapes checked against the robot,
        sphere and box counts (the library reads exactly that many values)."""
        R = len(self.q_offset)
        S = len(self.sphere_radius)
        a = dict(
            q_offset=np.ascontiguousarray(self.q_offset, dtype=np.int32).reshape(-1),
            base_kind=np.ascontiguousarray(self.base_kind, dtype=np.int32).reshape(-1),
            base_pose=np.ascontiguousarray(self.base_pose, dtype=np.float64),
            n_links=np.ascontiguousarray(self.n_links, dtype=np.int32).reshape(-1),
            dh=np.ascontiguousarray(self.dh, dtype=np.float64),
            sphere_robot=np.ascontiguousarray(self.sphere_robot, dtype=np.int32).reshape(-1),
            sphere_link=np.ascontiguousarray(self.sphere_link, dtype=np.int32).reshape(-1),
            sphere_local=np.ascontiguousarray(self.sphere_local, dtype=np.float64),
            sphere_radius=np.ascontiguousarray(self.sphere_radius, dtype=np.float64).reshape(-1),
            box_lo=np.ascontiguousarray(self.box_lo, dtype=np.float64),
            box_hi=np.ascontiguousarray(self.box_hi, dtype=np.float64),
        )
        want = dict(q_offset=(R,), base_kind=(R,), base_pose=(R, 12), n_links=(R,), dh=(R, MAX_LINKS, 4),
                    sphere_robot=(S,), sphere_link=(S,), sphere_local=(S, 3), sphere_radius=(S,))
        for k, shape in want.items():
            if a[k].size != int(np.prod(shape)):
                raise ValueError(f"ArmScene.{k}: {a[k].shape} does not hold {shape} values")
            a[k] = a[k].reshape(shape)
        if a["box_lo"].size % 3 or a["box_lo"].size != a["box_hi"].size:
            raise ValueError(f"ArmScene boxes: box_lo {a['box_lo'].shape} and box_hi {a['box_hi'].shape} "
                             "must both be [B, 3]")
        a["box_lo"] = a["box_lo"].reshape(-1, 3)
        a["box_hi"] = a["box_hi"].reshape(-1, 3)
        off = np.zeros(self.q_dim) if self.joint_offset is None else np.asarray(self.joint_offset, np.float64)
        if off.size != self.q_dim:
            raise ValueError(f"ArmScene.joint_offset: {off.shape} does not hold {self.q_dim} values")
        a["joint_offset"] = np.ascontiguousarray(off.reshape(-1))
        return a


def _rz(theta: float) -> np.ndarray:
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def _link_spheres(rng, a, d, ca, sa, per_link, r_lo, r_hi):
    """Spheres evenly spaced along the segment from the previous joint origin
    to this link's origin, in this link's frame: the previous origin sits at
    -(a, d sin(alpha), d cos(alpha)) in frame k for T = Rz Tz(d) Tx(a) Rx(alpha)."""
    t = (np.arange(per_link) + 0.5) / per_link
    prev = -np.array([a, d * sa, d * ca])
    loc = (1.0 - t)[:, None] * prev[None, :]
    rad = rng.uniform(r_lo, r_hi, per_link)
    return loc, rad


def make_arm_scene(seed: int = 0, n_boxes: int = 50, n_links: int = 7, spheres_per_link: int = 6):
    """Four serial 7-DoF arms on the corners of a 1.2 m square table (bases at
    (+-0.6, +-0.6, 0), facing the centre).  DH a and d ~ U[0.1, 0.4] m,
    alpha = +-pi/2; 6 spheres per link, radius U[0.03, 0.07] m, spread along
    the link.  Boxes: centres uniform in [-0.75, 0.75]^2 x [0, 1] m, half
    extents U[0.02, 0.15]^3.  Configuration: 28-D, joints in [-pi, pi]."""
    rng = np.random.default_rng(seed)
    R = 4
    corners = np.array([[0.6, 0.6], [-0.6, 0.6], [-0.6, -0.6], [0.6, -0.6]])
    base_pose = np.zeros((R, 12))
    dh = np.zeros((R, MAX_LINKS, 4))
    s_robot, s_link, s_loc, s_rad = [], [], [], []
    for r in range(R):
        yaw = np.arctan2(-corners[r, 1], -corners[r, 0])
        base_pose[r, :9] = _rz(yaw).reshape(-1)
        base_pose[r, 9:] = [corners[r, 0], corners[r, 1], 0.0]
        for k in range(n_links):
            a = rng.uniform(0.1, 0.4)
            d = rng.uniform(0.1, 0.4)
            sa = float(rng.choice([-1.0, 1.0]))
            dh[r, k] = [a, d, 0.0, sa]
            loc, rad = _link_spheres(rng, a, d, 0.0, sa, spheres_per_link, 0.03, 0.07)
            s_robot += [r] * spheres_per_link
            s_link += [k + 1] * spheres_per_link
            s_loc.append(loc)
            s_rad.append(rad)
    c = np.stack([rng.uniform(-0.75, 0.75, n_boxes), rng.uniform(-0.75, 0.75, n_boxes), rng.uniform(0.0, 1.0, n_boxes)], -1)
    h = rng.uniform(0.02, 0.15, (n_boxes, 3))
    D = R * n_links
    lim = np.stack([np.full(D, -np.pi), np.full(D, np.pi)])
    return ArmScene(
        q_offset=np.arange(R, dtype=np.int32) * n_links,
        base_kind=np.zeros(R, dtype=np.int32),
        base_pose=base_pose,
        n_links=np.full(R, n_links, dtype=np.int32),
        dh=dh,
        sphere_robot=np.array(s_robot, dtype=np.int32),
        sphere_link=np.array(s_link, dtype=np.int32),
        sphere_local=np.concatenate(s_loc),
        sphere_radius=np.concatenate(s_rad),
        box_lo=c - h,
        box_hi=c + h,
        q_dim=D,
        limits=lim,
    )


def make_arm_mode_scene(seed: int = 0, n_objects: int = 6, n_modes: int = 12, n_static: int = 40):
    """The four-arm table scene with movable objects, for per-mode tables.
    Each object j is a box (half extents U[0.03, 0.06] m) with two resting
    poses on the table (centres uniform in [-0.7, 0.7]^2, resting on z = 0)
    and a grasp by robot j % 4: held, it is three spheres of radius 0.04 m
    along the z axis of that robot's last link frame (offsets 0.05, 0.10,
    0.15 m).  Mode m draws, per object, resting pose A, pose B or held (at
    most one object per robot); the box pool is the static boxes then the
    objects' pose-A and pose-B boxes."""
    rng = np.random.default_rng(seed)
    sc = make_arm_scene(seed, n_boxes=n_static)
    R, L = sc.n_robots, int(sc.n_links[0])
    half = rng.uniform(0.03, 0.06, (n_objects, 3))
    lo, hi = [sc.box_lo], [sc.box_hi]
    for p in range(2):
        c = np.stack([rng.uniform(-0.7, 0.7, n_objects), rng.uniform(-0.7, 0.7, n_objects), half[:, 2]], -1)
        lo.append(c - half)
        hi.append(c + half)
    s_robot, s_link, s_loc, s_rad, s_att = [sc.sphere_robot], [sc.sphere_link], [sc.sphere_local], [sc.sphere_radius], \
        [np.full(len(sc.sphere_radius), -1, dtype=np.int32)]
    for j in range(n_objects):
        s_robot.append(np.full(3, j % R, dtype=np.int32))
        s_link.append(np.full(3, L, dtype=np.int32))
        s_loc.append(np.array([[0.0, 0.0, 0.05], [0.0, 0.0, 0.10], [0.0, 0.0, 0.15]]))
        s_rad.append(np.full(3, 0.04))
        s_att.append(np.full(3, j, dtype=np.int32))
    mode_boxes, mode_attach = [], []
    for m in range(n_modes):
        boxes, att, busy = list(range(n_static)), [], set()
        for j in range(n_objects):
            st = int(rng.integers(0, 3))
            if st == 2 and (j % R) not in busy:
                att.append(j)
                busy.add(j % R)
            else:
                boxes.append(n_static + (st % 2) * n_objects + j)
        mode_boxes.append(boxes)
        mode_attach.append(att)
    sc.box_lo, sc.box_hi = np.concatenate(lo), np.concatenate(hi)
    sc.sphere_robot, sc.sphere_link = np.concatenate(s_robot), np.concatenate(s_link)
    sc.sphere_local, sc.sphere_radius = np.concatenate(s_loc), np.concatenate(s_rad)
    sc.sphere_attach, sc.mode_boxes, sc.mode_attach = np.concatenate(s_att), mode_boxes, mode_attach
    return sc


def make_mobile_scene(seed: int = 0, n_robots: int = 8, n_boxes: int = 200):
    """Eight mobile manipulators: planar base (x, y, theta) carrying 8 spheres
    (radius 0.12 m on a 0.5 m footprint) and a 6-DoF DH arm mounted 0.3 m
    above the base origin (a, d ~ U[0.1, 0.4] m, alpha = +-pi/2, 5 spheres per
    link).  200 boxes in a 6 x 6 x 2 m room (centres uniform, half extents
    U[0.05, 0.25]).  Configuration: 8 x 9 = 72-D."""
    rng = np.random.default_rng(seed)
    L = 6
    base_pose = np.zeros((n_robots, 12))
    dh = np.zeros((n_robots, MAX_LINKS, 4))
    s_robot, s_link, s_loc, s_rad = [], [], [], []
    foot = np.array([[x, y, 0.15 - 0.3] for x, y in
                     [(0.25, 0.25), (-0.25, 0.25), (-0.25, -0.25), (0.25, -0.25), (0.25, 0.0), (-0.25, 0.0), (0.0, 0.25), (0.0, -0.25)]])
    for r in range(n_robots):
        base_pose[r, :9] = np.eye(3).reshape(-1)
        base_pose[r, 9:] = [0.0, 0.0, 0.3]
        s_robot += [r] * 8
        s_link += [0] * 8
        s_loc.append(foot)
        s_rad.append(np.full(8, 0.12))
        for k in range(L):
            a = rng.uniform(0.1, 0.4)
            d = rng.uniform(0.1, 0.4)
            sa = float(rng.choice([-1.0, 1.0]))
            dh[r, k] = [a, d, 0.0, sa]
            loc, rad = _link_spheres(rng, a, d, 0.0, sa, 5, 0.03, 0.07)
            s_robot += [r] * 5
            s_link += [k + 1] * 5
            s_loc.append(loc)
            s_rad.append(rad)
    c = np.stack([rng.uniform(-3, 3, n_boxes), rng.uniform(-3, 3, n_boxes), rng.uniform(0, 2, n_boxes)], -1)
    h = rng.uniform(0.05, 0.25, (n_boxes, 3))
    D = n_robots * (L + 3)
    lo = np.tile(np.array([-3.0, -3.0, -np.pi] + [-np.pi] * L), n_robots)
    return ArmScene(
        q_offset=np.arange(n_robots, dtype=np.int32) * (L + 3),
        base_kind=np.ones(n_robots, dtype=np.int32),
        base_pose=base_pose,
        n_links=np.full(n_robots, L, dtype=np.int32),
        dh=dh,
        sphere_robot=np.array(s_robot, dtype=np.int32),
        sphere_link=np.array(s_link, dtype=np.int32),
        sphere_local=np.concatenate(s_loc),
        sphere_radius=np.concatenate(s_rad),
        box_lo=c - h,
        box_hi=c + h,
        q_dim=D,
        limits=np.stack([lo, -lo]),
    )


def uniform_configs(scene, n: int, seed: int, dtype=np.float32) -> np.ndarray:
    rng = np.random.default_rng(seed)
    lim = scene.limits
    return rng.uniform(lim[0], lim[1], (n, lim.shape[1])).astype(dtype)


def edges_with_steps(scene, N: np.ndarray, resolution: float, seed: int, dtype=np.float32):
    """Edges whose interpolation count int(max|q2 - q1| / resolution) + 1 is
    exactly N: the largest joint change is (N - 0.5) * resolution, the others
    are uniform in +-that.  q1 is uniform in the joint limits."""
    rng = np.random.default_rng(seed)
    n = len(N)
    D = scene.limits.shape[1]
    q1 = rng.uniform(scene.limits[0], scene.limits[1], (n, D)).astype(dtype)
    m = (N.astype(np.float64) - 0.5) * resolution
    u = rng.uniform(-1.0, 1.0, (n, D))
    lead = rng.integers(0, D, n)
    u[np.arange(n), lead] = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    q2 = (q1.astype(np.float64) + u * m[:, None]).astype(dtype)
    got = (np.abs(q1.astype(np.float64) - q2.astype(np.float64)).max(1) / resolution).astype(np.int64) + 1
    got = np.maximum(got, 2)
    if not np.array_equal(got, N):
        raise AssertionError("edge step counts do not match after rounding")
    return q1, q2


def lognormal_steps(n: int, seed: int, median: float = 40.0, sigma: float = 0.6, lo: int = 5, hi: int = 500):
    rng = np.random.default_rng(seed)
    return np.clip(np.round(rng.lognormal(np.log(median), sigma, n)), lo, hi).astype(np.int64)


def make_arm_workload(scene: ArmScene, seed: int = 0, n_configs: int = 1_000_000, n_edges: int = 100_000,
                      resolution: float = 0.05):
    """1M uniform configurations and 100k edges with lognormal step counts
    (median 40, sigma 0.6, clipped to 5..500) at resolution 0.05 rad."""
    N = lognormal_steps(n_edges, seed + 7)
    q1, q2 = edges_with_steps(scene, N, resolution, seed + 11)
    return dict(configs=uniform_configs(scene, n_configs, seed + 3), q1=q1, q2=q2, N=N, resolution=resolution)


def make_knn_workload(seed: int = 0, n_nodes: int = 200_000, n_modes: int = 16, n_centers: int = 64,
                      n_queries: int = 4096, dim: int = 28, agents: int = 4, zipf: float = 1.1, sigma: float = 0.3):
    """Per-mode nearest-neighbour workload on the four-arm configuration space:
    `n_nodes` nodes in `dim`-D as Gaussian clusters (sigma rad) around
    `n_centers` centres uniform in [-pi, pi]^dim, split over `n_modes` modes
    with Zipf(`zipf`) sizes; `n_queries` queries uniform in [-pi, pi]^dim,
    each in a mode drawn with the same Zipf probabilities.  Agent slices are
    `agents` equal blocks (max_euclidean = max over the blocks)."""
    rng = np.random.default_rng(seed)
    p = 1.0 / np.arange(1, n_modes + 1) ** zipf
    p /= p.sum()
    sizes = np.floor(p * n_nodes).astype(np.int64)
    sizes[0] += n_nodes - sizes.sum()
    centers = rng.uniform(-np.pi, np.pi, (n_centers, dim))
    which = rng.integers(0, n_centers, n_nodes)
    nodes = centers[which] + rng.normal(0.0, sigma, (n_nodes, dim))
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    queries = rng.uniform(-np.pi, np.pi, (n_queries, dim))
    q_mode = rng.choice(n_modes, n_queries, p=p).astype(np.int32)
    blk = dim // agents
    slices = np.array([[a * blk, (a + 1) * blk] for a in range(agents)], dtype=np.int64)
    return dict(nodes=nodes, mode_offsets=offsets, queries=queries, q_mode=q_mode, slices=slices, k=10)


def make_path_workload(scene: ArmScene, seed: int = 0, n_paths: int = 512, n_waypoints: int = 256,
                       noise: float = 0.05, is_free=None) -> np.ndarray:
    """Paths for the penetration cost: straight lines between endpoints drawn
    uniform in the joint limits (only collision-free ones when ``is_free``,
    a callable on [n, D] float32 arrays returning per-row verdicts, is given),
    interior waypoints perturbed by N(0, noise^2) per joint.  FP32 [P, T, D]."""
    rng = np.random.default_rng(seed)
    lim = scene.limits
    D = lim.shape[1]
    need = 2 * n_paths
    ends = []
    got = 0
    for _ in range(10_000):
        if got >= need:
            break
        cand = rng.uniform(lim[0], lim[1], (max(4 * need, 1024), D)).astype(np.float32)
        if is_free is not None:
            cand = cand[np.asarray(is_free(cand)).astype(bool)]
        ends.append(cand)
        got += len(cand)
    if got < need:
        raise RuntimeError("could not draw enough collision-free endpoints")
    e = np.concatenate(ends)[:need]
    q1, q2 = e[:n_paths].astype(np.float64), e[n_paths:].astype(np.float64)
    s = np.linspace(0.0, 1.0, n_waypoints)
    paths = q1[:, None, :] + s[None, :, None] * (q2 - q1)[:, None, :]
    if n_waypoints > 2:
        paths[:, 1:-1] += rng.normal(0.0, noise, (n_paths, n_waypoints - 2, D))
    return paths.astype(np.float32)


def make_serving_requests(scene: ArmScene, seed: int = 0, n_instances: int = 64, configs=(100, 20_000),
                          edges=(10, 5_000), steps=(5, 800)) -> list:
    """One planner step of a serving load: each instance submits a uniform
    number of configurations (``configs`` range, inclusive) uniform in the
    joint limits and a uniform number of edges (``edges`` range) between
    endpoints uniform in the limits, each with an explicit interpolation count
    N uniform in ``steps``.  FP32 endpoints."""
    rng = np.random.default_rng(seed)
    lim = scene.limits
    D = lim.shape[1]
    out = []
    for _ in range(n_instances):
        nc = int(rng.integers(configs[0], configs[1] + 1))
        ne = int(rng.integers(edges[0], edges[1] + 1))
        out.append(dict(
            configs=rng.uniform(lim[0], lim[1], (nc, D)).astype(np.float32),
            q1=rng.uniform(lim[0], lim[1], (ne, D)).astype(np.float32),
            q2=rng.uniform(lim[0], lim[1], (ne, D)).astype(np.float32),
            N=rng.integers(steps[0], steps[1] + 1, ne).astype(np.int64),
        ))
    return out
