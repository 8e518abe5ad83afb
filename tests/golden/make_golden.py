"""Generate the golden vectors in this folder by running the REFERENCE itself.

Run in a container that has the reference checkout (it is not needed, and not
read, anywhere else):

    python tests/golden/make_golden.py /path/to/multirobot-pathplanning-benchmark

The reference imports numba, matplotlib and robotic at module level; none is
needed for the functions used here, so minimal stand-ins are put on sys.path:
numba.jit/njit become identity decorators (the kernels then run in plain
Python, i.e. in their written sequential IEEE order), matplotlib and robotic
become empty modules.  The package parents are pre-seeded so that
problems/__init__.py (which imports the rai scenes) is skipped.

Outputs (numpy .npz, seeded, small):
  binary_indices.npz     generate_binary_search_indices(N), N = 1..300 and a few large N
  abstract_disc.npz      2 discs + 10 boxes: config / edge verdicts, edge call counts
  abstract_test.npz      the reference's registered 'abstract.test' scene (sphere + box)
  abstract_10d.npz       'abstract.center_rect_10d': 10-D agents
  primitives3d.npz       Rectangle / Sphere collides_with_sphere in 3-D, incl. near-tangent
  dist_cost.npz          batch_config_dist / batch_config_cost over several slicings
  knn.npz                per-mode k nearest (argpartition + argsort, prm_graph.py:446-447)
  near.npz               per-mode radius neighbours (find_nearest_indices, rrtstar_base.py:439-453),
                         radii on and around node distances so that the added 1e-10 decides
  prm_search.npz         the composite PRM's lazy A* (MultimodalGraph.search, prm_graph.py:552-746)
                         on the disc scene over a fixed k-NN graph: path and printed counters
  known_answers.json     the reference tests' own known answers (tests/test.py)
  paths.npz              is_path_collision_free verdicts on the disc scene under four flag variants
                         (python tests/golden/make_golden.py <reference root> paths)
  batch_forms.npz        is_collision_free vs _batch_is_collision_free near a Sphere obstacle's contact
                         distance on 'abstract.test' (... <reference root> batch_forms)
  shortcut.npz           robot_mode_shortcut (planners/shortcutting.py:87-244) on the disc scene: start
                         paths, shortcut paths and cost traces (... <reference root> shortcut)
"""
from __future__ import annotations

import json
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def import_reference(ref_root: Path):
    src = ref_root / "src" / "multi_robot_multi_goal_planning"
    stub_dir = Path(tempfile.mkdtemp(prefix="mrmg_stubs_"))
    (stub_dir / "numba").mkdir()
    (stub_dir / "numba" / "__init__.py").write_text(
        "def jit(*a, **k):\n"
        "    if a and callable(a[0]) and not k: return a[0]\n"
        "    return lambda f: f\n"
        "njit = jit\n"
        "class _T:\n"
        "    def __getitem__(self, k): return self\n"
        "    def __call__(self, *a, **k): return self\n"
        "float64 = _T(); int64 = _T(); boolean = _T(); prange = range\n"
    )
    (stub_dir / "matplotlib").mkdir()
    (stub_dir / "matplotlib" / "__init__.py").write_text("")
    (stub_dir / "matplotlib" / "pyplot.py").write_text("")
    (stub_dir / "robotic").mkdir()
    (stub_dir / "robotic" / "__init__.py").write_text("")
    sys.path.insert(0, str(stub_dir))
    for name, path in [
        ("multi_robot_multi_goal_planning", src),
        ("multi_robot_multi_goal_planning.problems", src / "problems"),
        ("multi_robot_multi_goal_planning.problems.core", src / "problems" / "core"),
    ]:
        m = types.ModuleType(name)
        m.__path__ = [str(path)]
        sys.modules[name] = m
    import importlib

    pe = importlib.import_module("multi_robot_multi_goal_planning.problems.planning_env")
    ae = importlib.import_module("multi_robot_multi_goal_planning.problems.abstract_env")
    cf = importlib.import_module("multi_robot_multi_goal_planning.problems.core.configuration")
    reg = importlib.import_module("multi_robot_multi_goal_planning.problems.core.registry")
    return pe, ae, cf, reg


class CallCounter:
    def __init__(self, fn):
        self.fn = fn
        self.n = 0

    def __call__(self, *a, **k):
        self.n += 1
        return self.fn(*a, **k)


def disc_env(ae, reg, centers, half):
    env = reg.get_env_by_name("abstract.test")
    env.obstacles = [ae.Rectangle(centers[i], 2.0 * half[i]) for i in range(len(centers))]
    env.agent_radii = [0.1, 0.1]
    return env


def near_tangent_disc_configs(rng, centers, half, n):
    """Disc centres placed at distance 0.1 +- tiny from a box face or corner."""
    out = []
    for _ in range(n):
        b = rng.integers(len(centers))
        c, h = centers[b], half[b]
        side = rng.integers(4)
        eps = rng.choice([0.0, 1e-17, -1e-17, 1e-15, -1e-15, 1e-12, -1e-12, 1e-9, -1e-9])
        t = rng.uniform(-1, 1)
        if side == 0:
            p = [c[0] + h[0] + 0.1 + eps, c[1] + t * h[1]]
        elif side == 1:
            p = [c[0] - h[0] - 0.1 - eps, c[1] + t * h[1]]
        elif side == 2:
            p = [c[0] + t * h[0], c[1] + h[1] + 0.1 + eps]
        else:
            p = [c[0] + t * h[0], c[1] - h[1] - 0.1 - eps]
        other = rng.uniform(-1, 1, 2)
        out.append(np.array(p + list(other)) if rng.random() < 0.5 else np.array(list(other) + p))
    # agent - agent near 0.2 apart
    for _ in range(n // 2):
        a = rng.uniform(-0.5, 0.5, 2)
        ang = rng.uniform(0, 2 * np.pi)
        eps = rng.choice([0.0, 1e-16, -1e-16, 1e-12, -1e-12])
        b = a + (0.2 + eps) * np.array([np.cos(ang), np.sin(ang)])
        out.append(np.concatenate([a, b]))
    return np.array(out)


def main(ref_root: str):
    pe, ae, cf, reg = import_reference(Path(ref_root))
    Np = cf.NpConfiguration
    rng = np.random.default_rng(20240601)

    # --- binary search order -------------------------------------------------
    Ns = list(range(1, 301)) + [511, 512, 513, 777, 1000, 1024, 2049]
    flat = np.concatenate([np.array(pe.generate_binary_search_indices(N), dtype=np.int64) for N in Ns])
    np.savez_compressed(OUT / "binary_indices.npz", Ns=np.array(Ns, dtype=np.int64), flat=flat)

    # --- disc scene (2 discs r=0.1, 10 boxes) ----------------------------------
    srng = np.random.default_rng(0)
    centers = srng.uniform(-0.8, 0.8, (10, 2))
    half = srng.uniform(0.05, 0.2, (10, 2))
    env = disc_env(ae, reg, centers, half)
    start = env.start_pos
    configs = np.concatenate([rng.uniform(-1, 1, (3000, 4)), near_tangent_disc_configs(rng, centers, half, 1000)])
    cfg_free = np.array([env.is_collision_free(start.from_flat(q), None) for q in configs], dtype=np.uint8)
    q1 = rng.uniform(-1, 1, (400, 4))
    q2 = rng.uniform(-1, 1, (400, 4))
    # short edges too, so that some are free
    q1s = rng.uniform(-1, 1, (400, 4))
    q2s = q1s + rng.uniform(-0.05, 0.05, (400, 4))
    Q1 = np.concatenate([q1, q1s])
    Q2 = np.concatenate([q2, q2s])
    variants = [dict(resolution=0.01), dict(resolution=0.01, include_endpoints=True),
                dict(resolution=0.05, N_start=3, N_max=13), dict(resolution=0.02, N_start=10),
                dict(resolution=0.1, include_endpoints=True, N_start=1, N_max=4)]
    edge_out, edge_calls = [], []
    counter = CallCounter(env.is_collision_free)
    env.is_collision_free = counter
    for v in variants:
        outs, calls = [], []
        for a, b in zip(Q1, Q2):
            counter.n = 0
            qa, qb = start.from_flat(a), start.from_flat(b)
            N = int(cf.config_dist(qa, qb, "max") / v["resolution"]) + 1
            N = max(2, N)
            if v.get("N_start", 0) > N:
                outs.append(255)
                calls.append(-1)
                continue
            outs.append(int(env.is_edge_collision_free(qa, qb, None, **v)))
            calls.append(counter.n)
        edge_out.append(outs)
        edge_calls.append(calls)
    del env.is_collision_free
    np.savez_compressed(
        OUT / "abstract_disc.npz", centers=centers, half=half, configs=configs, config_free=cfg_free,
        q1=Q1, q2=Q2, edge_free=np.array(edge_out, dtype=np.uint8), edge_calls=np.array(edge_calls, dtype=np.int64),
        variants=json.dumps(variants),
    )

    # --- the reference's abstract.test scene (Sphere + Rectangle) -------------
    env = reg.get_env_by_name("abstract.test")
    start = env.start_pos
    configs = rng.uniform(-2, 2, (3000, 4))
    cfg_free = np.array([env.is_collision_free(start.from_flat(q), None) for q in configs], dtype=np.uint8)
    q1 = rng.uniform(-2, 2, (300, 4))
    q2 = q1 + rng.uniform(-0.4, 0.4, (300, 4))
    e_free = np.array([env.is_edge_collision_free(start.from_flat(a), start.from_flat(b), None) for a, b in zip(q1, q2)],
                      dtype=np.uint8)
    obs = env.obstacles
    np.savez_compressed(
        OUT / "abstract_test.npz", configs=configs, config_free=cfg_free, q1=q1, q2=q2, edge_free=e_free,
        sphere_pos=np.array([obs[0].pos]), sphere_radius=np.array([obs[0].radius]),
        box_center=np.array([obs[1].center]), box_bounds=np.array([obs[1].bounds]),
        resolution=env.collision_resolution,
    )

    # --- 10-D agents -----------------------------------------------------------
    env = reg.get_env_by_name("abstract.center_rect_10d")
    start = env.start_pos
    configs = rng.uniform(-0.6, 0.6, (2000, 20))
    cfg_free = np.array([env.is_collision_free(start.from_flat(q), None) for q in configs], dtype=np.uint8)
    q1 = rng.uniform(-1, 1, (200, 20))
    q2 = q1 + rng.uniform(-0.3, 0.3, (200, 20))
    e_free = np.array([env.is_edge_collision_free(start.from_flat(a), start.from_flat(b), None, resolution=0.05)
                       for a, b in zip(q1, q2)], dtype=np.uint8)
    np.savez_compressed(OUT / "abstract_10d.npz", configs=configs, config_free=cfg_free, q1=q1, q2=q2,
                        edge_free=e_free, box_center=env.obstacles[0].center, box_bounds=env.obstacles[0].bounds)

    # --- 3-D primitives ------------------------------------------------------------
    n = 8000
    bc = rng.uniform(-1, 1, (n, 3))
    bh = rng.uniform(0.02, 0.3, (n, 3))
    sc = rng.uniform(-1.5, 1.5, (n, 3))
    sr = rng.uniform(0.01, 0.2, n)
    # half of them moved to within a hair of contact along one axis
    for i in range(n // 2):
        k = rng.integers(3)
        sgn = rng.choice([-1.0, 1.0])
        sc[i] = bc[i] + rng.uniform(-1, 1, 3) * bh[i]
        sc[i, k] = bc[i, k] + sgn * (bh[i, k] + sr[i] + rng.choice([0.0, 1e-16, -1e-16, 1e-13, -1e-13]))
    rect = np.array([ae.Rectangle(bc[i], 2.0 * bh[i]).collides_with_sphere(sc[i], float(sr[i])) for i in range(n)], dtype=np.uint8)
    pa = rng.uniform(-1, 1, (n, 3))
    ra = rng.uniform(0.01, 0.2, n)
    rb = rng.uniform(0.01, 0.2, n)
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    gap = rng.choice([0.0, 1e-16, -1e-16, 1e-13, -1e-13, 0.01, -0.01], n)
    pb = pa + dirs * (ra + rb + gap)[:, None]
    sph = np.array([ae.Sphere(pa[i], float(ra[i])).collides_with_sphere(pb[i], float(rb[i])) for i in range(n)], dtype=np.uint8)
    np.savez_compressed(OUT / "primitives3d.npz", box_center=bc, box_half=bh, sphere_c=sc, sphere_r=sr, rect_hit=rect,
                        pa=pa, ra=ra, pb=pb, rb=rb, sphere_hit=sph)

    # --- distances / costs -----------------------------------------------------------
    dd = {}
    for tag, dims in [("2_2", [2, 2]), ("7_7", [7, 7]), ("3_3_3", [3, 3, 3]), ("2_5", [2, 5]), ("14", [14]), ("7x4", [7, 7, 7, 7])]:
        D = sum(dims)
        slices = [(sum(dims[:i]), sum(dims[:i + 1])) for i in range(len(dims))]
        pt = rng.uniform(-np.pi, np.pi, D)
        pts = rng.uniform(-np.pi, np.pi, (600, D))
        q = Np(pt, slices)
        dd[f"{tag}_pt"] = pt
        dd[f"{tag}_pts"] = pts
        dd[f"{tag}_slices"] = np.array(slices, dtype=np.int64)
        for metric in ["euclidean", "sum_euclidean", "max_euclidean", "max"]:
            dd[f"{tag}_dist_{metric}"] = cf.batch_config_dist(q, pts, metric)
        for metric in ["euclidean", "max"]:
            for red in ["max", "sum"]:
                dd[f"{tag}_cost_{metric}_{red}"] = cf.batch_config_cost(q, pts, metric, red)
                dd[f"{tag}_rowcost_{metric}_{red}"] = cf.batch_config_cost(pts[:300], pts[300:], metric, red,
                                                                           tmp_agent_slice=np.array(slices))
                dd[f"{tag}_pathcost_{metric}_{red}"] = cf.batch_config_cost(list(pts[:100]), None, metric, red,
                                                                            tmp_agent_slice=np.array(slices))
    np.savez_compressed(OUT / "dist_cost.npz", **dd)

    # --- per-mode kNN (PRM selection) --------------------------------------------------
    D = 28
    slices = [(7 * i, 7 * i + 7) for i in range(4)]
    sizes = [300, 120, 45, 9, 3]
    nodes = np.concatenate([rng.normal(rng.uniform(-np.pi, np.pi, D), 0.3, (s, D)) for s in sizes])
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    Q = 64
    qs = rng.uniform(-np.pi, np.pi, (Q, D))
    qm = rng.integers(0, len(sizes), Q).astype(np.int32)
    k = 10
    res = {}
    for metric in ["euclidean", "max_euclidean"]:
        idx = np.full((Q, k), -1, dtype=np.int64)
        for i in range(Q):
            arr = nodes[off[qm[i]]:off[qm[i] + 1]]
            dists = cf.batch_config_dist(Np(qs[i], slices), arr, metric)
            kc = min(k, len(arr))
            topk = np.argpartition(dists, kc - 1)[:kc]
            topk = topk[np.argsort(dists[topk])]
            idx[i, :kc] = topk
        res[f"idx_{metric}"] = idx
    np.savez_compressed(OUT / "knn.npz", nodes=nodes, mode_off=off, queries=qs, q_mode=qm, k=k,
                        slices=np.array(slices, dtype=np.int64), **res)

    # --- known answers from the reference's own tests (tests/test.py) -------------------
    env = reg.get_env_by_name("abstract.test")
    counter = CallCounter(env.is_collision_free)
    a = env.start_pos.from_flat(np.array([-1, 0, 1, 1]))
    b = env.start_pos.from_flat(np.array([-1, 1, 1, 0]))
    c3 = env.start_pos.from_flat(np.array([-1, 2, 1, -1]))
    ka = {"edge_free": bool(env.is_edge_collision_free(a, b, env.start_mode))}
    env.is_collision_free = lambda q, m: (setattr(counter, "n", counter.n + 1) or True)
    calls = []
    for res_, inc in [(0.5, True), (0.5, False), (0.1, False), (0.1, True)]:
        counter.n = 0
        env.is_edge_collision_free(a, b, env.start_mode, resolution=res_, include_endpoints=inc)
        calls.append(counter.n)
    ka["edge_calls"] = calls
    S = pe.State
    path = [S(a, env.start_mode), S(b, env.start_mode), S(c3, env.start_mode)]
    pcalls = []
    for res_, order in [(0.5, True), (0.5, False), (0.1, True), (0.1, False)]:
        counter.n = 0
        env.is_path_collision_free(path, resolution=res_, check_edges_in_order=order)
        pcalls.append(counter.n)
    ka["path_calls"] = pcalls
    del env.is_collision_free
    ka["path_free"] = bool(env.is_path_collision_free(path, resolution=0.5))
    (OUT / "known_answers.json").write_text(json.dumps(ka, indent=1))
    make_near(cf)
    make_prm_search(pe, ae, cf, reg)
    print("golden vectors written to", OUT)


def make_near(cf):
    """Radius neighbours per mode by the reference's own find_nearest_indices
    over batch_config_dist (RRT* near, rrtstar_base.py:1296-1337)."""
    src_mod = "multi_robot_multi_goal_planning.planners"
    if src_mod not in sys.modules:
        m = types.ModuleType(src_mod)
        m.__path__ = [str(Path(cf.__file__).resolve().parents[2] / "planners")]
        sys.modules[src_mod] = m
    import importlib

    rb = importlib.import_module(src_mod + ".rrtstar_base")
    rng = np.random.default_rng(20)
    D = 28
    slices = [(7 * i, 7 * i + 7) for i in range(4)]
    sizes = [400, 150, 33, 1, 0, 64]
    nodes = np.concatenate([rng.normal(rng.uniform(-np.pi, np.pi, D), 0.3, (s, D)) for s in sizes])
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    Q = 96
    qm = rng.integers(0, len(sizes), Q).astype(np.int32)
    qs = np.empty((Q, D))
    for i in range(Q):
        lo, hi = off[qm[i]], off[qm[i] + 1]
        if hi > lo and i % 4 != 3:     # near the mode's nodes, one query exactly on a node
            base = nodes[rng.integers(lo, hi)]
            qs[i] = base if i % 16 == 0 else base + rng.normal(0, 0.2, D)
        else:
            qs[i] = rng.uniform(-np.pi, np.pi, D)
    res = {}
    for metric in ["euclidean", "max_euclidean"]:
        radius = np.empty(Q)
        idx, offs = [], [0]
        for i in range(Q):
            arr = nodes[off[qm[i]]:off[qm[i] + 1]]
            q = cf.NpConfiguration(qs[i], slices)
            dists = cf.batch_config_dist(q, arr, metric) if len(arr) else np.zeros(0)
            kind = i % 6
            if len(dists) == 0:
                r = 0.7
            elif kind == 0:
                r = float(np.quantile(dists, 0.1))
            elif kind == 1:
                r = float(dists[rng.integers(len(dists))])             # a node exactly on the radius
            elif kind == 2:
                r = float(dists[rng.integers(len(dists))]) - 0.5e-10   # inside only by the added 1e-10
            elif kind == 3:
                r = float(dists[rng.integers(len(dists))]) - 2e-10     # just outside
            elif kind == 4:
                r = 0.0
            else:
                r = float(dists.max()) * 1.01                          # the whole mode
            radius[i] = r
            sel = rb.find_nearest_indices(dists, r) if len(dists) else np.zeros(0, dtype=np.int64)
            idx.append(np.asarray(sel, dtype=np.int64))
            offs.append(offs[-1] + len(sel))
        res[f"radius_{metric}"] = radius
        res[f"offsets_{metric}"] = np.array(offs, dtype=np.int64)
        res[f"idx_{metric}"] = np.concatenate(idx) if idx else np.zeros(0, dtype=np.int64)
    np.savez_compressed(OUT / "near.npz", nodes=nodes, mode_off=off, queries=qs, q_mode=qm,
                        slices=np.array(slices, dtype=np.int64), **res)


def _seed_planners(cf):
    import importlib

    base = "multi_robot_multi_goal_planning.planners"
    root = Path(cf.__file__).resolve().parents[2] / "planners"
    for name, path in [(base, root), (base + ".prm", root / "prm")]:
        if name not in sys.modules:
            m = types.ModuleType(name)
            m.__path__ = [str(path)]
            sys.modules[name] = m
    return importlib


def make_prm_search(pe, ae, cf, reg):
    """The reference's own MultimodalGraph.search (prm_graph.py:552-746) on
    the disc scene (the one of abstract_disc.npz) over a fixed graph: 250
    collision-free configurations, each joined to its 10 nearest (euclidean
    batch_config_dist, stable order), start = configuration 0, the goal the
    mode's only transition node (lower bound 0, so h is the cost to the
    goal), resolution 0.1.  Saved: the graph, the path as
    configuration indices and the counters the search prints, for a goal it
    reaches and one it cannot."""
    import contextlib
    import io

    importlib = _seed_planners(cf)
    pg = importlib.import_module("multi_robot_multi_goal_planning.planners.prm.prm_graph")
    srng = np.random.default_rng(0)
    centers = srng.uniform(-0.8, 0.8, (10, 2))
    half = srng.uniform(0.05, 0.2, (10, 2))
    env = disc_env(ae, reg, centers, half)
    mode = env.start_mode
    rng = np.random.default_rng(31)
    qs = []
    while len(qs) < 250:
        q = rng.uniform(-1, 1, 4)
        if env.is_collision_free(env.start_pos.from_flat(q), mode):
            qs.append(q)
    qs = np.array(qs)
    nodes = [pg.Node(pe.State(env.start_pos.from_flat(q), mode)) for q in qs]
    pos = {n.id: i for i, n in enumerate(nodes)}
    k = 10
    nbr = np.zeros((len(qs), k), dtype=np.int64)
    for i, n in enumerate(nodes):
        d = cf.batch_config_dist(n.state.q, qs, "euclidean")
        nbr[i] = np.argsort(d, kind="stable")[1:k + 1]
    def run(gi):
        for n in nodes:
            n.whitelist, n.blacklist = set(), set()
        goal = nodes[gi]
        goal.lb_cost_to_goal = 0.0
        graph = types.SimpleNamespace(
            get_neighbors=lambda n, space_extent=None: ([nodes[j] for j in nbr[pos[n.id]]], qs[nbr[pos[n.id]]]),
            transition_nodes={mode: [goal]}, transition_node_array_cache={}, transition_node_lb_cache={})
        out = io.StringIO()
        with contextlib.redirect_stdout(out):
            path = pg.MultimodalGraph.search(graph, nodes[0], [goal], env, best_cost=None, resolution=0.1)
        txt = out.getvalue()
        return ([pos[n.id] for n in path], int(txt.split("Wasted pops")[1].split()[0]),
                int(txt.split("Processed edges")[1].split()[0]))

    # goals: the first configuration (after 0) the search reaches over at
    # least five edges, and the first it cannot reach
    found = missing = None
    for gi in range(1, len(qs)):
        r = run(gi)
        if found is None and len(r[0]) >= 6:
            found = (gi,) + r
        if missing is None and not r[0]:
            missing = (gi,) + r
        if found and missing:
            break
    res = {}
    for tag, (gi, path, wasted, processed) in [("found", found), ("missing", missing)]:
        res[f"goal_{tag}"] = gi
        res[f"path_{tag}"] = np.array(path, dtype=np.int64)
        res[f"wasted_pops_{tag}"] = wasted
        res[f"processed_edges_{tag}"] = processed
    np.savez_compressed(OUT / "prm_search.npz", centers=centers, half=half, configs=qs, neighbors=nbr, start=0,
                        resolution=0.1, **res)


PATH_VARIANTS = [dict(resolution=0.01), dict(resolution=0.01, check_edges_in_order=True),
                 dict(resolution=0.02, check_start_and_end=False),
                 dict(resolution=0.02, check_edges_in_order=True, check_start_and_end=False)]


def make_paths(pe, ae, reg):
    """Verdicts of the reference's own is_path_collision_free
    (planning_env.py:1765-1881) on the disc scene: 400 paths of 2 to 6 states
    (random walks with steps up to 0.15 per coordinate, and some long jumps),
    under the flag variants of PATH_VARIANTS.  A one-state path makes the
    reference raise (generate_binary_search_indices(0) indexes an empty
    list), so none is generated."""
    srng = np.random.default_rng(0)
    centers = srng.uniform(-0.8, 0.8, (10, 2))
    half = srng.uniform(0.05, 0.2, (10, 2))
    env = disc_env(ae, reg, centers, half)
    rng = np.random.default_rng(77)
    paths, lens = [], []
    for p in range(400):
        P = int(rng.integers(2, 7))
        step = 0.15 if p % 4 else 0.8
        q = [rng.uniform(-1, 1, 4)]
        for _ in range(P - 1):
            q.append(np.clip(q[-1] + rng.uniform(-step, step, 4), -1, 1))
        paths.append(np.array(q))
        lens.append(P)
    free = []
    for v in PATH_VARIANTS:
        row = []
        for qs in paths:
            states = [pe.State(env.start_pos.from_flat(q), env.start_mode) for q in qs]
            row.append(int(env.is_path_collision_free(states, **v)))
        free.append(row)
    np.savez_compressed(OUT / "paths.npz", centers=centers, half=half, states=np.concatenate(paths),
                        offsets=np.concatenate([[0], np.cumsum(lens)]).astype(np.int64),
                        free=np.array(free, dtype=np.uint8), variants=json.dumps(PATH_VARIANTS))


def make_batch_forms(reg):
    """The reference's two forms of the configuration check on its
    'abstract.test' scene (Sphere r 0.2 at the origin, Rectangle above it):
    is_collision_free (abstract_env.py:255-276) and _batch_is_collision_free
    (:278-299) of one configuration at a time, for 4,000 configurations whose
    first or second disc sits within 2e-16 of the sphere obstacle's contact
    distance (the other disc far away), plus 200 batches of 8 of them."""
    env = reg.get_env_by_name("abstract.test")
    rng = np.random.default_rng(91)
    qs = []
    for k in range(4000):
        ang = rng.uniform(np.pi, 2 * np.pi)          # below the sphere: clear of the rectangle
        eps = rng.choice([0.0, 1e-17, -1e-17, 5e-17, -5e-17, 1e-16, -1e-16, 2e-16, -2e-16])
        p = (0.3 + eps) * np.array([np.cos(ang), np.sin(ang)])
        far = np.array([1.5, -1.5])
        qs.append(np.concatenate([p, far]) if k % 2 == 0 else np.concatenate([far, p]))
    qs = np.array(qs)
    single = np.array([env.is_collision_free(env.start_pos.from_flat(q), None) for q in qs], dtype=np.uint8)
    batch1 = np.array([env._batch_is_collision_free([env.start_pos.from_flat(q)], None) for q in qs], dtype=np.uint8)
    groups = rng.integers(0, len(qs), (200, 8))
    batch8 = np.array([env._batch_is_collision_free([env.start_pos.from_flat(qs[j]) for j in g], None)
                       for g in groups], dtype=np.uint8)
    np.savez_compressed(OUT / "batch_forms.npz", configs=qs, single=single, batch1=batch1, groups=groups,
                        batch8=batch8)


def make_shortcut(ref_root: Path, pe, ae, reg):
    """The reference's robot_mode_shortcut (planners/shortcutting.py:87-244)
    on the disc scene: 12 collision-free start paths (random walks whose
    states and edges the reference env accepts at resolution 0.01; the
    second half of every odd path in a second mode whose task of robot 0
    differs), shortcut under np.random.seed(1000 + p) with max_iter 120,
    resolution 0.01, interpolation_resolution 0.1, round-robin robots for
    even paths and random ones for odd paths.  Saved: the start paths, the
    shortcut paths and the cost trace (the returned costs list)."""
    import contextlib
    import importlib
    import io

    m = types.ModuleType("multi_robot_multi_goal_planning.planners")
    m.__path__ = [str(ref_root / "src" / "multi_robot_multi_goal_planning" / "planners")]
    sys.modules[m.__name__] = m
    sc = importlib.import_module("multi_robot_multi_goal_planning.planners.shortcutting")
    srng = np.random.default_rng(0)
    centers = srng.uniform(-0.8, 0.8, (10, 2))
    half = srng.uniform(0.05, 0.2, (10, 2))
    env = disc_env(ae, reg, centers, half)
    modes = [pe.Mode([0, 0], None), pe.Mode([1, 0], None)]
    rng = np.random.default_rng(4242)
    S = env.start_pos.from_flat
    starts, outs, costs, slen, olen, smode, omode, clen = [], [], [], [], [], [], [], []
    for p in range(12):
        P = int(rng.integers(5, 10))
        while True:
            q = rng.uniform(-1, 1, 4)
            if env.is_collision_free(S(q), None):
                break
        qs = [q]
        while len(qs) < P:
            c = np.clip(qs[-1] + rng.uniform(-0.35, 0.35, 4), -1, 1)
            if env.is_collision_free(S(c), None) and env.is_edge_collision_free(S(qs[-1]), S(c), None,
                                                                                resolution=0.01):
                qs.append(c)
        mi = [0] * P if p % 2 == 0 else [0] * (P // 2) + [1] * (P - P // 2)
        path = [pe.State(S(qs[t]), modes[mi[t]]) for t in range(P)]
        np.random.seed(1000 + p)
        with contextlib.redirect_stdout(io.StringIO()):
            new_path, (cst, _times) = sc.robot_mode_shortcut(
                env, path, max_iter=120, resolution=0.01, tolerance=0.01,
                robot_choice="round_robin" if p % 2 == 0 else "random", interpolation_resolution=0.1)
        starts.append(np.array(qs))
        smode += mi
        slen.append(P)
        outs.append(np.array([s.q.state() for s in new_path]))
        omode += [modes.index(s.mode) for s in new_path]
        olen.append(len(new_path))
        costs.append(np.array(cst, dtype=np.float64))
        clen.append(len(cst))
    np.savez_compressed(OUT / "shortcut.npz", centers=centers, half=half, starts=np.concatenate(starts),
                        start_len=np.array(slen, dtype=np.int64), start_mode=np.array(smode, dtype=np.int64),
                        outs=np.concatenate(outs), out_len=np.array(olen, dtype=np.int64),
                        out_mode=np.array(omode, dtype=np.int64), costs=np.concatenate(costs),
                        cost_len=np.array(clen, dtype=np.int64),
                        task_ids=np.array([md.task_ids for md in modes], dtype=np.int64))


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "shortcut":
        pe_, ae_, cf_, reg_ = import_reference(Path(sys.argv[1]))
        make_shortcut(Path(sys.argv[1]), pe_, ae_, reg_)
    elif len(sys.argv) > 2 and sys.argv[2] == "batch_forms":
        make_batch_forms(import_reference(Path(sys.argv[1]))[3])
    elif len(sys.argv) > 2 and sys.argv[2] == "paths":
        pe_, ae_, cf_, reg_ = import_reference(Path(sys.argv[1]))
        make_paths(pe_, ae_, reg_)
    elif len(sys.argv) > 2 and sys.argv[2] == "prm_search":
        pe_, ae_, cf_, reg_ = import_reference(Path(sys.argv[1]))
        make_prm_search(pe_, ae_, cf_, reg_)
    elif len(sys.argv) > 2 and sys.argv[2] == "near":
        make_near(import_reference(Path(sys.argv[1]))[2])
    else:
        if len(sys.argv) < 2:
            sys.exit("usage: make_golden.py <reference root> [batch_forms|paths|prm_search|near|shortcut]")
        main(sys.argv[1])
