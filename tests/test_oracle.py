"""The oracle against the reference's own outputs (golden vectors generated by
tests/golden/make_golden.py from the reference) -- the pin for every GPU parity
test.  CPU only."""
import json

import numpy as np
import pytest

from conftest import golden, pkg


def test_binary_indices_known_answers(oracle):
    # tests/test.py:36-47 of the reference
    expect = {1: (0,), 2: (0, 1), 3: (1, 0, 2), 4: (1, 0, 2, 3), 5: (2, 0, 3, 1, 4)}
    for n, e in expect.items():
        assert oracle.binary_search_indices(n) == e
        assert oracle.binary_search_indices_py(n) == e


def test_binary_indices_golden(oracle):
    g = golden("binary_indices.npz")
    off = 0
    for N in g["Ns"]:
        ref = tuple(int(x) for x in g["flat"][off:off + N])
        off += N
        assert oracle.binary_search_indices(int(N)) == ref
        if N <= 300:
            assert oracle.binary_search_indices_py(int(N)) == ref


def _disc_scene(g):
    scenes = pkg("scenes")
    return scenes.AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["centers"],
        box_bounds=2.0 * g["half"], sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)


def test_disc_scene_matches_generator():
    g = golden("abstract_disc.npz")
    s = pkg("scenes").make_disc_scene(0)
    assert np.array_equal(s.box_center, g["centers"]) and np.array_equal(s.box_bounds, 2.0 * g["half"])


def test_abstract_disc_configs(oracle):
    g = golden("abstract_disc.npz")
    o = oracle.OracleScene(_disc_scene(g))
    assert np.array_equal(o.configs_free(g["configs"]), g["config_free"])


def test_abstract_disc_edges_and_call_counts(oracle):
    g = golden("abstract_disc.npz")
    o = oracle.OracleScene(_disc_scene(g))
    variants = json.loads(str(g["variants"]))
    for vi, v in enumerate(variants):
        for e in range(len(g["q1"])):
            ref = int(g["edge_free"][vi, e])
            if ref == 255:   # N_start > N: the reference asserts
                with pytest.raises(ValueError):
                    o.edge_free(g["q1"][e], g["q2"][e], count=True, **v)
                continue
            free, calls = o.edge_free(g["q1"][e], g["q2"][e], count=True, **v)
            assert int(free) == ref, (vi, e)
            assert calls == g["edge_calls"][vi, e], (vi, e)


def test_abstract_test_scene(oracle):
    g = golden("abstract_test.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["box_center"],
        box_bounds=g["box_bounds"], sphere_pos=g["sphere_pos"], sphere_radius=[float(g["sphere_radius"][0])], q_dim=4)
    o = oracle.OracleScene(scene)
    assert np.array_equal(o.configs_free(g["configs"]), g["config_free"])
    assert np.array_equal(o.edges_free(g["q1"], g["q2"], float(g["resolution"])), g["edge_free"])


def test_abstract_10d(oracle):
    g = golden("abstract_10d.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 10], [10, 20]]), agent_radii=[0.1, 0.1], box_center=g["box_center"][None],
        box_bounds=g["box_bounds"][None], sphere_pos=np.zeros((0, 10)), sphere_radius=[], q_dim=20)
    o = oracle.OracleScene(scene)
    assert np.array_equal(o.configs_free(g["configs"]), g["config_free"])
    assert np.array_equal(o.edges_free(g["q1"], g["q2"], 0.05), g["edge_free"])


def test_primitives_3d(oracle):
    g = golden("primitives3d.npz")
    scenes = pkg("scenes")
    n = len(g["rect_hit"])
    for i in range(0, n, 7):
        s = scenes.AbstractScene(np.array([[0, 3]]), [float(g["sphere_r"][i])], g["box_center"][i][None],
                                 2.0 * g["box_half"][i][None], np.zeros((0, 3)), [], 3)
        assert oracle.OracleScene(s).config_free(g["sphere_c"][i]) == (not g["rect_hit"][i]), i
        s2 = scenes.AbstractScene(np.array([[0, 3]]), [float(g["rb"][i])], np.zeros((0, 3)), np.zeros((0, 3)),
                                  g["pa"][i][None], [float(g["ra"][i])], 3)
        assert oracle.OracleScene(s2).config_free(g["pb"][i]) == (not g["sphere_hit"][i]), i


TAGS = ["2_2", "7_7", "3_3_3", "2_5", "14", "7x4"]


@pytest.mark.parametrize("tag", TAGS)
def test_dist_cost(oracle, tag):
    g = golden("dist_cost.npz")
    pt, pts, sl = g[f"{tag}_pt"], g[f"{tag}_pts"], g[f"{tag}_slices"]
    for metric in ["euclidean", "sum_euclidean", "max_euclidean", "max"]:
        assert np.array_equal(oracle.batch_dist(pt, pts, sl, metric), g[f"{tag}_dist_{metric}"]), metric
    for metric in ["euclidean", "max"]:
        for red in ["max", "sum"]:
            assert np.array_equal(oracle.batch_cost(pt, pts, sl, metric, red), g[f"{tag}_cost_{metric}_{red}"])
            assert np.array_equal(oracle.batch_cost(pts[:300], pts[300:], sl, metric, red),
                                  g[f"{tag}_rowcost_{metric}_{red}"])
            assert np.array_equal(oracle.batch_cost(pts[:100], None, sl, metric, red),
                                  g[f"{tag}_pathcost_{metric}_{red}"])


def test_knn(oracle):
    g = golden("knn.npz")
    for metric in ["euclidean", "max_euclidean"]:
        idx, _ = oracle.knn(g["queries"], g["q_mode"], g["nodes"], g["mode_off"], g["slices"], metric, int(g["k"]))
        assert np.array_equal(idx, g[f"idx_{metric}"]), metric


def test_near(oracle):
    """Radius neighbours against the reference's find_nearest_indices, with
    radii on, just inside (by less than the added 1e-10) and just outside
    node distances, r = 0 and whole modes; an empty and a one-node mode."""
    g = golden("near.npz")
    for metric in ["euclidean", "max_euclidean"]:
        offs, idx, dist = oracle.near(g["queries"], g["q_mode"], g["nodes"], g["mode_off"], g["slices"], metric,
                                      g[f"radius_{metric}"])
        assert np.array_equal(offs, g[f"offsets_{metric}"]), metric
        assert np.array_equal(idx, g[f"idx_{metric}"]), metric
        assert np.all(dist <= g[f"radius_{metric}"][np.repeat(np.arange(len(offs) - 1), np.diff(offs))] + 1e-10)
        # the boundary cases are present: the added 1e-10 changes some selection
        o0, _, _ = oracle.near(g["queries"], g["q_mode"], g["nodes"], g["mode_off"], g["slices"], metric,
                               g[f"radius_{metric}"], add_eps=0.0)
        assert o0[-1] < offs[-1], metric


class _Node:
    """A graph node as the PRM search uses it (prm_graph.py:29-67)."""

    def __init__(self, i, q, mode=0):
        self.id = i
        self.state = type("State", (), {"q": q, "mode": mode})()
        self.whitelist, self.blacklist = set(), set()


def prm_search_case(g, tag):
    """Nodes, neighbour function, costs and heuristic of the stored search."""
    qs, nbr = g["configs"], g["neighbors"]
    nodes = [_Node(i, q) for i, q in enumerate(qs)]
    goal = nodes[int(g[f"goal_{tag}"])]
    return nodes, goal, (lambda n: ([nodes[j] for j in nbr[n.id]], qs[nbr[n.id]]))


@pytest.mark.parametrize("window", [1, 16])
def test_prm_lazy_search_golden(oracle, window):
    """The lazy A* restatement, with oracle edge checks and speculative
    windows of 1 and 16 edges, reproduces the reference's own search: the
    path (start twice, as its reconstruction writes it) and both counters,
    for a reachable and an unreachable goal."""
    lazy = pkg("lazy")
    g = golden("prm_search.npz")
    o = oracle.OracleScene(pkg("scenes").make_disc_scene(0))
    sl = [[0, 2], [2, 4]]
    bcost = lambda a, B: oracle.batch_cost(a, np.asarray(B), sl, "euclidean", "max", 0.01)
    cost = lambda a, b: float(bcost(a, np.asarray(b)[None])[0])
    res = float(g["resolution"])
    for tag in ("found", "missing"):
        nodes, goal, nb = prm_search_case(g, tag)
        h = lambda n: float(np.min(0.0 + bcost(n.state.q, goal.state.q[None])))
        checker = lazy.SpeculativeEdgeChecker(check=lambda q0, q1, m: o.edges_free(q0, q1, res).astype(bool),
                                              window=window)
        r = lazy.lazy_astar(nodes[0], [goal], nb, cost, bcost, h, checker)
        assert [n.id for n in r["path"]] == g[f"path_{tag}"].tolist(), tag
        assert r["processed_edges"] == int(g[f"processed_edges_{tag}"]), tag
        assert r["wasted_pops"] == int(g[f"wasted_pops_{tag}"]), tag
        if window > 1:
            assert r["calls"] < r["lookups"]


def test_known_answers_edge_calls(oracle):
    """tests/test.py:61-90 of the reference: 3 / 1 / 9 / 11 calls."""
    ka = golden("known_answers.json")
    g = golden("abstract_test.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["box_center"],
        box_bounds=g["box_bounds"], sphere_pos=g["sphere_pos"], sphere_radius=[float(g["sphere_radius"][0])], q_dim=4)
    o = oracle.OracleScene(scene)
    a, b = np.array([-1.0, 0, 1, 1]), np.array([-1.0, 1, 1, 0])
    assert o.edge_free(a, b, 0.01) == ka["edge_free"]
    # counting is_collision_free calls needs every check to pass: an empty scene
    empty = pkg("scenes").AbstractScene(np.array([[0, 2], [2, 4]]), [0.0, 0.0], np.zeros((0, 2)), np.zeros((0, 2)),
                                        np.zeros((0, 2)), [], 4)
    oe = oracle.OracleScene(empty)
    calls = [oe.edge_free(a, b, r, include_endpoints=inc, count=True)[1]
             for r, inc in [(0.5, True), (0.5, False), (0.1, False), (0.1, True)]]
    assert calls == ka["edge_calls"]


def test_sincos_close_to_libm(oracle):
    import math

    xs = np.concatenate([np.linspace(-30, 30, 20001), [0.0, -0.0, math.pi, -math.pi, 1e6, 1e-300]])
    for x in xs:
        s, c = oracle.sincos(float(x))
        assert abs(s - math.sin(x)) <= 4e-16 * max(1.0, abs(x) / 8) and abs(c - math.cos(x)) <= 4e-16 * max(1.0, abs(x) / 8)
    assert all(math.isnan(v) for v in oracle.sincos(float("inf")))
    assert all(math.isnan(v) for v in oracle.sincos(2.0 ** 31))


def test_oracle_robot_mask_semantics(oracle):
    """The masked check: all robots = is_collision_free; a robot's verdict
    ignores the other robots (their spheres and pairs with them)."""
    from conftest import pkg

    scenes = pkg("scenes")
    sc = scenes.make_arm_scene(0)
    o = oracle.OracleScene(sc)
    q = scenes.uniform_configs(sc, 500, seed=2, dtype=np.float64)
    assert np.array_equal(o.configs_free_for_robots(q, 0b1111), o.configs_free(q))
    single = [o.configs_free_for_robots(q, 1 << r) for r in range(4)]
    both = o.configs_free_for_robots(q, 0b0011)
    # a pair of robots is free only if each robot alone is free
    assert np.all(both <= single[0] & single[1])


def _path_fixture():
    g = golden("paths.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["centers"],
        box_bounds=2.0 * g["half"], sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)
    off = g["offsets"]
    paths = [g["states"][off[i]:off[i + 1]] for i in range(len(off) - 1)]
    return g, scene, paths, json.loads(str(g["variants"]))


def test_path_check_golden(oracle):
    """is_path_collision_free (planning_env.py:1765-1881): the env's batched
    path check (its vertex rules, every edge interior submitted at once) with
    the oracle's exact verdicts in place of the device gives the reference's
    own verdicts on 400 disc-scene paths under four flag variants."""
    import torch

    envm = pkg("env")
    g, scene, paths, variants = _path_fixture()
    o = oracle.OracleScene(scene)

    class OracleBacked:
        mode = -1

        def is_collision_free_host(self, qs):
            return o.configs_free(np.asarray(qs)).astype(np.uint8)

        def is_edge_collision_free_host(self, q1s, q2s, resolution, include_endpoints=False, N=None):
            return o.edges_free(np.asarray(q1s), np.asarray(q2s), resolution,
                                include_endpoints=include_endpoints, N=N).astype(np.uint8)

    env = object.__new__(envm.Gb300AbstractEnvironment)
    env._gb300 = OracleBacked()

    class S:
        def __init__(self, q):
            self.q, self.mode = q, None

    for vi, v in enumerate(variants):
        got = [int(env.is_path_collision_free([S(q) for q in qs], **v)) for qs in paths]
        assert got == g["free"][vi].tolist(), v


def test_batched_check_forms_golden(oracle):
    """The reference's is_collision_free and _batch_is_collision_free on
    configurations within 2e-16 of a Sphere obstacle's contact distance
    ('abstract.test'): the oracle's single-configuration check (the kernels'
    semantics) reproduces the first, its numpy restatement of the batched
    form the second, and the two reference forms differ on some of these
    ties (batch_forms.npz)."""
    g, a = golden("batch_forms.npz"), golden("abstract_test.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=a["box_center"],
        box_bounds=a["box_bounds"], sphere_pos=a["sphere_pos"], sphere_radius=[float(a["sphere_radius"][0])], q_dim=4)
    o = oracle.OracleScene(scene)
    assert np.array_equal(o.configs_free(g["configs"]), g["single"])
    got1 = np.array([oracle.batch_free_batched_form(scene, q[None]) for q in g["configs"]], dtype=np.uint8)
    assert np.array_equal(got1, g["batch1"])
    got8 = np.array([oracle.batch_free_batched_form(scene, g["configs"][grp]) for grp in g["groups"]], dtype=np.uint8)
    assert np.array_equal(got8, g["batch8"])
    assert 0 < int((g["single"] != g["batch1"]).sum()) < 200


def _fk_homogeneous(scene, q):
    """Sphere centres [S, 3] of one configuration from 4x4 homogeneous
    transforms: the base pose (planar bases: translation (x, y), then Rz(yaw),
    then the mount pose), then per link Rz(theta) Tz(d) Tx(a) Rx(alpha)
    (standard DH), spheres at their local offsets in their link frames."""
    def hom(R, p):
        T = np.eye(4)
        T[:3, :3], T[:3, 3] = R, p
        return T

    def rz(t):
        c, s = np.cos(t), np.sin(t)
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])

    off = np.zeros(scene.q_dim) if scene.joint_offset is None else np.asarray(scene.joint_offset, np.float64)
    q = np.asarray(q, dtype=np.float64) + off   # revolute joints turn by q + offset (planar x, y: offset 0)
    frames = []
    for r in range(scene.n_robots):
        bp = np.asarray(scene.base_pose[r], dtype=np.float64)
        mount = hom(bp[:9].reshape(3, 3), bp[9:])
        j = int(scene.q_offset[r])
        if scene.base_kind[r] == 1:
            T = hom(np.eye(3), [q[j], q[j + 1], 0.0]) @ hom(rz(q[j + 2]), np.zeros(3)) @ mount
            j += 3
        else:
            T = mount
        fr = [T]
        for k in range(int(scene.n_links[r])):
            a, d, ca, sa = scene.dh[r][k]
            rx = np.array([[1, 0, 0], [0, ca, -sa], [0, sa, ca]])
            T = T @ hom(rz(q[j + k]), [0, 0, 0]) @ hom(np.eye(3), [0, 0, d]) @ hom(np.eye(3), [a, 0, 0]) \
                @ hom(rx, np.zeros(3))
            fr.append(T)
        frames.append(fr)
    out = []
    for s in range(len(scene.sphere_radius)):
        T = frames[int(scene.sphere_robot[s])][int(scene.sphere_link[s])]
        out.append(T[:3, :3] @ np.asarray(scene.sphere_local[s]) + T[:3, 3])
    return np.array(out)


@pytest.mark.parametrize("factory", ["make_arm_scene", "make_mobile_scene"])
def test_arm_kinematics_with_joint_offsets(oracle, factory):
    """Fixed joint-angle offsets (the form imported general chains take):
    the oracle's frames agree with the homogeneous restatement, and a scene
    with offsets at q gives exactly the centres of the same scene without
    offsets at q + offset (one IEEE addition per joint)."""
    import copy

    scenes = pkg("scenes")
    sc = getattr(scenes, factory)(0)
    rng = np.random.default_rng(11)
    off = rng.uniform(-np.pi, np.pi, sc.q_dim)
    for r in range(sc.n_robots):
        if sc.base_kind[r] == 1:   # planar-base translations take no offset
            off[sc.q_offset[r]:sc.q_offset[r] + 2] = 0.0
    so = copy.deepcopy(sc)
    so.joint_offset = off
    o, o0 = oracle.OracleScene(so), oracle.OracleScene(sc)
    q = scenes.uniform_configs(sc, 40, seed=4, dtype=np.float64)
    for i in range(len(q)):
        got = o.sphere_centers(q[i])
        assert np.max(np.abs(got - _fk_homogeneous(so, q[i]))) <= 1e-12 * (1.0 + np.max(np.abs(got))), i
        assert np.array_equal(got, o0.sphere_centers(q[i] + off)), i


@pytest.mark.parametrize("factory", ["make_arm_scene", "make_mobile_scene"])
def test_arm_kinematics_independent_restatement(oracle, factory):
    """The arm kinematics have no counterpart in the reference: the oracle's
    C frames (composed row by row) agree with an independent homogeneous-
    matrix restatement of the same convention to 1e-12 of the reach, for
    fixed DH arms and planar mobile bases."""
    scenes = pkg("scenes")
    sc = getattr(scenes, factory)(0)
    o = oracle.OracleScene(sc)
    q = scenes.uniform_configs(sc, 50, seed=3, dtype=np.float64)
    for i in range(len(q)):
        got, want = o.sphere_centers(q[i]), _fk_homogeneous(sc, q[i])
        assert got.shape == want.shape == (len(sc.sphere_radius), 3)
        assert np.max(np.abs(got - want)) <= 1e-12 * (1.0 + np.max(np.abs(want))), i
