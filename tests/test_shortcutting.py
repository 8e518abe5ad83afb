"""Shortcutting (planners/shortcutting.py:87-244) on the CPU: the restated
robot_mode_shortcut, with the oracle's exact verdicts and costs in place of
the device, reproduces the reference's own shortcut paths and cost traces
(shortcut.npz, made by the reference); the batched shortcutter keeps the end
states, never raises the cost and returns a path the oracle finds free."""
import numpy as np
import pytest

from conftest import golden, pkg

SLICES = [(0, 2), (2, 4)]


class _Mode:
    def __init__(self, task_ids):
        self.task_ids = list(task_ids)


class _State:
    def __init__(self, q, mode):
        self.q, self.mode = q, mode


def _oracle_env(oracle, scene):
    envm = pkg("env")
    o = oracle.OracleScene(scene)

    class OracleBacked:
        mode = -1
        kind = 0

        def is_collision_free_host(self, qs, robot_mask=None, flags=0):
            return o.configs_free(np.asarray(qs)).astype(np.uint8)

        def is_edge_collision_free_host(self, q1s, q2s, resolution, include_endpoints=False, N=None):
            return o.edges_free(np.asarray(q1s), np.asarray(q2s), resolution,
                                include_endpoints=include_endpoints, N=N).astype(np.uint8)

    env = object.__new__(envm.Gb300AbstractEnvironment)
    env._gb300 = OracleBacked()
    env.robots = ["a1", "a2"]
    env.robot_dims = {"a1": 2, "a2": 2}
    env.collision_resolution = 0.01
    env.batch_config_cost = lambda s, e, tmp_agent_slice=None: oracle.batch_cost(
        np.asarray(s, dtype=np.float64), None if e is None else np.asarray(e, dtype=np.float64), tmp_agent_slice)
    return env, o


def _fixture():
    g = golden("shortcut.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array(SLICES), agent_radii=[0.1, 0.1], box_center=g["centers"],
        box_bounds=2.0 * g["half"], sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)
    return g, scene


def _split(a, lens):
    off = np.concatenate([[0], np.cumsum(lens)])
    return [a[off[i]:off[i + 1]] for i in range(len(lens))]


def start_paths(g):
    cfg = pkg("configuration").Gb300Configuration
    modes = [_Mode(t) for t in g["task_ids"]]
    paths = []
    for qs, ms in zip(_split(g["starts"], g["start_len"]), _split(g["start_mode"], g["start_len"])):
        paths.append([_State(cfg(q, SLICES), modes[m]) for q, m in zip(qs, ms)])
    return paths, modes


def run_golden(env, g):
    """robot_mode_shortcut on every start path of the fixture, seeded as
    the reference was; asserts equality with its results."""
    sc = pkg("shortcutting")
    paths, modes = start_paths(g)
    outs = _split(g["outs"], g["out_len"])
    omodes = _split(g["out_mode"], g["out_len"])
    costs = _split(g["costs"], g["cost_len"])
    for p, path in enumerate(paths):
        np.random.seed(1000 + p)
        new, (cst, _t) = sc.robot_mode_shortcut(
            env, path, max_iter=120, resolution=0.01, tolerance=0.01,
            robot_choice="round_robin" if p % 2 == 0 else "random", interpolation_resolution=0.1)
        got = np.array([s.q.state() for s in new])
        assert got.shape == outs[p].shape, p
        np.testing.assert_array_equal(got, outs[p], err_msg=f"path {p}")
        assert [modes.index(s.mode) for s in new] == omodes[p].tolist(), p
        np.testing.assert_array_equal(np.array(cst), costs[p], err_msg=f"costs of path {p}")


def test_robot_mode_shortcut_golden(oracle):
    g, scene = _fixture()
    env, _ = _oracle_env(oracle, scene)
    run_golden(env, g)


def test_preprocessing_steps():
    """remove_interpolated_nodes keeps direction changes and mode switches
    and drops collinear states; interpolate_path spaces states by the
    max-abs metric and keeps the last state."""
    sc = pkg("shortcutting")
    cfg = pkg("configuration").Gb300Configuration
    m0, m1 = _Mode([0, 0]), _Mode([1, 0])
    qs = [[0, 0, 0, 0], [0.1, 0.1, 0, 0], [0.2, 0.2, 0, 0], [0.2, 0.5, 0, 0], [0.2, 0.8, 0, 0]]
    path = [_State(cfg(np.array(q, float), SLICES), m) for q, m in zip(qs, [m0, m0, m0, m1, m1])]
    kept = sc.remove_interpolated_nodes(path)
    assert [np.round(s.q.state()[:2], 3).tolist() for s in kept] == [[0, 0], [0.2, 0.2], [0.2, 0.5], [0.2, 0.8]]
    dense = sc.interpolate_path(kept, 0.05)
    assert dense[-1].q.state().tolist() == kept[-1].q.state().tolist()
    d = np.array([s.q.state() for s in dense])
    seg = [np.abs(kept[i + 1].q.state() - kept[i].q.state()).max() for i in range(len(kept) - 1)]
    n = [max(1, int(x / 0.05)) for x in seg]          # int() truncates: 0.3 / 0.05 < 6
    assert len(dense) == sum(n) + 1
    assert np.abs(np.diff(d, axis=0)).max() <= max(x / k for x, k in zip(seg, n)) + 1e-15
    assert [s.mode for s in dense] == [m0] * n[0] + [m0] * n[1] + [m1] * n[2] + [m1]


@pytest.mark.parametrize("robot_choice", ["round_robin", "random"])
def test_batched_shortcut_keeps_paths_free(oracle, robot_choice):
    g, scene = _fixture()
    env, o = _oracle_env(oracle, scene)
    sc = pkg("shortcutting")
    paths, _ = start_paths(g)
    for p, path in enumerate(paths[:6]):
        st = {}
        new, (cst, _t) = sc.batched_robot_mode_shortcut(env, path, rounds=8, batch=64, resolution=0.01,
                                                         robot_choice=robot_choice, interpolation_resolution=0.1,
                                                         rng=np.random.default_rng(p), stats=st)
        Q = np.array([s.q.state() for s in new])
        np.testing.assert_array_equal(Q[0], path[0].q.state())
        np.testing.assert_array_equal(Q[-1], path[-1].q.state())
        assert all(b <= a for a, b in zip(cst, cst[1:])), cst
        assert o.configs_free(Q).all()
        assert o.edges_free(Q[:-1], Q[1:], 0.01).all()
        assert st["accepted"] <= st["free"] <= st["improving"] <= st["proposed"]
        assert st["accepted"] >= 1


def test_batched_check_applies_the_env_tolerance_rule():
    """The batched shortcutter's per-mode path check applies the env's own
    verdict rule (the rai penetration tolerance) on top of the scene's
    verdicts, as the env's is_path_collision_free does, and leaves the
    scene's verdicts alone when the env has no tolerance."""
    sc_mod = pkg("shortcutting")

    class Scene:
        mode = 0

        def set_mode(self, m):
            self.mode = m

        def is_collision_free_host(self, q):
            return np.zeros(len(q), np.uint8)          # every vertex collides

        def is_edge_collision_free_host(self, a, b, res, incl):
            return np.zeros(len(a), np.uint8)          # every edge collides

    class Env:
        _gb300 = Scene()
        calls = []

        def __init__(self, tol):
            self.tol = tol

        @staticmethod
        def _mode_index(m):
            return m

        def _tol(self, t):
            return self.tol

        def _tolerate_configs(self, qs, v, tol):
            self.calls.append(("configs", len(qs), tol))
            return np.ones(len(qs), bool)

        def _tolerate_edges(self, a, b, v, res, incl, N, N_start, N_max, tol):
            self.calls.append(("edges", len(a), tol))
            return np.ones(len(a), bool)

    el = np.zeros((4, 2))
    modes = [0, 0, 1, 1]
    tolerant = Env(0.01)
    assert sc_mod._segments_free(tolerant, [el], [modes], 0.1).tolist() == [True]
    assert sorted(c[0] for c in tolerant.calls) == ["configs", "configs", "edges", "edges"]
    assert all(c[2] == 0.01 for c in tolerant.calls)
    Env.calls = []
    exact = Env(None)
    assert sc_mod._segments_free(exact, [el], [modes], 0.1).tolist() == [False]
    assert exact.calls == []


def test_batched_shortcut_on_an_env_without_batched_checks(oracle):
    """An env with only the reference's surface (is_path_collision_free,
    batch_config_cost, robots, robot_dims) runs the batched shortcutter
    too: each candidate goes through the env's own is_path_collision_free;
    the result keeps its ends, never raises the cost and is free."""
    g, scene = _fixture()
    o = oracle.OracleScene(scene)
    sc = pkg("shortcutting")
    calls = []

    class ReferenceLikeEnv:
        robots = ["a1", "a2"]
        robot_dims = {"a1": 2, "a2": 2}
        collision_resolution = 0.01

        def batch_config_cost(self, s, e, tmp_agent_slice=None):
            return oracle.batch_cost(np.asarray(s, dtype=np.float64), None if e is None else
                                     np.asarray(e, dtype=np.float64), tmp_agent_slice)

        def is_path_collision_free(self, path, resolution=None, tolerance=None, check_start_and_end=True):
            calls.append(len(path))
            Q = np.array([s.q.state() for s in path])
            inner = Q[1:-1] if not check_start_and_end else Q
            return bool(o.configs_free(inner).all() and o.edges_free(Q[:-1], Q[1:], resolution).all())

    env = ReferenceLikeEnv()
    paths, _ = start_paths(g)
    for p, path in enumerate(paths[:3]):
        new, (cst, _t) = sc.batched_robot_mode_shortcut(env, path, rounds=4, batch=32, resolution=0.01,
                                                         interpolation_resolution=0.1, rng=np.random.default_rng(p))
        Q = np.array([s.q.state() for s in new])
        np.testing.assert_array_equal(Q[0], path[0].q.state())
        np.testing.assert_array_equal(Q[-1], path[-1].q.state())
        assert all(b <= a for a, b in zip(cst, cst[1:])), cst
        assert o.configs_free(Q).all() and o.edges_free(Q[:-1], Q[1:], 0.01).all()
    assert calls
