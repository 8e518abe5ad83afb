"""The rai engine's penetration tolerance (rai_base_env.py:442-700) on the
CPU: the env's rule -- a configuration that collides still counts as free
while the scene's total penetration depth is at most the tolerance; an edge
is free when every checked position is -- composed with the oracle's exact
verdicts and its total penetration, against a direct position-by-position
evaluation of the same rule.  The oracle's total penetration is zero on free
configurations and positive on colliding ones."""
import numpy as np

from conftest import pkg


def _oracle_arm_env(oracle, scene, tolerance):
    envm = pkg("env")
    o = oracle.OracleScene(scene)

    class OracleBacked:
        mode = -1
        kind = 1

        def is_collision_free_host(self, qs, robot_mask=0, flags=0):
            qs = np.atleast_2d(np.asarray(qs, dtype=np.float64))
            if robot_mask:
                return o.configs_free_for_robots(qs, robot_mask).astype(np.uint8)
            return o.configs_free(qs).astype(np.uint8)

        def config_free1(self, q, robot_mask=0):
            return bool(self.is_collision_free_host(q, robot_mask)[0])

        def is_edge_collision_free_host(self, q1s, q2s, resolution, include_endpoints=False, N=None):
            return o.edges_free(np.asarray(q1s), np.asarray(q2s), resolution,
                                include_endpoints=include_endpoints, N=N).astype(np.uint8)

        def edge_free1(self, a, b, resolution, include_endpoints=False, N=None, N_start=0, N_max=None):
            return bool(o.edges_free(a[None], b[None], resolution, include_endpoints=include_endpoints)[0])

        def total_penetration(self, qs):
            return o.total_penetration(qs)

    env = object.__new__(envm.Gb300ArmEnvironment)
    env._gb300 = OracleBacked()
    env.robots = [f"r{i}" for i in range(scene.n_robots)]
    env.collision_resolution = 0.05
    env.collision_tolerance = tolerance
    env.tolerance_semantics = True
    return env, o


def test_total_penetration_matches_exact_verdicts(oracle):
    scenes = pkg("scenes")
    sc = scenes.make_arm_scene(2, n_boxes=20)
    o = oracle.OracleScene(sc)
    q = scenes.uniform_configs(sc, 3000, seed=4, dtype=np.float64)
    free = o.configs_free(q).astype(bool)
    pen = o.total_penetration(q)
    assert 0 < free.sum() < len(q)
    assert (pen[free] == 0).all()
    assert (pen[~free] > 0).all()


def test_tolerance_rule_configs_and_edges(oracle):
    scenes = pkg("scenes")
    sc = scenes.make_arm_scene(2, n_boxes=20)
    q = scenes.uniform_configs(sc, 3000, seed=4, dtype=np.float64)
    _, o = _oracle_arm_env(oracle, sc, 0.0)
    pen = o.total_penetration(q)
    free = o.configs_free(q).astype(bool)
    tol = float(np.percentile(pen[~free], 30))
    env, _ = _oracle_arm_env(oracle, sc, tol)
    want = free | (pen <= tol)
    assert want.sum() > free.sum()
    assert np.array_equal(env.batch_is_collision_free(q), want)
    for i in range(0, 3000, 97):
        assert env.is_collision_free(q[i], None) == want[i]
        assert env.is_collision_free(q[i], None, collision_tolerance=0.0) == (free[i] or pen[i] <= 0.0)
    # per robot: exact relevant-pair check, or the scene total within the tolerance
    rfree = o.configs_free_for_robots(q, 0b0011).astype(bool)
    assert np.array_equal(env.batch_is_collision_free_for_robot(["r0", "r1"], q), rfree | (pen <= tol))
    # edges: every position (endpoints excluded) free under the rule
    rng = np.random.default_rng(5)
    a = q[:200]
    b = np.clip(a + rng.uniform(-0.3, 0.3, a.shape), sc.limits[0], sc.limits[1])
    got = env.batch_is_edge_collision_free(a, b, None, 0.05)
    for e in range(len(a)):
        n = max(2, int(np.abs(a[e] - b[e]).max() / 0.05) + 1)
        i = np.arange(1, n - 1, dtype=np.float64)
        pos = a[e][None, :] + ((b[e] - a[e]) / (n - 1))[None, :] * i[:, None]
        ok = o.configs_free(pos).astype(bool) | (o.total_penetration(pos) <= tol) if len(pos) else np.ones(0, bool)
        assert bool(got[e]) == bool(ok.all()), e
        if e % 20 == 0:
            assert env.is_edge_collision_free(a[e], b[e], None, 0.05) == bool(ok.all())


def test_exact_by_default(oracle):
    scenes = pkg("scenes")
    sc = scenes.make_arm_scene(2, n_boxes=20)
    env, o = _oracle_arm_env(oracle, sc, 10.0)
    env.tolerance_semantics = False
    q = scenes.uniform_configs(sc, 500, seed=4, dtype=np.float64)
    assert np.array_equal(env.batch_is_collision_free(q), o.configs_free(q).astype(bool))
