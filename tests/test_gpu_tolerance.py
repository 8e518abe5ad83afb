"""The total penetration depth on the device (mrmg_arm_total_penetration)
equals the oracle's bit for bit (FP64 centres, overlaps summed as 2^-40 m
integers) on the four-arm table, the mobile manipulators, a per-mode scene
and imported arms with joint offsets; the env's rai tolerance rule on the
device gives the oracle composition's verdicts."""
import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def _scenes():
    scenes, imp = pkg("scenes"), pkg("importers")
    from test_importers import MJCF_ARMS

    return [("table", scenes.make_arm_scene(2, n_boxes=20)), ("dense", scenes.make_arm_scene(0)),
            ("mobile", scenes.make_mobile_scene(1, n_robots=3, n_boxes=40)),
            ("mjcf", imp.load_mjcf_arms(MJCF_ARMS))]


@pytest.mark.parametrize("which", [0, 1, 2, 3])
def test_total_penetration_bit_exact(gpu, oracle, which):
    col = pkg("collision")
    name, sc = _scenes()[which]
    s = col.Gb300Scene(sc)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(11)
    q = rng.uniform(sc.limits[0], sc.limits[1], (3000, sc.q_dim))
    for dt in (np.float64, np.float32):
        qq = q.astype(dt)
        got = s.total_penetration(qq)
        want = o.total_penetration(qq)
        assert np.array_equal(got, want), (name, dt, np.abs(got - want).max())
    free = o.configs_free(q).astype(bool)
    pen = s.total_penetration(q)
    assert (pen[free] == 0).all() and (pen[~free] > 0).all()


def test_total_penetration_per_mode(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    sc = scenes.make_arm_mode_scene(0)
    s = col.Gb300Scene(sc)
    q = scenes.uniform_configs(sc, 2000, seed=3, dtype=np.float64)
    for m in (0, 4, 11):
        s.set_mode(m)
        assert np.array_equal(s.total_penetration(q), oracle.OracleScene(sc.for_mode(m)).total_penetration(q)), m
    s.set_mode(-1)
    assert np.array_equal(s.total_penetration(q), oracle.OracleScene(sc).total_penetration(q))


def test_env_tolerance_rule_on_device(gpu, oracle):
    scenes, envm = pkg("scenes"), pkg("env")
    sc = scenes.make_arm_scene(2, n_boxes=20)
    o = oracle.OracleScene(sc)
    q = scenes.uniform_configs(sc, 3000, seed=4, dtype=np.float64)
    free = o.configs_free(q).astype(bool)
    pen = o.total_penetration(q)
    tol = float(np.percentile(pen[~free], 30))
    env = envm.Gb300ArmEnvironment(sc, collision_tolerance=tol, tune_samples=256, tolerance_semantics=True)
    want = free | (pen <= tol)
    assert np.array_equal(env.batch_is_collision_free(q), want)
    for i in range(0, 3000, 151):
        assert env.is_collision_free(q[i], None) == want[i]
    rfree = o.configs_free_for_robots(q, 0b0101).astype(bool)
    assert np.array_equal(env.batch_is_collision_free_for_robot(["r0", "r2"], q), rfree | (pen <= tol))
    rng = np.random.default_rng(5)
    a = q[:150]
    b = np.clip(a + rng.uniform(-0.3, 0.3, a.shape), sc.limits[0], sc.limits[1])
    got = env.batch_is_edge_collision_free(a, b, None, 0.05)
    for e in range(len(a)):
        n = max(2, int(np.abs(a[e] - b[e]).max() / 0.05) + 1)
        i = np.arange(1, n - 1, dtype=np.float64)
        pos = a[e][None, :] + ((b[e] - a[e]) / (n - 1))[None, :] * i[:, None]
        ok = (o.configs_free(pos).astype(bool) | (o.total_penetration(pos) <= tol)).all() if len(pos) else True
        assert bool(got[e]) == bool(ok), e
    exact = envm.Gb300ArmEnvironment(sc, collision_tolerance=tol, tune_samples=256)
    assert np.array_equal(exact.batch_is_collision_free(q), free)
