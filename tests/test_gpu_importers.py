"""GPU parity on imported planar MJCF scenes (planar-base robots without
links, a disc and a sphere-covered bar): configuration and edge verdicts
equal the oracle's on the same imported scene."""
import numpy as np
import pytest

from conftest import pkg
from test_importers import SCENE

pytestmark = pytest.mark.gpu


def test_imported_planar_scene_vs_oracle(gpu, oracle):
    imp, col, envm = pkg("importers"), pkg("collision"), pkg("env")
    sc = imp.load_mjcf_planar(SCENE)
    s = col.Gb300Scene(sc)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(3)
    q = rng.uniform(sc.limits[0], sc.limits[1], (20000, sc.q_dim))
    for dt in (np.float32, np.float64):
        qq = q.astype(dt)
        assert np.array_equal(s.is_collision_free_batch(qq).cpu().numpy(), o.configs_free(qq)), dt
    q1 = rng.uniform(sc.limits[0], sc.limits[1], (600, sc.q_dim))
    q2 = q1 + rng.uniform(-0.3, 0.3, q1.shape)
    got = s.is_edge_collision_free_batch(q1, q2, 0.01).cpu().numpy()
    assert np.array_equal(got, o.edges_free(q1, q2, 0.01))
    assert 0.05 < got.mean() < 0.95
    env = envm.Gb300ArmEnvironment(sc, collision_resolution=0.01, tune_samples=512)
    free = o.configs_free(q[:50]).astype(bool)
    assert [env.is_collision_free(x, None) for x in q[:50]] == free.tolist()
