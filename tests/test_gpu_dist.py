"""GPU parity for distances and costs: bit-identical float64 against the
reference's own outputs (golden vectors) and the oracle."""
import numpy as np
import pytest

from conftest import golden, pkg

pytestmark = pytest.mark.gpu

TAGS = ["2_2", "7_7", "3_3_3", "2_5", "14", "7x4"]


@pytest.mark.parametrize("tag", TAGS)
def test_batch_config_dist_golden(gpu, tag):
    cfg = pkg("configuration")
    g = golden("dist_cost.npz")
    pt, pts, sl = g[f"{tag}_pt"], g[f"{tag}_pts"], g[f"{tag}_slices"]
    q = cfg.Gb300Configuration(pt, [tuple(s) for s in sl])
    for metric in ["euclidean", "sum_euclidean", "max_euclidean", "max"]:
        got = cfg.batch_config_dist(q, pts, metric)             # dispatches on type(pt)._batch_dist
        assert np.array_equal(got, g[f"{tag}_dist_{metric}"]), metric
        assert cfg.config_dist(q, q.from_flat(pts[3]), metric) == g[f"{tag}_dist_{metric}"][3]


@pytest.mark.parametrize("tag", TAGS)
def test_batch_config_cost_golden(gpu, tag):
    cfg = pkg("configuration")
    g = golden("dist_cost.npz")
    pt, pts, sl = g[f"{tag}_pt"], g[f"{tag}_pts"], g[f"{tag}_slices"]
    q = cfg.Gb300Configuration(pt, [tuple(s) for s in sl])
    for metric in ["euclidean", "max"]:
        for red in ["max", "sum"]:
            assert np.array_equal(cfg.batch_config_cost(q, pts, metric, red), g[f"{tag}_cost_{metric}_{red}"])
            assert np.array_equal(cfg.batch_config_cost(pts[:300], pts[300:], metric, red, tmp_agent_slice=sl),
                                  g[f"{tag}_rowcost_{metric}_{red}"])
            assert np.array_equal(cfg.batch_config_cost(list(pts[:100]), None, metric, red, tmp_agent_slice=sl),
                                  g[f"{tag}_pathcost_{metric}_{red}"])
            # ndarray x ndarray broadcasts as `starts - batch_other` does (one row against many,
            # either way round: |d| and d*d do not see the sign)
            want = g[f"{tag}_cost_{metric}_{red}"]
            assert np.array_equal(cfg.batch_config_cost(pt, pts, metric, red, tmp_agent_slice=sl), want)
            assert np.array_equal(cfg.batch_config_cost(pts, pt[None], metric, red, tmp_agent_slice=sl), want)
    with pytest.raises(ValueError):      # a 1-D difference: the reference's diff[:, s:e] fails too
        cfg.batch_config_cost(pt, pts[0], "max", "max", tmp_agent_slice=sl)
    with pytest.raises(ValueError):
        cfg.batch_config_cost(pts[:3], pts[:2], "max", "max", tmp_agent_slice=sl)
    # path_cost (problems/util.py:51-67): per-edge costs, then np.sum
    costs = g[f"{tag}_pathcost_euclidean_max"]
    assert cfg.path_cost(list(pts[:100]), lambda a, b, tmp_agent_slice: cfg.batch_config_cost(
        a, b, "euclidean", "max", tmp_agent_slice=tmp_agent_slice), agent_slices=sl) == np.sum(costs)


def test_distance_matrix_disc_workload(gpu, oracle):
    """config[0]'s 1,000 x 10,000 euclidean distance matrix, bit-identical."""
    cfg, scenes = pkg("configuration"), pkg("scenes")
    w = scenes.make_disc_workload(0)
    got = cfg.config_dist_matrix(w["queries"], w["configs"], [[0, 2], [2, 4]], "euclidean").cpu().numpy()
    ref = oracle.dist_matrix(w["queries"], w["configs"], [[0, 2], [2, 4]], "euclidean")
    assert np.array_equal(got, ref)


def test_env_cost_methods(gpu):
    """config_cost / batch_config_cost of the env use cost_metric/cost_reduction
    exactly as abstract_env.py:238-253."""
    cfg, scenes, envm = pkg("configuration"), pkg("scenes"), pkg("env")
    env = envm.Gb300AbstractEnvironment(scenes.make_disc_scene(0))
    rng = np.random.default_rng(3)
    a = env.start_pos.from_flat(rng.uniform(-1, 1, 4))
    b = rng.uniform(-1, 1, (50, 4))
    got = env.batch_config_cost(a, b)
    want = cfg.batch_config_cost(a, b, "euclidean", "max")
    assert np.array_equal(got, want)
    assert env.config_cost(a, a.from_flat(b[0])) == want[0]
