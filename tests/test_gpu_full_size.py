"""Parity at the full sizes of the benchmark workloads, against the oracle,
on every item (no sampling):

* four 7-DoF arms among 50 boxes: all 100,000 edges of the benchmark step
  (lognormal step counts, median 40, clipped 5..500, resolution 0.05 rad) and
  1,000,000 configurations uniform in the joint limits;
* the same arms among 5 boxes with short edges between free configurations
  (100,000 edges, most of them free: the interpolation path, not early
  exits);
* per-mode k-NN: 200,000 nodes in 16 Zipf-sized modes, 4,096 queries, k = 10,
  euclidean and max over agents: indices and FP64 distances;
* serving: two full steps of 64 mobile-manipulator instances (100-20,000
  configurations and 10-5,000 edges each), every instance.
"""
import sys

import numpy as np
import pytest

from conftest import ROOT, pkg

pytestmark = pytest.mark.gpu


def _bench():
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    import bench

    return bench


def test_full_edge_step_and_million_configs(gpu, oracle):
    bench, scenes, envm = _bench(), pkg("scenes"), pkg("env")
    scene, q1, q2, N = bench.workload(0)
    assert len(q1) == 100_000
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=bench.RESOLUTION)
    o = oracle.OracleScene(scene)
    got = env.batch_is_edge_collision_free(q1, q2).astype(np.uint8)
    ref = o.edges_free(q1, q2, bench.RESOLUTION)
    assert np.array_equal(got, ref), int((got != ref).sum())
    # the step counts the workload was built with are the ones the formula gives
    assert np.array_equal(np.maximum(2, (np.abs(q1.astype(np.float64) - q2).max(1) / bench.RESOLUTION)
                                     .astype(np.int64) + 1), N)
    q = scenes.uniform_configs(scene, 1_000_000, seed=77, dtype=np.float32)
    got = env.batch_is_collision_free(q).astype(np.uint8)
    ref = o.configs_free(q)
    assert np.array_equal(got, ref), int((got != ref).sum())
    assert 0 < ref.sum() < len(ref)


def test_full_size_sparse_scene_edges(gpu, oracle):
    """100,000 edges of up to 0.3 rad per joint between free configurations of
    the four arms among 5 boxes, resolution 0.02: most edges are free, so
    every interpolated position is evaluated."""
    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_scene(1, n_boxes=5)
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=0.02, tune_samples=1024)
    o = oracle.OracleScene(scene)
    q = scenes.uniform_configs(scene, 600_000, seed=5, dtype=np.float64)
    free = q[env.batch_is_collision_free(q)]
    assert len(free) >= 100_000
    a = free[:100_000]
    rng = np.random.default_rng(6)
    b = a + rng.uniform(-0.3, 0.3, a.shape)
    for dt in (np.float64, np.float32):
        got = env.batch_is_edge_collision_free(a.astype(dt), b.astype(dt)).astype(np.uint8)
        ref = o.edges_free(a.astype(dt), b.astype(dt), 0.02)
        assert np.array_equal(got, ref), (dt, int((got != ref).sum()))
        assert ref.mean() > 0.2, ref.mean()


@pytest.mark.parametrize("metric", ["euclidean", "max_euclidean"])
def test_full_size_knn(gpu, oracle, metric):
    knn, scenes = pkg("knn"), pkg("scenes")
    w = scenes.make_knn_workload(seed=0)
    assert len(w["nodes"]) == 200_000 and len(w["queries"]) == 4096 and len(w["mode_offsets"]) == 17
    store = knn.NodeStore(w["nodes"], w["mode_offsets"], w["slices"], metric)
    idx, dist = store.knn(w["queries"], w["q_mode"], w["k"])
    oi, od = oracle.knn(w["queries"], w["q_mode"], w["nodes"], w["mode_offsets"], w["slices"], metric, w["k"])
    assert np.array_equal(idx.cpu().numpy(), oi)
    assert np.array_equal(dist.cpu().numpy(), od)
    assert store.last_stats["tensor_core"]
    store.close()


def test_full_size_serving_steps(gpu, oracle):
    scenes, envm, srv = pkg("scenes"), pkg("env"), pkg("serving")
    sc = scenes.make_mobile_scene(0)
    env = envm.Gb300ArmEnvironment(sc)
    o = oracle.OracleScene(sc)
    b = srv.ServingBatcher(env._gb300)
    for seed in (100, 101):
        reqs = scenes.make_serving_requests(sc, seed=seed)
        assert len(reqs) == 64
        res = b.step(reqs)
        for r, cf, ef in zip(reqs, res.config_free, res.edge_free):
            assert np.array_equal(cf, o.configs_free(r["configs"]))
            assert np.array_equal(ef, o.edges_free(r["q1"], r["q2"], 0.05, N=r["N"]))
