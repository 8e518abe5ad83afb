"""Host-side logic that needs no GPU: the edge step-count formula of the
serving batcher, the workload generators, the penetration parameter record
and the C library's export of the new entry points."""
import math

import numpy as np
import pytest

from conftest import pkg


def test_edge_steps_matches_reference_formula():
    """N = max(2, int(max|q2 - q1| / res) + 1) in float64
    (abstract_env.py:321-329), row by row."""
    import importlib

    scenes = pkg("scenes")
    # serving.py imports torch at module level; the formula itself is numpy
    srv = importlib.import_module("multirobot-pathplanning-benchmark_gb300.serving")
    sc = scenes.make_arm_scene(0)
    rng = np.random.default_rng(0)
    q1 = rng.uniform(-3, 3, (500, 28)).astype(np.float32)
    q2 = (q1 + rng.normal(0, 0.4, q1.shape)).astype(np.float32)
    q2[:5] = q1[:5]                      # zero-length edges: N = 2
    for res in (0.05, 0.01, 0.3):
        want = [max(2, int(max(abs(float(b) - float(a)) for a, b in zip(x, y)) / res) + 1) for x, y in zip(q1, q2)]
        assert np.array_equal(srv.edge_steps(q1, q2, res), np.array(want))
    N = scenes.lognormal_steps(2000, 3)
    a, b = scenes.edges_with_steps(sc, N, 0.05, 4)
    assert np.array_equal(srv.edge_steps(a, b, 0.05), N)


def test_serving_requests_shapes():
    scenes = pkg("scenes")
    sc = scenes.make_mobile_scene(0)
    reqs = scenes.make_serving_requests(sc, seed=1, n_instances=5, configs=(3, 9), edges=(0, 4), steps=(5, 800))
    assert len(reqs) == 5
    for r in reqs:
        assert r["configs"].shape[1] == 72 and 3 <= len(r["configs"]) <= 9
        assert r["q1"].shape == r["q2"].shape and len(r["N"]) == len(r["q1"]) <= 4
        assert r["configs"].dtype == np.float32 and r["N"].dtype == np.int64
        if len(r["N"]):
            assert r["N"].min() >= 5 and r["N"].max() <= 800
        lo, hi = sc.limits
        assert np.all(r["configs"] >= lo.astype(np.float32) - 1e-6) and np.all(r["configs"] <= hi.astype(np.float32) + 1e-6)


def test_penetration_params_record():
    pen = pkg("penetration")
    p = pen.PenetrationParams()
    assert list(p.array()) == [0.02, 0.02, 1.0, 0.1]
    q = pen.PenetrationParams(margin=0.05, beta=40.0)
    assert q.array()[0] == 0.05 and q.array()[2] == 40.0
    with pytest.raises(Exception):
        p.margin = 1.0                   # frozen


def test_new_entry_points_exported(cuda_lib):
    for name in ("mrmg_path_penetration", "mrmg_penetration_info", "mrmg_microbench_fma"):
        assert hasattr(cuda_lib, name)


def test_radius_fp32_band():
    """The FP32 pre-test of radius queries assumes the FP32 sum of squared
    coordinate differences lies within 2.4e-6 (|q| + |x|)^2 of the exact
    squared distance (the kernel decides outside 7.7e-6 of that).  Checked
    with numpy FP32 arithmetic (separate multiply and add: more rounding than
    the kernel's fused chain) on 28-D inputs from 1e-3 to 1e4 in scale,
    including near-duplicate pairs and mixed signs."""
    rng = np.random.default_rng(0)
    worst = 0.0
    for scale in (1e-3, 1.0, 3.14, 1e2, 1e4):
        q = rng.uniform(-scale, scale, (4000, 28))
        x = np.where(rng.random((4000, 1)) < 0.3, q + rng.normal(0, 1e-5 * scale, q.shape),
                     rng.uniform(-scale, scale, q.shape))
        qf, xf = q.astype(np.float32), x.astype(np.float32)
        m = np.zeros(len(q), dtype=np.float32)
        for k in range(28):
            d = qf[:, k] - xf[:, k]
            m = (m + d * d).astype(np.float32)
        exact = np.array([float(sum((a - b) ** 2 for a, b in zip(map(np.longdouble, qi), map(np.longdouble, xi))))
                          for qi, xi in zip(q[:400], x[:400])])
        e = np.linalg.norm(q[:400], axis=1) + np.linalg.norm(x[:400], axis=1)
        ratio = np.abs(m[:400].astype(np.float64) - exact) / (e * e)
        worst = max(worst, float(ratio.max()))
    assert worst <= 2.4e-6, worst
