"""CPU checks of the FP64 penetration-cost oracle: its kinematics against the
C oracle's centres (the convention the collision path is pinned to), its
autograd gradient against central finite differences, and the workload
generator."""
import numpy as np
import pytest
import torch

from conftest import pkg


def _scene(kind):
    scenes = pkg("scenes")
    return scenes.make_arm_scene(0) if kind == "arm" else scenes.make_mobile_scene(1, n_robots=2, n_boxes=30)


@pytest.mark.parametrize("kind", ["arm", "mobile"])
def test_fk_matches_c_oracle(oracle, kind):
    import penetration_f64 as pen

    sc = _scene(kind)
    q = pkg("scenes").uniform_configs(sc, 16, seed=5, dtype=np.float64)
    orc = oracle.OracleScene(sc)
    want = np.stack([orc.sphere_centers(x) for x in q])
    got = pen.fk_centers(sc.arrays(), torch.from_numpy(q)).numpy()
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)


@pytest.mark.parametrize("kind", ["arm", "mobile"])
def test_autograd_matches_finite_differences(kind):
    import penetration_f64 as pen

    sc = _scene(kind)
    paths = pkg("scenes").make_path_workload(sc, seed=2, n_paths=2, n_waypoints=5).astype(np.float64)
    cost, g = pen.penetration_grad(sc.arrays(), paths)
    rng = np.random.default_rng(0)
    coords = [(int(rng.integers(2)), int(rng.integers(5)), int(rng.integers(sc.q_dim))) for _ in range(12)]
    fd = pen.finite_difference(sc.arrays(), paths, coords, h=1e-3)
    ag = np.array([g[c] for c in coords])
    assert np.linalg.norm(ag - fd) <= 1e-5 * np.linalg.norm(fd)


def test_cost_terms_by_hand():
    """Explicit loops over every sphere-box pair and every inter-robot sphere
    pair of three waypoints: the literal softplus(0.02 - d) / 0.02 terms plus
    the smoothness term give the oracle's cost."""
    import penetration_f64 as pen

    scenes = pkg("scenes")
    sc = scenes.make_arm_scene(0)
    paths = scenes.make_path_workload(sc, seed=3, n_paths=1, n_waypoints=3).astype(np.float64)
    a = sc.arrays()
    c = pen.fk_centers(a, torch.from_numpy(paths)).numpy()[0]
    r = a["sphere_radius"]
    lo, hi = a["box_lo"], a["box_hi"]
    ctr, half = 0.5 * (lo + hi), 0.5 * (hi - lo)
    total = 0.0
    for t in range(3):
        for s in range(len(r)):
            for b in range(len(lo)):
                q = np.abs(c[t, s] - ctr[b]) - half[b]
                sdf = np.linalg.norm(np.maximum(q, 0)) + min(q.max(), 0.0)
                total += np.log1p(np.exp(0.02 - (sdf - r[s]))) / 0.02
        for i in range(len(r)):
            for j in range(i + 1, len(r)):
                if a["sphere_robot"][i] != a["sphere_robot"][j]:
                    d = np.linalg.norm(c[t, i] - c[t, j]) - r[i] - r[j]
                    total += np.log1p(np.exp(0.02 - d)) / 0.02
    total += 0.1 * ((paths[0, 1:] - paths[0, :-1]) ** 2).sum()
    got = pen.penetration_cost(a, torch.from_numpy(paths)).item()
    assert abs(got - total) <= 1e-10 * abs(total)


def test_path_workload_shape_and_endpoints():
    scenes = pkg("scenes")
    sc = scenes.make_arm_scene(0)
    p = scenes.make_path_workload(sc, seed=0, n_paths=8, n_waypoints=33, noise=0.0)
    assert p.shape == (8, 33, 28) and p.dtype == np.float32
    # noise-free paths are straight lines
    s = np.linspace(0, 1, 33)
    line = p[:, :1].astype(np.float64) + s[None, :, None] * (p[:, -1:] - p[:, :1]).astype(np.float64)
    np.testing.assert_allclose(p, line, atol=1e-5)
