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


def test_imported_arms_with_joint_offsets_vs_oracle(gpu, oracle):
    """Two six-joint MJCF arms in DH form with joint offsets: the FP64 sphere
    centres are the oracle's bit for bit, the FP32 ones within a tenth of the
    band; configuration and edge verdicts equal the oracle's; the penetration
    cost and gradient match the float64 autograd restatement."""
    import sys

    import torch

    from test_importers import MJCF_ARMS

    imp, col = pkg("importers"), pkg("collision")
    sc = imp.load_mjcf_arms(MJCF_ARMS)
    s = col.Gb300Scene(sc)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(6)
    q = rng.uniform(sc.limits[0], sc.limits[1], (20000, sc.q_dim))
    c32, c64 = s.sphere_centers(q[:500])
    c32, c64 = c32.cpu().numpy().astype(np.float64), c64.cpu().numpy()
    for i in range(0, 500, 37):
        assert np.array_equal(c64[i], o.sphere_centers(q[i])), i
    assert np.abs(c32 - c64).max() * 10 <= s.info()["band"]
    for dt in (np.float32, np.float64):
        qq = q.astype(dt)
        assert np.array_equal(s.is_collision_free_batch(qq).cpu().numpy(), o.configs_free(qq)), dt
    free = q[o.configs_free(q).astype(bool)][:800]
    assert len(free) >= 200
    q2 = free + rng.uniform(-0.8, 0.8, free.shape)
    ref = o.edges_free(free, q2, 0.02)
    assert np.array_equal(s.is_edge_collision_free_batch(free, q2, 0.02).cpu().numpy(), ref)
    assert np.array_equal(s.is_edge_collision_free_host(free[:100], q2[:100], 0.02), ref[:100])
    assert ref.mean() > 0.1 and (ref == 0).sum() >= 10
    sys.path.insert(0, str(pkg("_lib").HERE.parent / "oracle"))
    import penetration_f64 as orc_pen

    pen = pkg("penetration")
    paths = (free[:4, None, :] + (q2[:4, None, :] - free[:4, None, :]) * np.linspace(0, 1, 40)[None, :, None])
    paths = np.ascontiguousarray(paths.astype(np.float32))
    res = pen.path_penetration(s, torch.from_numpy(paths).cuda(), cost=True, grad=True)
    c_ref, g_ref = orc_pen.penetration_grad(sc.arrays(), paths)
    assert np.all(np.abs(res["cost"].cpu().numpy() - c_ref) <= 1e-5 * np.abs(c_ref) + 1e-9)
    g = res["grad"].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)


def test_imported_urdf_planar_scene_vs_oracle(gpu, oracle):
    from test_importers import URDF_SCENE

    imp, col = pkg("importers"), pkg("collision")
    sc = imp.load_urdf_planar(URDF_SCENE)
    s = col.Gb300Scene(sc)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(9)
    q = rng.uniform(sc.limits[0], sc.limits[1], (8000, sc.q_dim))
    assert np.array_equal(s.is_collision_free_batch(q).cpu().numpy(), o.configs_free(q))
    q2 = q + rng.uniform(-0.3, 0.3, q.shape)
    assert np.array_equal(s.is_edge_collision_free_batch(q, q2, 0.01).cpu().numpy(), o.edges_free(q, q2, 0.01))
