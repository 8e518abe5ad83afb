"""GPU parity of the path-penetration cost and its hand-written gradient:
against the float64 torch-autograd oracle and central finite differences
(h = 1e-3, float64).  Tolerances: cost relative error <= 1e-5 per path,
gradient relative error (2-norm over the compared entries) <= 1e-4."""
import numpy as np
import pytest
import torch

from conftest import pkg

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-5
GRAD_RTOL = 1e-4


def _setup(kind="arm", n_paths=3, n_waypoints=40, seed=1):
    scenes = pkg("scenes")
    sc = scenes.make_arm_scene(0) if kind == "arm" else scenes.make_mobile_scene(1, n_robots=2, n_boxes=30)
    paths = scenes.make_path_workload(sc, seed=seed, n_paths=n_paths, n_waypoints=n_waypoints)
    return sc, paths


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("kind", ["arm", "mobile"])
@pytest.mark.parametrize("T", [1, 31, 40, 64])
def test_cost_and_grad_vs_fp64_autograd(gpu, kind, T):
    import penetration_f64 as orc_pen

    pen, col = pkg("penetration"), pkg("collision")
    sc, paths = _setup(kind, n_waypoints=T)
    s = col.Gb300Scene(sc)
    out = pen.path_penetration(s, torch.from_numpy(paths).cuda(), cost=True, waypoint_cost=True, grad=True)
    c_ref, g_ref = orc_pen.penetration_grad(sc.arrays(), paths)
    wp_ref = orc_pen.penetration_cost(sc.arrays(), torch.from_numpy(paths.astype(np.float64)), per_waypoint=True)
    c = out["cost"].cpu().numpy()
    assert np.all(np.abs(c - c_ref) <= COST_RTOL * np.abs(c_ref))
    np.testing.assert_allclose(out["waypoint_cost"].cpu().numpy(), wp_ref.numpy(), rtol=1e-5)
    g = out["grad"].cpu().numpy()
    for p in range(len(paths)):
        assert _rel(g[p], g_ref[p]) <= GRAD_RTOL, p


def test_grad_vs_finite_differences(gpu):
    """The headline accuracy check: kernel gradient against central finite
    differences of the float64 cost at h = 1e-3."""
    import penetration_f64 as orc_pen

    pen, col = pkg("penetration"), pkg("collision")
    sc, paths = _setup("arm", n_paths=2, n_waypoints=36, seed=4)
    s = col.Gb300Scene(sc)
    g = pen.path_penetration(s, paths, cost=False, grad=True)["grad"].cpu().numpy()
    rng = np.random.default_rng(1)
    coords = [(int(rng.integers(2)), int(rng.integers(36)), int(rng.integers(28))) for _ in range(40)]
    fd = orc_pen.finite_difference(sc.arrays(), paths, coords, h=1e-3)
    got = np.array([g[c] for c in coords])
    assert _rel(got, fd) <= GRAD_RTOL


def test_autograd_function(gpu):
    """backward of PathPenetrationCost scales by the incoming gradient."""
    import penetration_f64 as orc_pen

    pen, col = pkg("penetration"), pkg("collision")
    sc, paths = _setup("arm", n_paths=3, n_waypoints=33)
    s = col.Gb300Scene(sc)
    w = torch.from_numpy(paths).cuda().requires_grad_(True)
    cost = pen.penetration_cost(w, s)
    assert cost.dtype == torch.float32 and cost.shape == (3,)
    weights = torch.tensor([1.0, -2.0, 0.5], device="cuda")
    (cost * weights).sum().backward()
    wd = torch.tensor(paths.astype(np.float64), requires_grad=True)
    (orc_pen.penetration_cost(sc.arrays(), wd) * torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64)).sum().backward()
    for p in range(3):
        assert _rel(w.grad[p].cpu().numpy(), wd.grad[p].numpy()) <= GRAD_RTOL
    # a single path (2-D input) gives a scalar
    c1 = pen.penetration_cost(torch.from_numpy(paths[0]).cuda(), s)
    assert c1.dim() == 0 and abs(c1.item() - cost[0].item()) <= 1e-6 * abs(cost[0].item())


def test_params_and_exact_scaling(gpu):
    """Other margin / scale / beta / smoothness values; the grad_cost factor
    is applied exactly (a power of two scales every gradient bit-exactly)."""
    import penetration_f64 as orc_pen

    pen, col = pkg("penetration"), pkg("collision")
    sc, paths = _setup("arm", n_paths=2, n_waypoints=20, seed=7)
    s = col.Gb300Scene(sc)
    prm = pen.PenetrationParams(margin=0.05, scale=0.1, beta=40.0, smooth_weight=0.5)
    out = pen.path_penetration(s, paths, prm, grad=True)
    c_ref, g_ref = orc_pen.penetration_grad(sc.arrays(), paths, margin=0.05, scale=0.1, beta=40.0, smooth_weight=0.5)
    assert np.all(np.abs(out["cost"].cpu().numpy() - c_ref) <= COST_RTOL * np.abs(c_ref))
    g = out["grad"].cpu().numpy()
    for p in range(2):
        assert _rel(g[p], g_ref[p]) <= GRAD_RTOL
    g4 = pen.path_penetration(s, paths, prm, cost=False, grad=True, grad_cost=[4.0, 4.0])["grad"].cpu().numpy()
    g1 = pen.path_penetration(s, paths, prm, cost=False, grad=True)["grad"].cpu().numpy()
    assert np.array_equal(g4, 4.0 * g1)


def test_deterministic_and_launch_shape_independent(gpu):
    pen, col = pkg("penetration"), pkg("collision")
    sc, paths = _setup("arm", n_paths=4, n_waypoints=70)
    s = col.Gb300Scene(sc)
    a = pen.path_penetration(s, paths)["cost"].cpu().numpy()
    b = pen.path_penetration(s, paths)["cost"].cpu().numpy()
    assert np.array_equal(a, b)
    g0 = pen.path_penetration(s, paths, cost=False, grad=True)["grad"].cpu().numpy()
    g1 = pen.path_penetration(s, paths, cost=True, grad=True)["grad"].cpu().numpy()
    assert np.array_equal(g0, g1)          # deterministic, and the same with the cost fused
    for warps in (4, 8, 12):
        c = pen.path_penetration(s, paths, warps_per_cta=warps)["cost"].cpu().numpy()
        np.testing.assert_allclose(c, a, rtol=1e-6)


def test_full_size_batch_properties(gpu):
    """512 paths x 256 waypoints x 28 joints: finite, per-waypoint costs add up
    to the path cost, two sampled paths match the float64 oracle."""
    import penetration_f64 as orc_pen

    pen, col, scenes = pkg("penetration"), pkg("collision"), pkg("scenes")
    sc = scenes.make_arm_scene(0)
    s = col.Gb300Scene(sc)
    paths = scenes.make_path_workload(sc, seed=0, is_free=lambda q: s.is_collision_free_batch(q).cpu().numpy())
    assert paths.shape == (512, 256, 28)
    out = pen.path_penetration(s, paths, cost=True, waypoint_cost=True, grad=True)
    c = out["cost"].cpu().numpy()
    g = out["grad"]
    assert np.all(np.isfinite(c)) and bool(torch.isfinite(g).all())
    wsum = out["waypoint_cost"].double().sum(1).cpu().numpy()
    np.testing.assert_allclose(wsum, c, rtol=1e-6)
    for p in (0, 311):
        c_ref, g_ref = orc_pen.penetration_grad(sc.arrays(), paths[p:p + 1])
        assert abs(c[p] - c_ref[0]) <= COST_RTOL * abs(c_ref[0])
        assert _rel(g[p].cpu().numpy(), g_ref[0]) <= GRAD_RTOL


def test_repair_lowers_cost(gpu):
    pen, col, scenes = pkg("penetration"), pkg("collision"), pkg("scenes")
    sc = scenes.make_arm_scene(0)
    s = col.Gb300Scene(sc)
    paths = scenes.make_path_workload(sc, seed=3, n_paths=16, n_waypoints=64,
                                      is_free=lambda q: s.is_collision_free_batch(q).cpu().numpy())
    prm = pen.PenetrationParams(beta=50.0)
    r = pen.repair_paths(s, paths, prm, iters=20, step=1e-3, limits=sc.limits)
    assert bool((r["cost_after"] <= r["cost_before"]).all())
    np.testing.assert_array_equal(r["paths"][:, 0].cpu().numpy(), paths[:, 0])
    np.testing.assert_array_equal(r["paths"][:, -1].cpu().numpy(), paths[:, -1])
    assert r["collision_free"].shape == (16,)


def test_errors(gpu):
    pen, col, scenes = pkg("penetration"), pkg("collision"), pkg("scenes")
    s = col.Gb300Scene(scenes.make_arm_scene(0))
    with pytest.raises(ValueError):
        pen.path_penetration(s, np.zeros((2, 5, 27), np.float32))
    with pytest.raises(ValueError):
        pen.path_penetration(s, np.zeros((2, 5, 28), np.float32), pen.PenetrationParams(scale=0.0))
    ab = col.Gb300Scene(scenes.make_disc_scene(0))
    with pytest.raises(TypeError):
        pen.path_penetration(ab, np.zeros((1, 3, 4), np.float32))
    # the 304-sphere mobile scene: cost and (grouped) gradient both run
    big = col.Gb300Scene(scenes.make_mobile_scene(0))
    out = pen.path_penetration(big, np.zeros((1, 3, 72), np.float32), grad=True)
    assert bool(torch.isfinite(out["cost"]).all()) and bool(torch.isfinite(out["grad"]).all())


def test_gradient_of_the_304_sphere_mobile_scene(gpu):
    """Eight mobile manipulators (304 spheres): the single-launch gradient
    kernel would need more shared memory than a CTA has, so the gradient runs
    per group of robots; cost and gradient match the float64 autograd
    oracle, cost alone and cost with gradient agree."""
    import penetration_f64 as orc_pen

    pen, col, scenes = pkg("penetration"), pkg("collision"), pkg("scenes")
    sc = scenes.make_mobile_scene(0)
    s = col.Gb300Scene(sc)
    info = pen.penetration_info(s)
    assert info["spheres"] == 304
    smem_max = getattr(torch.cuda.get_device_properties(0), "shared_memory_per_block_optin", 232448)
    assert info["smem_grad"] > smem_max
    paths = scenes.make_path_workload(sc, seed=4, n_paths=3, n_waypoints=40)
    out = pen.path_penetration(s, torch.from_numpy(paths).cuda(), cost=True, waypoint_cost=True, grad=True)
    c_ref, g_ref = orc_pen.penetration_grad(sc.arrays(), paths)
    c = out["cost"].cpu().numpy()
    assert np.all(np.abs(c - c_ref) <= COST_RTOL * np.abs(c_ref))
    for p in range(3):
        assert _rel(out["grad"][p].cpu().numpy(), g_ref[p]) <= GRAD_RTOL, p
    c_only = pen.path_penetration(s, torch.from_numpy(paths).cuda(), cost=True)["cost"].cpu().numpy()
    assert np.array_equal(c_only, c)
    go = torch.tensor([1.0, -2.0, 0.5])
    g2 = pen.path_penetration(s, torch.from_numpy(paths).cuda(), cost=False, grad=True, grad_cost=go)["grad"]
    for p in range(3):
        np.testing.assert_allclose(g2[p].cpu().numpy(), float(go[p]) * out["grad"][p].cpu().numpy(), rtol=1e-6, atol=1e-9)
