"""GPU parity of the host-pointer calls (mrmg_is_collision_free_host,
mrmg_is_edge_collision_free_host) that the env's single-query methods use:
the single-launch path for small arm batches (every configuration or edge
position a warp's work item, pending configurations decided in FP64 at once)
and the staged batched path for everything else.  Verdicts must equal the
oracle's bit for bit, and the status codes those of the batched calls."""
import numpy as np
import pytest

from conftest import golden, pkg

pytestmark = pytest.mark.gpu


def _free_configs(o, scene, n, seed):
    q = pkg("scenes").uniform_configs(scene, 40 * n, seed=seed, dtype=np.float64)
    return q[o.configs_free(q).astype(bool)][:n]


@pytest.mark.parametrize("kind", ["arm", "sparse", "mobile"])
def test_host_configs_vs_oracle(gpu, oracle, kind):
    scenes, col = pkg("scenes"), pkg("collision")
    scene = {"arm": lambda: scenes.make_arm_scene(0), "sparse": lambda: scenes.make_arm_scene(1, n_boxes=5),
             "mobile": lambda: scenes.make_mobile_scene(0)}[kind]()
    sc = col.Gb300Scene(scene)
    o = oracle.OracleScene(scene)
    for n, dt in ((1, np.float64), (37, np.float32), (4096, np.float64), (6000, np.float32)):
        q = scenes.uniform_configs(scene, n, seed=n, dtype=dt)
        assert np.array_equal(sc.is_collision_free_host(q), o.configs_free(q)), (n, dt)
    # single calls, free and colliding, through the env's method
    env = pkg("env").Gb300ArmEnvironment(scene, tune_samples=256)
    q = scenes.uniform_configs(scene, 200, seed=3, dtype=np.float64)
    q = np.concatenate([q, _free_configs(o, scene, 50, 4)])
    ref = o.configs_free(q)
    got = np.array([env.is_collision_free(x, None) for x in q], dtype=np.uint8)
    assert np.array_equal(got, ref)
    assert ref.sum() < len(ref)
    if kind != "mobile":   # uniform configurations of the eight mobile robots all collide
        assert ref.sum() > 0


def test_host_configs_near_contact_and_bad_inputs(gpu, oracle):
    """Configurations the FP32 pass leaves pending are decided in FP64 inside
    the single launch: a box face at r + eps from a sphere centre, eps down
    to a few ulps; NaN, inf and huge joint values as the batched call."""
    import copy

    scenes, col = pkg("scenes"), pkg("collision")
    base = scenes.make_arm_scene(2, n_boxes=0)
    o0 = oracle.OracleScene(base)
    qs = _free_configs(o0, base, 18, 11)
    rng = np.random.default_rng(5)
    eps_set = [-1e-7, -1e-10, -1e-13, 0.0, 1e-13, 1e-10, 1e-7]
    pending = 0
    for i, q in enumerate(qs):
        c = o0.sphere_centers(q)
        s = rng.integers(len(c))
        r = float(base.sphere_radius[s])
        k = rng.integers(3)
        lo, hi = c[s] - 0.05, c[s] + 0.05
        lo[k] = c[s][k] + r + eps_set[i % len(eps_set)]
        hi[k] = lo[k] + 0.1
        scene = copy.deepcopy(base)
        scene.box_lo = lo.reshape(1, 3)
        scene.box_hi = hi.reshape(1, 3)
        sc = col.Gb300Scene(scene)
        o = oracle.OracleScene(scene)
        assert sc.config_free1(q) == bool(o.config_free(q)), i
        pending += sc.last_call_stats()["rechecked_fp64"]
    assert pending > 0
    scene = scenes.make_arm_scene(1, n_boxes=5)
    sc, o = col.Gb300Scene(scene), oracle.OracleScene(scene)
    q = scenes.uniform_configs(scene, 64, seed=1, dtype=np.float64)
    q[0, 3], q[1, 5], q[2, 0], q[3, 27] = np.nan, 1e7, 3e9, np.inf
    assert np.array_equal(sc.is_collision_free_host(q), o.configs_free(q))


def test_host_edges_vs_oracle(gpu, oracle):
    """Dense and sparse arm scenes: one edge at a time (the planners' calls),
    batches of up to 256 edges (single launch) and larger ones (staged
    batched path), with N_start / N_max / include_endpoints / given N."""
    scenes, col, envm = pkg("scenes"), pkg("collision"), pkg("env")
    scene = scenes.make_arm_scene(0)
    sc, o = col.Gb300Scene(scene), oracle.OracleScene(scene)
    w = scenes.make_arm_workload(scene, seed=4, n_configs=10, n_edges=1200)
    ref = o.edges_free(w["q1"], w["q2"], w["resolution"])
    for n in (1, 7, 256, 257, 1200):
        got = sc.is_edge_collision_free_host(w["q1"][:n], w["q2"][:n], w["resolution"])
        assert np.array_equal(got, ref[:n]), n
    scene = scenes.make_arm_scene(1, n_boxes=5)
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=0.02, tune_samples=256)
    sc, o = env._gb300, oracle.OracleScene(scene)
    a = _free_configs(o, scene, 300, 3)
    b = a + np.random.default_rng(0).uniform(-0.15, 0.15, a.shape)
    res = 0.02
    N = np.maximum(2, (np.abs(a - b).max(1) / res).astype(np.int64) + 1)
    for kw in [dict(), dict(include_endpoints=True), dict(N_start=2, N_max=9), dict(N_start=4), dict(N=N)]:
        keep = N >= kw.get("N_start", 0)
        ref = o.edges_free(a[keep], b[keep], res, **kw) if "N" not in kw else o.edges_free(a, b, res, N=N)
        if "N" in kw:
            got = sc.is_edge_collision_free_host(a, b, res, N=N)
        else:
            got = sc.is_edge_collision_free_host(a[keep], b[keep], res, **kw)
        assert np.array_equal(got, ref), kw
        assert ref.mean() > 0.2
        # the same edges one call at a time through the env's method
        idx = np.nonzero(keep)[0][:60]
        one = [env.is_edge_collision_free(a[i], b[i], None, res, None, kw.get("include_endpoints", False),
                                          kw.get("N_start", 0), kw.get("N_max"), int(N[i]) if "N" in kw else None)
               for i in idx]
        sub = ref[:60] if "N" not in kw else ref[idx]
        assert np.array_equal(np.array(one, dtype=np.uint8), sub), kw


def test_host_edges_errors_match_batched_call(gpu):
    scenes, col = pkg("scenes"), pkg("collision")
    sc = col.Gb300Scene(scenes.make_arm_scene(1, n_boxes=5))
    q = scenes.uniform_configs(sc.scene, 4, seed=2, dtype=np.float64)
    with pytest.raises(AssertionError):
        sc.is_edge_collision_free_host(q[:2], q[2:], 0.05, N=[3, 3], N_start=5)
    bad = q.copy()
    bad[0, 0] = np.nan
    with pytest.raises(ValueError):
        sc.is_edge_collision_free_host(bad[:2], q[2:], 0.05)
    with pytest.raises(ValueError):
        sc.is_edge_collision_free_host(q[:2], q[2:], 0.0)


def test_host_calls_disc_scene_golden(gpu):
    """The abstract scenes take the staged batched path: the reference's own
    verdicts (abstract_disc.npz), one call at a time and batched."""
    g = golden("abstract_disc.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["centers"],
        box_bounds=2.0 * g["half"], sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)
    env = pkg("env").Gb300AbstractEnvironment(scene)
    sc = env._gb300
    assert np.array_equal(sc.is_collision_free_host(g["configs"]), g["config_free"])
    got = [env.is_collision_free(q, None) for q in g["configs"][:300]]
    assert np.array_equal(np.array(got, dtype=np.uint8), g["config_free"][:300])
    import json

    for vi, v in enumerate(json.loads(str(g["variants"]))):
        v = dict(v)
        res = v.pop("resolution")
        ok = g["edge_free"][vi] != 255   # 255: the reference asserted (N_start > N)
        got = sc.is_edge_collision_free_host(g["q1"][ok], g["q2"][ok], res, **v)
        assert np.array_equal(got, g["edge_free"][vi][ok]), v
    got = [env.is_edge_collision_free(a, b, None, 0.01) for a, b in zip(g["q1"][:200], g["q2"][:200])]
    assert np.array_equal(np.array(got, dtype=np.uint8), g["edge_free"][0][:200])


def test_host_robot_mask_and_modes(gpu, oracle):
    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_scene(0)
    env = envm.Gb300ArmEnvironment(scene, tune_samples=256)
    o = oracle.OracleScene(scene)
    q = scenes.uniform_configs(scene, 300, seed=17, dtype=np.float64)
    for m in (1, 0b10, 0b101, 0b1111):
        names = [env.robots[r] for r in range(scene.n_robots) if (m >> r) & 1]
        want = o.configs_free_for_robots(q, m)
        got = np.array([env.is_collision_free_for_robot(names, x) for x in q[:120]], dtype=np.uint8)
        assert np.array_equal(got, want[:120]), m
        assert np.array_equal(env._gb300.is_collision_free_host(q, robot_mask=m), want), m


def test_abstract_edges_both_kernels_vs_oracle(gpu, oracle):
    """Two-disc scene: batches up to 65,536 edges run the flat single-launch
    kernel (positions side by side, pending ones decided in FP64 at once),
    larger ones the warp-per-edge kernel with its FP64 pass; device and host
    inputs, FP64 and FP32 endpoints, against the oracle."""
    import torch

    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_disc_scene(0)
    sc, o = col.Gb300Scene(scene), oracle.OracleScene(scene)
    rng = np.random.default_rng(12)
    for n in (1, 999, 65536, 70000):
        q1 = rng.uniform(-1, 1, (n, 4))
        q2 = q1 + rng.uniform(-0.3, 0.3, (n, 4))
        for dt in (np.float64, np.float32):
            a, b = q1.astype(dt), q2.astype(dt)
            ref = o.edges_free(a, b, 0.01)
            assert np.array_equal(sc.is_edge_collision_free_host(a, b, 0.01), ref), (n, dt)
            got = sc.is_edge_collision_free_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), 0.01)
            assert np.array_equal(got.cpu().numpy(), ref), (n, dt)
        assert 0 < ref.sum() < n or n < 10
    # near-tangent positions: pending classifications decided in FP64
    g = golden("abstract_disc.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["centers"],
        box_bounds=2.0 * g["half"], sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)
    sc = col.Gb300Scene(scene)
    assert np.array_equal(sc.is_collision_free_host(g["configs"]), g["config_free"])
    assert sc.last_call_stats() is not None


def test_abstract_host_edge_errors(gpu):
    """Errors found by the flat kernel on the mapped buffer come back as the
    batched call's status: N_start > N -> AssertionError, a NaN edge length
    -> ValueError; the scene stays usable."""
    scenes, col = pkg("scenes"), pkg("collision")
    sc = col.Gb300Scene(scenes.make_disc_scene(0))
    rng = np.random.default_rng(3)
    q1, q2 = rng.uniform(-1, 1, (50, 4)), rng.uniform(-1, 1, (50, 4))
    with pytest.raises(AssertionError):
        sc.is_edge_collision_free_host(q1, q2, 0.01, N=np.full(50, 3), N_start=5)
    bad = q1.copy()
    bad[7, 0] = np.nan
    with pytest.raises(ValueError):
        sc.is_edge_collision_free_host(bad, q2, 0.01)
    ok = sc.is_edge_collision_free_host(q1, q2, 0.01)
    assert np.array_equal(ok, sc.is_edge_collision_free_batch(q1, q2, 0.01).cpu().numpy())


def test_host_calls_staged_inputs_match(gpu, oracle, monkeypatch):
    """The same host-pointer calls with the inputs staged in the mapped
    buffer (MRMG_STAGE_HOST_INPUTS=1; the path of devices that cannot read
    pageable host memory): identical verdicts, arm and abstract scenes."""
    monkeypatch.setenv("MRMG_STAGE_HOST_INPUTS", "1")
    scenes, col = pkg("scenes"), pkg("collision")
    arm = scenes.make_arm_scene(0)
    sc, o = col.Gb300Scene(arm), oracle.OracleScene(arm)
    w = scenes.make_arm_workload(arm, seed=8, n_configs=3000, n_edges=400)
    assert np.array_equal(sc.is_collision_free_host(w["configs"]), o.configs_free(w["configs"]))
    ref = o.edges_free(w["q1"], w["q2"], w["resolution"])
    assert np.array_equal(sc.is_edge_collision_free_host(w["q1"], w["q2"], w["resolution"]), ref)
    assert np.array_equal(sc.is_edge_collision_free_host(w["q1"][:50], w["q2"][:50], w["resolution"]), ref[:50])
    disc = scenes.make_disc_scene(0)
    sd, od = col.Gb300Scene(disc), oracle.OracleScene(disc)
    rng = np.random.default_rng(4)
    q1, q2 = rng.uniform(-1, 1, (700, 4)), rng.uniform(-1, 1, (700, 4))
    assert np.array_equal(sd.is_edge_collision_free_host(q1, q2, 0.01), od.edges_free(q1, q2, 0.01))
    assert np.array_equal(sd.is_collision_free_host(q1), od.configs_free(q1))
