"""GPU parity for sphere-arm scenes: FK error bound, configuration and edge
verdicts against the FP64 oracle, including constructed near-contact cases
that exercise the FP64 re-check pass.  Verdicts must be bit-exact."""
import copy

import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def sparse_arm_scene(seed=1, n_boxes=5):
    return pkg("scenes").make_arm_scene(seed, n_boxes=n_boxes)


def test_fk_fp64_bit_exact_and_fp32_within_band(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    for scene in (scenes.make_arm_scene(0), scenes.make_mobile_scene(0)):
        sc = col.Gb300Scene(scene)
        o = oracle.OracleScene(scene)
        q = scenes.uniform_configs(scene, 4000, seed=5, dtype=np.float64)
        c32, c64 = sc.sphere_centers(q)
        c32, c64 = c32.cpu().numpy().astype(np.float64), c64.cpu().numpy()
        for i in range(0, 4000, 97):
            assert np.array_equal(c64[i], o.sphere_centers(q[i])), i
        err = np.abs(c32 - c64).max()
        band = sc.info()["band"]
        assert err * 10 <= band, (err, band)


def test_arm_configs_vs_oracle(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    for scene in (scenes.make_arm_scene(0), sparse_arm_scene()):
        sc = col.Gb300Scene(scene)
        o = oracle.OracleScene(scene)
        for dt in (np.float32, np.float64):
            q = scenes.uniform_configs(scene, 20000, seed=9, dtype=dt)
            got = sc.is_collision_free_batch(q).cpu().numpy()
            ref = o.configs_free(q)
            assert np.array_equal(got, ref), (dt, int((got != ref).sum()))


def test_mobile_configs_vs_oracle(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_mobile_scene(0)
    sc = col.Gb300Scene(scene)
    o = oracle.OracleScene(scene)
    q = scenes.uniform_configs(scene, 5000, seed=4, dtype=np.float32)
    assert np.array_equal(sc.is_collision_free_batch(q).cpu().numpy(), o.configs_free(q))


def _free_configs(o, scene, n, seed):
    q = pkg("scenes").uniform_configs(scene, 40 * n, seed=seed, dtype=np.float64)
    f = o.configs_free(q).astype(bool)
    return q[f][:n]


def test_arm_edges_vs_oracle(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_arm_scene(0)
    w = scenes.make_arm_workload(scene, seed=0, n_configs=10, n_edges=3000)
    sc = col.Gb300Scene(scene)
    o = oracle.OracleScene(scene)
    got = sc.is_edge_collision_free_batch(w["q1"], w["q2"], w["resolution"]).cpu().numpy()
    ref = o.edges_free(w["q1"], w["q2"], w["resolution"])
    assert np.array_equal(got, ref)
    # a sparse scene with short edges between free configurations: many free edges
    scene = sparse_arm_scene()
    sc = col.Gb300Scene(scene)
    o = oracle.OracleScene(scene)
    a = _free_configs(o, scene, 600, 3)
    rng = np.random.default_rng(0)
    b = a + rng.uniform(-0.15, 0.15, a.shape)
    for kw in [dict(), dict(include_endpoints=True), dict(N_start=2, N_max=9), dict(N_start=4)]:
        res = 0.02
        N = np.maximum(2, (np.abs(a - b).max(1) / res).astype(np.int64) + 1)
        keep = N >= kw.get("N_start", 0)
        got = sc.is_edge_collision_free_batch(a[keep], b[keep], res, **kw).cpu().numpy()
        ref = o.edges_free(a[keep], b[keep], res, **kw)
        assert np.array_equal(got, ref), kw
        assert ref.mean() > 0.2   # the test covers free edges, not only early exits


def test_mobile_edges_vs_oracle(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_mobile_scene(0)
    sc = col.Gb300Scene(scene)
    o = oracle.OracleScene(scene)
    N = np.random.default_rng(2).integers(5, 80, 400)
    q1, q2 = scenes.edges_with_steps(scene, N, 0.05, seed=8)
    assert np.array_equal(sc.is_edge_collision_free_batch(q1, q2, 0.05).cpu().numpy(), o.edges_free(q1, q2, 0.05))


def _with_boxes(scene, lo, hi):
    s = copy.deepcopy(scene)
    s.box_lo = np.asarray(lo, dtype=np.float64).reshape(-1, 3)
    s.box_hi = np.asarray(hi, dtype=np.float64).reshape(-1, 3)
    return s


def test_near_contact_sphere_box(gpu, oracle):
    """A box face placed at distance r + eps from one sphere centre, eps from
    -1e-5 to 1e-5 m (inside the FP32 band) down to a few ulps."""
    scenes, col = pkg("scenes"), pkg("collision")
    base = sparse_arm_scene(2, n_boxes=0)
    o0 = oracle.OracleScene(base)
    qs = _free_configs(o0, base, 30, 11)
    rng = np.random.default_rng(5)
    eps_set = [-1e-5, -1e-7, -1e-10, -1e-13, 0.0, 1e-13, 1e-10, 1e-7, 1e-5]
    rechecked = 0
    for i, q in enumerate(qs):
        c = o0.sphere_centers(q)
        s = rng.integers(len(c))
        r = float(base.sphere_radius[s])
        eps = eps_set[i % len(eps_set)]
        k = rng.integers(3)
        lo = c[s] - 0.05
        hi = c[s] + 0.05
        lo[k] = c[s][k] + r + eps          # face at +k, distance r + eps
        hi[k] = lo[k] + 0.1
        scene = _with_boxes(base, lo, hi)
        sc = col.Gb300Scene(scene)
        o = oracle.OracleScene(scene)
        got = sc.is_collision_free_batch(q[None]).item()
        rechecked += sc.last_call_stats()["rechecked_fp64"]
        assert got == o.config_free(q), (i, eps)
    assert rechecked > 0


def test_near_contact_sphere_sphere(gpu, oracle):
    """Robot 1 translated towards its closest sphere pair (a on another robot,
    b on robot 1) until that pair is at distance r_a + r_b + eps; every other
    pair involving robot 1 keeps a gap >= eps."""
    scenes, col = pkg("scenes"), pkg("collision")
    base = sparse_arm_scene(3, n_boxes=0)
    o0 = oracle.OracleScene(base)
    qs = _free_configs(o0, base, 24, 13)
    eps_set = [-1e-5, -1e-9, -1e-14, 0.0, 1e-14, 1e-9, 1e-5]
    ids1 = np.where(base.sphere_robot == 1)[0]
    ids_o = np.where(base.sphere_robot != 1)[0]
    rad = base.sphere_radius
    rechecked = 0
    for i, q in enumerate(qs):
        c = o0.sphere_centers(q)
        gaps = np.linalg.norm(c[ids_o][:, None] - c[ids1][None], axis=-1) - (rad[ids_o][:, None] + rad[ids1][None])
        ia, ib = np.unravel_index(np.argmin(gaps), gaps.shape)
        a, b = ids_o[ia], ids1[ib]
        R = rad[a] + rad[b] + eps_set[i % len(eps_set)]
        d = c[b] - c[a]
        u = d / np.linalg.norm(d)
        shift = (c[a] + u * R) - c[b]
        scene = copy.deepcopy(base)
        scene.base_pose[1, 9:] = scene.base_pose[1, 9:] + shift
        sc = col.Gb300Scene(scene)
        o = oracle.OracleScene(scene)
        got = sc.is_collision_free_batch(q[None]).item()
        rechecked += sc.last_call_stats()["rechecked_fp64"]
        assert got == o.config_free(q), i
    assert rechecked > 0


def test_arm_nan_and_huge_inputs(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    scene = sparse_arm_scene()
    sc = col.Gb300Scene(scene)
    o = oracle.OracleScene(scene)
    q = scenes.uniform_configs(scene, 64, seed=1, dtype=np.float64)
    q[0, 3] = np.nan
    q[1, 5] = 1e7          # beyond the FP32 reduction range: exact path
    q[2, 0] = 3e9          # sine/cosine defined as NaN beyond 2^30
    q[3, 27] = np.inf
    assert np.array_equal(sc.is_collision_free_batch(q).cpu().numpy(), o.configs_free(q))


def test_tuned_test_order_keeps_verdicts(gpu, oracle):
    """The autotuned box order changes how soon a collision is found, never a verdict."""
    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_scene(0)
    env = envm.Gb300ArmEnvironment(scene, tune_samples=2048, seed=3)
    assert sorted(env.box_order.tolist()) == list(range(len(scene.box_lo)))
    o = oracle.OracleScene(scene)
    w = scenes.make_arm_workload(scene, seed=5, n_configs=20000, n_edges=5000)
    assert np.array_equal(env.batch_is_collision_free(w["configs"]).astype(np.uint8), o.configs_free(w["configs"]))
    assert np.array_equal(env.batch_is_edge_collision_free(w["q1"], w["q2"]).astype(np.uint8),
                          o.edges_free(w["q1"], w["q2"], w["resolution"]))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_edge_check_plan_graph(gpu, oracle, dtype):
    """The graph-captured plan (pipelined host->device chunks) gives the oracle's
    verdicts, run after run, and reports bad edges as the plain call does;
    FP64 endpoint buffers (the default) and FP32 ones."""
    import torch

    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_scene(0)
    env = envm.Gb300ArmEnvironment(scene, tune_samples=0)
    o = oracle.OracleScene(scene)
    w = scenes.make_arm_workload(scene, seed=2, n_configs=10, n_edges=6000)
    ref = o.edges_free(w["q1"], w["q2"], w["resolution"])
    plan = env.edge_check_plan(6000, chunks=3, dtype=getattr(torch, dtype))
    assert plan.q1_host.dtype == np.dtype(dtype)
    plan.q1_host[:] = w["q1"]
    plan.q2_host[:] = w["q2"]
    for _ in range(3):
        assert np.array_equal(plan.run(), ref)
    plan.q2_host[17, 0] = np.nan
    plan.q1_host[17, 0] = np.nan
    with pytest.raises(ValueError):
        plan.run()


def test_edge_check_pipeline(gpu, oracle):
    """Two plans in flight on separate scene handles: every batch gets the
    oracle's verdicts, also when the slots hold different batches."""
    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_scene(0)
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=0.05, tune_samples=512)
    o = oracle.OracleScene(scene)
    w = [scenes.make_arm_workload(scene, seed=s, n_configs=10, n_edges=700) for s in (1, 2, 3)]
    want = [o.edges_free(x["q1"], x["q2"], 0.05) for x in w]
    pipe = env.edge_check_pipeline(700, depth=2)
    assert pipe.depth == 2
    got = []
    order = [0, 1, 2, 1, 0, 2]
    tickets = []
    for k, i in enumerate(order):
        slot = pipe.next
        if len(tickets) >= pipe.depth:
            t, j = tickets.pop(0)
            got.append((j, pipe.result(t).copy()))
        pipe.plans[slot].q1_host[:] = w[i]["q1"]
        pipe.plans[slot].q2_host[:] = w[i]["q2"]
        tickets.append((pipe.submit(), i))
    for t, j in tickets:
        got.append((j, pipe.result(t).copy()))
    assert len(got) == len(order)
    for j, v in got:
        assert np.array_equal(v, want[j]), j


@pytest.mark.parametrize("kind", ["arm", "mobile"])
def test_collision_free_for_robot(gpu, oracle, kind):
    """is_collision_free_for_robot: every robot subset tried gives the
    oracle's verdicts; the full set equals is_collision_free."""
    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_scene(0) if kind == "arm" else scenes.make_mobile_scene(0)
    env = envm.Gb300ArmEnvironment(scene, tune_samples=256)
    o = oracle.OracleScene(scene)
    q = scenes.uniform_configs(scene, 3000, seed=17)
    R = scene.n_robots
    masks = [1 << r for r in range(R)] + [0b11, (1 << R) - 1, 0b101]
    for m in masks:
        names = [env.robots[r] for r in range(R) if (m >> r) & 1]
        got = env.batch_is_collision_free_for_robot(names, q)
        want = o.configs_free_for_robots(q, m)
        assert np.array_equal(got.astype(np.uint8), want), m
    assert np.array_equal(env.batch_is_collision_free_for_robot(env.robots, q), env.batch_is_collision_free(q))
    assert env.is_collision_free_for_robot(env.robots[0], q[0]) == bool(o.configs_free_for_robots(q[:1], 1)[0])
    with pytest.raises(ValueError):
        env.is_collision_free_for_robot("no-such-robot", q[0])
