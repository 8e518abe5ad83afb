"""Shortcutting on the device: robot_mode_shortcut (planners/shortcutting.py:
87-244) through the GB300 abstract env reproduces the reference's own
shortcut paths and cost traces (shortcut.npz); gradient repair turns
colliding straight-line shortcuts into paths that pass the exact path check
(every verdict confirmed edge by edge by the oracle); the batched
shortcutter with repair returns paths the oracle finds free."""
import numpy as np
import pytest
import torch

from conftest import pkg
from test_shortcutting import _Mode, _State, _fixture, run_golden, start_paths

pytestmark = pytest.mark.gpu


def test_robot_mode_shortcut_golden_on_device(gpu):
    g, scene = _fixture()
    env = pkg("env").Gb300AbstractEnvironment(scene)
    run_golden(env, g)


def test_batched_shortcut_abstract_on_device(gpu, oracle):
    g, scene = _fixture()
    env = pkg("env").Gb300AbstractEnvironment(scene)
    o = oracle.OracleScene(scene)
    sc = pkg("shortcutting")
    paths, _ = start_paths(g)
    for p, path in enumerate(paths):
        st = {}
        new, (cst, _t) = sc.batched_robot_mode_shortcut(env, path, rounds=6, batch=128, resolution=0.01,
                                                         interpolation_resolution=0.1,
                                                         rng=np.random.default_rng(p), stats=st)
        Q = np.array([s.q.state() for s in new])
        np.testing.assert_array_equal(Q[0], path[0].q.state())
        np.testing.assert_array_equal(Q[-1], path[-1].q.state())
        assert all(b <= a for a, b in zip(cst, cst[1:]))
        assert o.configs_free(Q).all() and o.edges_free(Q[:-1], Q[1:], 0.01).all()


def _arm_setup(oracle, seed=2, n_boxes=20):
    scenes, col = pkg("scenes"), pkg("collision")
    sc = scenes.make_arm_scene(seed, n_boxes=n_boxes)
    return sc, col.Gb300Scene(sc), oracle.OracleScene(sc)


def test_repair_makes_colliding_shortcuts_free(gpu, oracle):
    """Straight lines between free configurations that collide, repaired
    with the end states held: at least one in eight becomes collision-free,
    and every path's verdict (free or not) is the oracle's exact edge check
    of its consecutive waypoints, end states included."""
    pen = pkg("penetration")
    sc, s, o = _arm_setup(oracle)
    rng = np.random.default_rng(5)
    q = rng.uniform(sc.limits[0], sc.limits[1], (20000, sc.q_dim))
    a = q[o.configs_free(q).astype(bool)]
    b = np.clip(a + rng.uniform(-0.8, 0.8, a.shape), sc.limits[0], sc.limits[1])
    ok = o.configs_free(b).astype(bool)
    a, b = a[ok], b[ok]
    T = 24
    paths = (a[:, None, :] + (b - a)[:, None, :] * np.linspace(0.0, 1.0, T)[None, :, None]).astype(np.float32)
    before = pen.path_collision_free(s, paths, 0.05).cpu().numpy()
    bad = paths[before == 0][:64]
    assert len(bad) >= 32
    res = pen.repair_paths(s, bad, pen.PenetrationParams(beta=50.0), iters=80, step=1e-3, resolution=0.05,
                           limits=sc.limits)
    W = res["paths"].cpu().numpy()
    free = res["collision_free"].cpu().numpy().astype(bool)
    np.testing.assert_array_equal(W[:, 0], bad[:, 0])
    np.testing.assert_array_equal(W[:, -1], bad[:, -1])
    assert bool((res["cost_after"] <= res["cost_before"]).all())
    for p in range(len(W)):
        ref = bool(o.edges_free(W[p, :-1], W[p, 1:], 0.05, include_endpoints=True).all())
        assert free[p] == ref, p
    print(f"repaired {free.sum()} of {len(W)} colliding straight-line paths")
    assert free.sum() * 8 >= len(W)


def _free_walk(o, sc, rng, n_states, step, resolution):
    while True:
        q = rng.uniform(sc.limits[0], sc.limits[1], sc.q_dim)
        if o.configs_free(q[None])[0]:
            break
    qs = [q]
    while len(qs) < n_states:
        c = np.clip(qs[-1] + rng.uniform(-step, step, sc.q_dim), sc.limits[0], sc.limits[1])
        if o.configs_free(c[None])[0] and o.edges_free(qs[-1][None], c[None], resolution)[0]:
            qs.append(c)
    return np.array(qs)


def test_batched_shortcut_with_repair_arm(gpu, oracle):
    """Four-arm table scene: a free random walk, shortcut with gradient
    repair of colliding candidates.  The result keeps its end states, never
    raises the cost, is free under the oracle (every state, every edge at the
    env's resolution) and some repaired candidates were accepted."""
    envm, sc_mod = pkg("env"), pkg("shortcutting")
    sc, _s, o = _arm_setup(oracle)
    env = envm.Gb300ArmEnvironment(sc, collision_resolution=0.05, tune_samples=512)
    cfg = pkg("configuration").Gb300Configuration
    sl = [tuple(map(int, x)) for x in sc.agent_slices()]
    mode = _Mode([0] * sc.n_robots)
    totals = {}
    for seed in range(3):
        rng = np.random.default_rng(100 + seed)
        qs = _free_walk(o, sc, rng, 10, 0.35, 0.05)
        path = [_State(cfg(q, sl), mode) for q in qs]
        st = {}
        new, (cst, _t) = sc_mod.batched_robot_mode_shortcut(env, path, rounds=6, batch=256, resolution=0.05,
                                                             interpolation_resolution=0.1, repair=True,
                                                             repair_iters=60, rng=rng, stats=st,
                                                             penetration_params=pkg("penetration").PenetrationParams(beta=50.0))
        Q = np.array([s.q.state() for s in new])
        np.testing.assert_array_equal(Q[0], qs[0])
        np.testing.assert_array_equal(Q[-1], qs[-1])
        assert all(b <= a for a, b in zip(cst, cst[1:]))
        assert o.configs_free(Q).all()
        assert o.edges_free(Q[:-1], Q[1:], 0.05).all()
        for k, v in st.items():
            totals[k] = totals.get(k, 0) + v
    print("shortcut stats", totals)
    assert totals["accepted"] >= 1 and totals["repaired"] >= 1


class _IdMode(_Mode):
    def __init__(self, i, task_ids):
        super().__init__(task_ids)
        self.id = i


def test_shortcutting_on_a_per_mode_scene(gpu, oracle):
    """Per-mode tables: a path through modes 1 and 2 (different box sets,
    robot 0's task changes at the switch).  Both shortcutters keep every
    state free in its own mode and every edge free in its first state's mode
    (the reference's rule, planning_env.py:1805-1816)."""
    import dataclasses

    scenes, envm, sc_mod = pkg("scenes"), pkg("env"), pkg("shortcutting")
    base = scenes.make_arm_scene(2, n_boxes=20)
    sc = dataclasses.replace(base, mode_boxes=[list(range(20)), list(range(0, 20, 2)), list(range(1, 20, 2))])
    env = envm.Gb300ArmEnvironment(sc, collision_resolution=0.05, tune_samples=256)
    orcs = {m: oracle.OracleScene(sc.for_mode(m)) for m in (1, 2)}
    modes = {1: _IdMode(1, [0, 0, 0, 0]), 2: _IdMode(2, [1, 0, 0, 0])}
    cfg = pkg("configuration").Gb300Configuration
    sl = [tuple(map(int, x)) for x in sc.agent_slices()]
    rng = np.random.default_rng(7)
    while True:
        w1 = _free_walk(orcs[1], sc, rng, 6, 0.3, 0.05)
        if orcs[2].configs_free(w1[-1:])[0]:
            break
    qs2 = [w1[-1]]
    while len(qs2) < 6:
        c = np.clip(qs2[-1] + rng.uniform(-0.3, 0.3, sc.q_dim), sc.limits[0], sc.limits[1])
        if orcs[2].configs_free(c[None])[0] and orcs[2].edges_free(qs2[-1][None], c[None], 0.05)[0]:
            qs2.append(c)
    path = [_State(cfg(q, sl), modes[1]) for q in w1] + [_State(cfg(q, sl), modes[2]) for q in qs2]

    def check(states, end_atol):
        Q = np.array([s.q.state() for s in states])
        ms = [s.mode.id for s in states]
        for i, m in enumerate(ms):
            assert orcs[m].configs_free(Q[i:i + 1])[0], i
        for i in range(len(Q) - 1):
            assert orcs[ms[i]].edges_free(Q[i:i + 1], Q[i + 1:i + 2], 0.05)[0], i
        np.testing.assert_array_equal(Q[0], w1[0])
        np.testing.assert_allclose(Q[-1], qs2[-1], rtol=0, atol=end_atol)

    # the reference's shortcutter rewrites the end state as q0 + diff * (j - i),
    # within an ulp of the original (it asserts 1e-6, shortcutting.py:236-238)
    np.random.seed(3)
    new, (cst, _t) = sc_mod.robot_mode_shortcut(env, path, max_iter=60, resolution=0.05, interpolation_resolution=0.1)
    check(new, 1e-6)
    assert cst[-1] <= cst[0]
    st = {}
    new, (cst, _t) = sc_mod.batched_robot_mode_shortcut(env, path, rounds=4, batch=128, resolution=0.05,
                                                         interpolation_resolution=0.1, rng=np.random.default_rng(3),
                                                         stats=st)
    check(new, 0.0)
    assert all(b <= a for a, b in zip(cst, cst[1:])) and st["accepted"] >= 1
