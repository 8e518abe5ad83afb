"""GPU parity for per-mode scene tables: in each mode the configuration and
edge verdicts, the per-robot check, the path check and the penetration cost
equal the oracle's on the scene as that mode sees it (its boxes and the
attached objects present).  Verdicts bit-exact; cost within 1e-5."""
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from conftest import pkg

pytestmark = pytest.mark.gpu

MODES = [-1, 0, 1, 5, 7, 11]


def _view(scene, m):
    return scene if m < 0 else scene.for_mode(m)


def test_mode_configs_and_edges(gpu, oracle):
    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_arm_mode_scene(0)
    sc = col.Gb300Scene(scene)
    q = scenes.uniform_configs(scene, 8000, seed=3, dtype=np.float32)
    N = np.random.default_rng(4).integers(5, 60, 600)
    q1, q2 = scenes.edges_with_steps(scene, N, 0.05, seed=6)
    verdicts = {}
    for m in MODES:
        sc.set_mode(m)
        o = oracle.OracleScene(_view(scene, m))
        got = sc.is_collision_free_batch(q).cpu().numpy()
        assert np.array_equal(got, o.configs_free(q)), m
        verdicts[m] = got
        e = sc.is_edge_collision_free_batch(q1, q2, 0.05).cpu().numpy()
        assert np.array_equal(e, o.edges_free(q1, q2, 0.05)), m
    # the modes' tables differ: objects move between poses and into grippers
    assert len({v.tobytes() for v in verdicts.values()}) >= 4


def test_mode_switch_back_and_forth(gpu, oracle):
    """Switching is a table selection: the same mode gives the same verdicts
    after other modes ran, including the scene as created (-1)."""
    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_arm_mode_scene(1, n_modes=4)
    sc = col.Gb300Scene(scene)
    q = scenes.uniform_configs(scene, 3000, seed=8, dtype=np.float64)
    first = {}
    for m in [2, -1, 0, 3, 1]:
        sc.set_mode(m)
        first[m] = sc.is_collision_free_batch(q).cpu().numpy()
    for m in [1, 3, -1, 2, 0]:
        sc.set_mode(m)
        assert np.array_equal(sc.is_collision_free_batch(q).cpu().numpy(), first[m]), m
    with pytest.raises(ValueError):
        sc.set_mode(4)


def test_mode_robot_mask(gpu, oracle):
    """is_collision_free_for_robot inside a mode: a held object moves with its
    robot and is checked with that robot."""
    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_arm_mode_scene(0)
    sc = col.Gb300Scene(scene)
    q = scenes.uniform_configs(scene, 4000, seed=9, dtype=np.float32)
    for m in [1, 7]:
        sc.set_mode(m)
        o = oracle.OracleScene(_view(scene, m))
        for mask in (0b0001, 0b0110, 0b1011):
            got = sc.is_collision_free_batch_robots(q, mask).cpu().numpy()
            assert np.array_equal(got, o.configs_free_for_robots(q, mask)), (m, mask)


def test_mode_env_path_check(gpu, oracle):
    """Gb300ArmEnvironment on a per-mode scene: single checks take the mode
    argument, and a path whose states carry modes is checked vertex by vertex
    and edge by edge in the reference's modes (an edge in its first state's)."""
    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_mode_scene(0)
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=0.05, tune_samples=512)
    rng = np.random.default_rng(2)
    orcs = {m: oracle.OracleScene(scene.for_mode(m)) for m in range(scene.n_modes)}
    free = {m: orcs[m].configs_free(scenes.uniform_configs(scene, 3000, seed=m, dtype=np.float64)) for m in orcs}
    qs = {m: scenes.uniform_configs(scene, 3000, seed=m, dtype=np.float64)[free[m].astype(bool)] for m in orcs}
    for m in (0, 5, 9):
        for q in qs[m][:5]:
            assert env.is_collision_free(q, m)
    n_checked = 0
    for trial in range(12):
        modes = sorted(rng.choice(scene.n_modes, 3, replace=False).tolist())
        states = []
        for m in modes:
            for q in qs[m][rng.integers(0, len(qs[m]), 2)]:
                states.append(SimpleNamespace(q=q, mode=m))
        path = states
        want = all(orcs[s.mode].configs_free(s.q[None])[0] for s in path)
        for i in range(len(path) - 1):
            want = want and bool(orcs[path[i].mode].edges_free(path[i].q[None], path[i + 1].q[None], 0.05)[0])
        assert env.is_path_collision_free(path) == want, trial
        n_checked += 1
    assert n_checked == 12


def test_mode_penetration_cost(gpu):
    """The penetration cost of a mode counts its boxes and the held objects."""
    import penetration_f64 as orc_pen

    scenes, col, pen = pkg("scenes"), pkg("collision"), pkg("penetration")
    scene = scenes.make_arm_mode_scene(0)
    sc = col.Gb300Scene(scene)
    paths = scenes.make_path_workload(scene, seed=3, n_paths=3, n_waypoints=40)
    costs = {}
    for m in [-1, 1, 7]:
        sc.set_mode(m)
        c = pen.path_penetration(sc, torch.from_numpy(paths).cuda())["cost"].cpu().numpy()
        ref = orc_pen.penetration_cost(_view(scene, m).arrays(), torch.from_numpy(paths.astype(np.float64))).numpy()
        assert np.all(np.abs(c - ref) <= 1e-5 * np.abs(ref)), m
        costs[m] = c
    assert not np.allclose(costs[1], costs[7])


def test_mode_edge_cases(gpu, oracle):
    """A mode with no boxes and no attached objects (only robot-robot
    contacts remain), a mode with every object held, and the argument
    checks: repeated or out-of-range boxes and a second set of modes are
    refused."""
    import copy

    scenes, col = pkg("scenes"), pkg("collision")
    base = scenes.make_arm_mode_scene(2, n_objects=4, n_modes=3)
    scene = copy.deepcopy(base)
    scene.mode_boxes = [[], list(range(len(scene.box_lo))), [0, 3]]
    scene.mode_attach = [[], [0, 1, 2, 3], [2]]
    sc = col.Gb300Scene(scene)
    q = scenes.uniform_configs(scene, 3000, seed=4, dtype=np.float32)
    for m in range(3):
        sc.set_mode(m)
        o = oracle.OracleScene(scene.for_mode(m))
        assert np.array_equal(sc.is_collision_free_batch(q).cpu().numpy(), o.configs_free(q)), m
    sc.set_mode(0)
    assert sc.is_collision_free_batch(q).cpu().numpy().mean() > 0.5   # no boxes: most configurations free
    for boxes in ([[0, 0]], [[len(scene.box_lo)]]):
        bad = copy.deepcopy(base)
        bad.mode_boxes, bad.mode_attach = boxes, [[]]
        with pytest.raises(ValueError):
            col.Gb300Scene(bad)
    t = scene.mode_tables()
    with pytest.raises(ValueError):
        pkg("_lib").check(sc.lib.mrmg_arm_scene_set_modes(
            sc.h, scene.n_modes, t["sphere_attach"].ctypes.data, t["box_off"].ctypes.data, t["boxes"].ctypes.data,
            t["attach_off"].ctypes.data, t["attach"].ctypes.data))
