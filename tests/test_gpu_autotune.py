"""Work-shape tuning of the arm kernels (obstacle tile = box_block, box head,
configurations per warp grab, phase-B1 depth, launch shape): every setting
gives the oracle's verdicts; the autotuner searches them on a sample of the
workload and leaves the fastest on the scene."""
import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def _setup(oracle, n_boxes=50, scene_seed=0):
    scenes, col = pkg("scenes"), pkg("collision")
    sc = scenes.make_arm_scene(scene_seed, n_boxes=n_boxes)
    N = scenes.lognormal_steps(3000, 5)
    q1, q2 = scenes.edges_with_steps(sc, N, 0.05, 6)
    q = scenes.uniform_configs(sc, 20000, seed=7)
    o = oracle.OracleScene(sc)
    return sc, col.Gb300Scene(sc), o, q1, q2, N, q


@pytest.mark.parametrize("n_boxes", [12, 50])
def test_tuning_never_changes_verdicts(gpu, oracle, n_boxes):
    sc, s, o, q1, q2, N, q = _setup(oracle, n_boxes)
    ref_e = o.edges_free(q1, q2, 0.05, N=N)
    ref_c = o.configs_free(q)
    assert 0 < ref_c.sum() < len(ref_c)
    settings = [(1, 0, 1, 1), (2, 64, 32, 64), (4, 4, 2, 2), (16, 16, 8, 6), (32, 8, 4, 3), (8, 0, 16, 1), (0, 0, 0, 0)]
    for bb, head, chunk, b1 in settings:
        s.set_tuning(bb, head, chunk, b1)
        got = s.get_tuning()
        assert got == {"box_block": bb or 8, "box_head": head, "cfg_chunk": chunk or 4, "phase_b1": b1 or 3}
        for flags in (0, pkg("_lib").MRMG_FLAG_FULL_EVAL):
            e = s.is_edge_collision_free_batch(q1, q2, 0.05, N=N, flags=flags).cpu().numpy()
            assert np.array_equal(e, ref_e), (bb, head, chunk, b1, flags)
        assert np.array_equal(s.is_collision_free_batch(q).cpu().numpy(), ref_c), (bb, head, chunk, b1)
        assert np.array_equal(s.is_edge_collision_free_host(q1[:300], q2[:300], 0.05), ref_e[:300])


def test_tuning_rejects_out_of_range(gpu):
    scenes, col = pkg("scenes"), pkg("collision")
    s = col.Gb300Scene(scenes.make_arm_scene(0))
    for bad in [(33, 0, 0, 0), (0, 65, 0, 0), (0, 0, 33, 0), (0, 0, 0, 65), (-1, 0, 0, 0)]:
        with pytest.raises(ValueError):
            s.set_tuning(*bad)
    assert s.get_tuning() == {"box_block": 8, "box_head": 8, "cfg_chunk": 4, "phase_b1": 3}
    a = col.Gb300Scene(scenes.make_disc_scene(0))
    with pytest.raises(ValueError):
        a.set_tuning(8, 8, 4, 3)


@pytest.mark.parametrize("kind", ["edges", "configs"])
def test_autotune_picks_a_setting_and_keeps_verdicts(gpu, oracle, kind):
    at = pkg("autotune")
    sc, s, o, q1, q2, N, q = _setup(oracle)
    space = {"launch": [(1, 8), (2, 4)], "box_block": (4, 16), "box_head": (0, 16), "phase_b1": (2, 6),
             "cfg_chunk": (2, 8)}
    if kind == "edges":
        r = at.autotune(s, q1, q2, N, resolution=0.05, space=space, repeats=1)
    else:
        r = at.autotune(s, configs=q, space=space, repeats=1)
    assert r["best_ms"] <= r["default_ms"]
    assert len(r["table"]) >= 5
    t = s.get_tuning()
    for k in ("box_block", "box_head", "cfg_chunk", "phase_b1"):
        assert t[k] == r["best"][k]
    assert np.array_equal(s.is_edge_collision_free_batch(q1, q2, 0.05, N=N).cpu().numpy(),
                          o.edges_free(q1, q2, 0.05, N=N))
    assert np.array_equal(s.is_collision_free_batch(q).cpu().numpy(), o.configs_free(q))
