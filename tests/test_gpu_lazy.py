"""GPU parity of batched lazy edge evaluation: the PRM's lazy A* with the
speculative batched checker on the GPU backend gives the reference search's
path and counters (golden vectors from the reference's own search), in far
fewer device calls than edges checked."""
import numpy as np
import pytest

from conftest import golden, pkg

pytestmark = pytest.mark.gpu


class _Node:
    def __init__(self, i, q, mode=0):
        self.id = i
        self.state = type("State", (), {"q": q, "mode": mode})()
        self.whitelist, self.blacklist = set(), set()


@pytest.mark.parametrize("window", [1, 64])
def test_prm_lazy_search_gpu_golden(gpu, window):
    lazy, scenes, envm = pkg("lazy"), pkg("scenes"), pkg("env")
    g = golden("prm_search.npz")
    env = envm.Gb300AbstractEnvironment(scenes.make_disc_scene(0))
    qs, nbr = g["configs"], g["neighbors"]
    for tag in ("found", "missing"):
        nodes = [_Node(i, env.start_pos.from_flat(q)) for i, q in enumerate(qs)]
        goal = nodes[int(g[f"goal_{tag}"])]
        gq = qs[int(g[f"goal_{tag}"])][None]
        checker = lazy.SpeculativeEdgeChecker(env, resolution=float(g["resolution"]), window=window)
        r = lazy.lazy_astar(nodes[0], [goal], lambda n: ([nodes[j] for j in nbr[n.id]], qs[nbr[n.id]]),
                            env.config_cost, env.batch_config_cost,
                            lambda n: float(np.min(env.batch_config_cost(n.state.q, gq))), checker)
        assert [n.id for n in r["path"]] == g[f"path_{tag}"].tolist(), tag
        assert r["processed_edges"] == int(g[f"processed_edges_{tag}"]), tag
        assert r["wasted_pops"] == int(g[f"wasted_pops_{tag}"]), tag
        if window > 1:
            assert r["calls"] * 4 <= r["lookups"], r


def test_lazy_checker_modes(gpu, oracle):
    """Speculated edges are grouped by the mode of their first node and
    checked in that mode's tables (a per-mode arm scene)."""
    lazy, scenes, envm = pkg("lazy"), pkg("scenes"), pkg("env")
    scene = scenes.make_arm_mode_scene(0)
    env = envm.Gb300ArmEnvironment(scene, tune_samples=256)
    rng = np.random.default_rng(5)
    n = 60
    q = scenes.uniform_configs(scene, 2 * n, seed=2, dtype=np.float64)
    q1, q2 = q[:n], q[:n] + rng.uniform(-0.05, 0.05, (n, scene.q_dim))
    modes = rng.integers(0, scene.n_modes, n)
    a = [_Node(2 * i, q1[i], int(modes[i])) for i in range(n)]
    b = [_Node(2 * i + 1, q2[i], int(modes[i])) for i in range(n)]
    checker = lazy.SpeculativeEdgeChecker(env, resolution=0.05, window=n)
    got = [checker.is_free(a[0], b[0], list(zip(a[1:], b[1:])))]
    got += [checker.is_free(a[i], b[i]) for i in range(1, n)]
    assert checker.stats()["edges_checked"] == n
    assert checker.stats()["calls"] == len(set(modes.tolist()))
    want = [bool(oracle.OracleScene(scene.for_mode(int(modes[i]))).edges_free(q1[i][None], q2[i][None], 0.05)[0])
            for i in range(n)]
    assert got == want
