"""GPU parity of the serving batcher: every verdict of a packed step equals
the oracle's verdict of the same configuration / edge checked alone, across
capacity buckets, empty instances and launch shapes."""
import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def _requests(scene, seed, n=6, configs=(0, 700), edges=(0, 300), steps=(5, 120)):
    return pkg("scenes").make_serving_requests(scene, seed=seed, n_instances=n, configs=configs, edges=edges,
                                               steps=steps)


def _check(orc, reqs, res, resolution=0.05):
    for r, cf, ef in zip(reqs, res.config_free, res.edge_free):
        c = r.get("configs", np.zeros((0, 1)))
        if len(c):
            assert np.array_equal(cf, orc.configs_free(c))
        else:
            assert len(cf) == 0
        if len(r.get("q1", [])):
            assert np.array_equal(ef, orc.edges_free(r["q1"], r["q2"], resolution, N=r["N"]))
        else:
            assert len(ef) == 0


def test_serving_steps_match_oracle(gpu, oracle):
    scenes, col, srv = pkg("scenes"), pkg("collision"), pkg("serving")
    sc = scenes.make_mobile_scene(0)
    s = col.Gb300Scene(sc)
    orc = oracle.OracleScene(sc)
    b = srv.ServingBatcher(s, config_quantum=1024, edge_quantum=256)
    for seed in range(3):
        reqs = _requests(sc, seed)
        reqs[1] = dict(configs=np.zeros((0, sc.q_dim), np.float32))          # an instance with nothing
        res = b.step(reqs)
        _check(orc, reqs, res)
        assert res.n_configs == sum(len(r.get("configs", [])) for r in reqs)
    assert len(b.graphs) >= 1
    lat = b.latency_percentiles()
    assert lat["steps"] == 3 and lat["p99_ms"] >= lat["p50_ms"] > 0


def test_serving_resolution_edges_and_free_configs(gpu, oracle):
    """Edges without N use the resolution formula; the arm scene has free
    configurations, so both verdicts occur."""
    scenes, col, srv = pkg("scenes"), pkg("collision"), pkg("serving")
    sc = scenes.make_arm_scene(0)
    s = col.Gb300Scene(sc)
    orc = oracle.OracleScene(sc)
    w = scenes.make_arm_workload(sc, seed=3, n_configs=3000, n_edges=400)
    reqs = [dict(configs=w["configs"][:1500], q1=w["q1"][:200], q2=w["q2"][:200]),
            dict(configs=w["configs"][1500:], q1=w["q1"][200:], q2=w["q2"][200:])]
    b = srv.ServingBatcher(s, resolution=w["resolution"], config_quantum=4096, edge_quantum=512)
    res = b.step(reqs)
    for r, cf, ef in zip(reqs, res.config_free, res.edge_free):
        assert np.array_equal(cf, orc.configs_free(r["configs"]))
        assert np.array_equal(ef, orc.edges_free(r["q1"], r["q2"], w["resolution"]))
    allc = np.concatenate(res.config_free)
    assert 0 < allc.sum() < len(allc)
    N = srv.edge_steps(w["q1"], w["q2"], w["resolution"])
    assert np.array_equal(N, w["N"])


def test_autotune_keeps_verdicts(gpu, oracle):
    scenes, col, srv = pkg("scenes"), pkg("collision"), pkg("serving")
    sc = scenes.make_mobile_scene(0)
    s = col.Gb300Scene(sc)
    reqs = _requests(sc, 11, n=2, configs=(200, 200), edges=(300, 300))
    q1 = np.concatenate([r["q1"] for r in reqs])
    q2 = np.concatenate([r["q2"] for r in reqs])
    N = np.concatenate([r["N"] for r in reqs])
    t = srv.autotune_launch(s, q1, q2, N, ctas_per_sm=(1, 2), warps=(4, 8), repeats=1)
    assert t["best"] is not None and len(t["table"]) == 4
    info = s.info()
    assert info["warps_per_cta"] == t["best"]["warps"]
    orc = oracle.OracleScene(sc)
    res = srv.ServingBatcher(s, config_quantum=512, edge_quantum=512).step(reqs)
    _check(orc, reqs, res)


def test_mismatched_edges_rejected(gpu):
    scenes, col, srv = pkg("scenes"), pkg("collision"), pkg("serving")
    sc = scenes.make_arm_scene(0)
    b = srv.ServingBatcher(col.Gb300Scene(sc))
    with pytest.raises(ValueError):
        b.step([dict(q1=np.zeros((3, 28), np.float32), q2=np.zeros((2, 28), np.float32))])
    with pytest.raises(ValueError):
        b.step([dict(q1=np.zeros((3, 28), np.float32), q2=np.zeros((3, 28), np.float32), N=[5, 5])])


def test_zero_copy_prepare_submit(gpu, oracle):
    """Requests written straight into the staging views give the same
    verdicts as the copying path."""
    scenes, col, srv = pkg("scenes"), pkg("collision"), pkg("serving")
    sc = scenes.make_mobile_scene(0)
    s = col.Gb300Scene(sc)
    orc = oracle.OracleScene(sc)
    b = srv.ServingBatcher(s, config_quantum=1024, edge_quantum=256)
    reqs = _requests(sc, 5, n=4)
    slots = b.prepare([(len(r["configs"]), len(r["q1"])) for r in reqs])
    for k, r in enumerate(reqs):
        slots.configs[k][:] = r["configs"]
        slots.q1[k][:] = r["q1"]
        slots.q2[k][:] = r["q2"]
        slots.N[k][:] = r["N"]
    res = b.submit(slots)
    _check(orc, reqs, res)
    res2 = b.step(reqs)
    for a, c in zip(res.config_free + res.edge_free, res2.config_free + res2.edge_free):
        assert np.array_equal(a, c)


def test_direct_gather_and_packed_steps_agree(gpu, oracle):
    """The direct step (the graph's first launch reads the requests' host
    arrays through the address table) and the packed step (host packing into
    pinned staging) give the oracle's verdicts, also with float64, strided
    and empty requests and edges without step counts."""
    import ctypes

    scenes, col, srv, lib = pkg("scenes"), pkg("collision"), pkg("serving"), pkg("_lib")
    v = ctypes.c_int32(0)
    lib.check(lib.load().mrmg_host_access(ctypes.byref(v)))
    if not v.value:
        pytest.skip("the device does not read pageable host memory")
    sc = scenes.make_mobile_scene(0)
    s = col.Gb300Scene(sc)
    orc = oracle.OracleScene(sc)
    b = srv.ServingBatcher(s, config_quantum=1024, edge_quantum=256)
    assert b.direct
    for seed in range(3):
        reqs = _requests(sc, 40 + seed)
        reqs[0] = dict(configs=reqs[0]["configs"].astype(np.float64), q1=reqs[0]["q1"], q2=reqs[0]["q2"],
                       N=reqs[0]["N"])
        reqs[2] = dict(configs=np.asfortranarray(reqs[2]["configs"]), q1=reqs[2]["q1"], q2=reqs[2]["q2"])
        reqs[3] = dict()
        d = b.step(reqs)
        p = b.step(reqs, direct=False)
        chk = [dict(r) for r in reqs]
        chk[2]["N"] = srv.edge_steps(reqs[2]["q1"], reqs[2]["q2"], 0.05)
        chk[0]["configs"] = reqs[0]["configs"].astype(np.float32)
        _check(orc, chk, d)
        for a, b_ in zip(d.config_free + d.edge_free, p.config_free + p.edge_free):
            assert np.array_equal(a, b_)
    assert any(k[2] for k in b.graphs) and any(not k[2] for k in b.graphs)


def test_direct_gather_rejects_a_bad_table(gpu):
    """A table row outside the step's capacities is refused on the device
    (error bits, ValueError) instead of copied."""
    import ctypes

    scenes, col, srv, lib = pkg("scenes"), pkg("collision"), pkg("serving"), pkg("_lib")
    v = ctypes.c_int32(0)
    lib.check(lib.load().mrmg_host_access(ctypes.byref(v)))
    if not v.value:
        pytest.skip("the device does not read pageable host memory")
    sc = scenes.make_mobile_scene(0)
    s = col.Gb300Scene(sc)
    g = srv._StepGraph(s, 1024, 256, False, direct=True, max_src=8)
    a = np.zeros((10, sc.q_dim), np.float32)
    tab = g.table.numpy()
    tab[0:8] = (1, 10, 0, 0, a.ctypes.data, 10, 1020, 0)      # rows 1020..1029 of a 1,024-row region
    with pytest.raises(ValueError):
        g.run()
    tab[0:8] = (1, 10, 0, 0, a.ctypes.data, 10, 0, 0)
    out = g.run()
    assert out.shape == (1024 + 256,)
