"""Time the REFERENCE's own Python code on the workloads of the benchmark's
CPU-runnable cases, and record the figures (with the host they ran on) in
reference_timings.json next to this script.

The reference cannot be installed on the GPU host (its build backend is not
available offline), so its own code path is timed where its checkout is,
with the import recipe of make_golden.py (numba, matplotlib and robotic
replaced by stand-ins: the reference's kernels then run as the plain Python
they are written in).  bench.py reports these figures beside its own, labelled
with the host they were measured on.

    python tests/golden/time_reference.py <reference root>

Workloads (seeded as in bench.py):
  * two discs among 10 boxes (abstract_env.py:255-354): 10,000 uniform
    configurations through is_collision_free and 1,000 uniform edges at
    resolution 0.01 through is_edge_collision_free, in one process and in a
    process pool of os.cpu_count() workers (run_experiment.py's parallelism);
  * per-mode k-NN (200,000 nodes in 16 Zipf modes, 28-D): for a sample of the
    4,096 queries, batch_config_dist (configuration.py:342-349) over the
    query's mode, then argpartition + argsort (prm_graph.py:446-447), k = 10,
    euclidean and max_euclidean; one process and a process pool.
Every verdict and index is checked against the repository's oracle.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

_REF = None
_W = {}


def _pkg(sub):
    import importlib

    return importlib.import_module(f"multirobot-pathplanning-benchmark_gb300.{sub}")


def _ref(root: str):
    global _REF
    if _REF is None:
        from make_golden import import_reference

        _REF = import_reference(Path(root))
    return _REF


def _disc_env(root):
    pe, ae, cf, reg = _ref(root)
    sc = _pkg("scenes").make_disc_scene(0)
    env = reg.get_env_by_name("abstract.test")
    env.obstacles = [ae.Rectangle(np.array(c), np.array(b)) for c, b in zip(sc.box_center, sc.box_bounds)]
    env.agent_radii = [0.1, 0.1]
    return env


def _disc_inputs():
    rng = np.random.default_rng(0)
    q = rng.uniform(-1, 1, (10_000, 4))
    q1, q2 = rng.uniform(-1, 1, (1000, 4)), rng.uniform(-1, 1, (1000, 4))
    return q, q1, q2


# --- pool workers (each builds its own env, as run_experiment's processes do)
def _init_worker(root):
    _W["env"] = _disc_env(root)
    _W["root"] = root


def _cfg_chunk(rows):
    env = _W["env"]
    return [bool(env.is_collision_free(env.start_pos.from_flat(r), None)) for r in rows]


def _edge_chunk(pairs):
    env = _W["env"]
    S = env.start_pos.from_flat
    return [bool(env.is_edge_collision_free(S(a), S(b), None, resolution=0.01)) for a, b in pairs]


def _knn_init(root, metric):
    _W["cf"] = _ref(root)[2]
    w = _pkg("scenes").make_knn_workload(seed=0)
    _W["w"], _W["metric"] = w, metric
    sl = [tuple(map(int, s)) for s in w["slices"]]
    off = w["mode_offsets"]
    S = _W["cf"].NpConfiguration
    _W["nodes"] = [w["nodes"][off[m]:off[m + 1]] for m in range(len(off) - 1)]
    _W["mk"] = lambda x: S(np.asarray(x, dtype=np.float64), sl)


def _knn_one(qi):
    w, cf = _W["w"], _W["cf"]
    m = int(w["q_mode"][qi])
    d = cf.batch_config_dist(_W["mk"](w["queries"][qi]), _W["nodes"][m], _W["metric"])
    k = w["k"]
    part = np.argpartition(d, k - 1)[:k]
    return part[np.argsort(d[part])].tolist()


def _timed(fn):
    t0 = time.perf_counter()
    out = fn()
    return out, time.perf_counter() - t0


def main(root: str):
    import oracle

    oracle.build()
    P = os.cpu_count() or 1
    res = {"host": {"cpu": platform.processor() or platform.machine(), "cpu_count": P,
                    "python": platform.python_version(), "numpy": np.__version__,
                    "numba": "replaced by a stand-in: the reference's kernels run as written, in plain Python"},
           "note": "the reference's own code, timed in its checkout's container (not on the GPU host)"}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    res["host"]["cpu"] = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    q, q1, q2 = _disc_inputs()
    sc = _pkg("scenes").make_disc_scene(0)
    o = oracle.OracleScene(sc)
    ref_c, ref_e = o.configs_free(q), o.edges_free(q1, q2, 0.01)
    _init_worker(root)
    got_c, t_c = _timed(lambda: _cfg_chunk(q))
    got_e, t_e = _timed(lambda: _edge_chunk(list(zip(q1, q2))))
    assert np.array_equal(np.array(got_c, dtype=np.uint8), ref_c)
    assert np.array_equal(np.array(got_e, dtype=np.uint8), ref_e)
    ctx = mp.get_context("spawn")
    with ctx.Pool(P, initializer=_init_worker, initargs=(root,)) as pool:
        pool.map(_cfg_chunk, np.array_split(q[:64], P))      # warm the workers
        pc, tpc = _timed(lambda: sum(pool.map(_cfg_chunk, np.array_split(q, 4 * P)), []))
        pe, tpe = _timed(lambda: sum(pool.map(_edge_chunk, np.array_split(np.stack([q1, q2], 1), 4 * P)), []))
    assert np.array_equal(np.array(pc, dtype=np.uint8), ref_c)
    assert np.array_equal(np.array(pe, dtype=np.uint8), ref_e)
    res["disc_two_agents"] = {
        "workload": "2 discs r 0.1, 10 boxes; 10,000 uniform configurations; 1,000 uniform edges at 0.01",
        "configs_per_s_1proc": len(q) / t_c, "edges_per_s_1proc": len(q1) / t_e,
        "configs_per_s_pool": len(q) / tpc, "edges_per_s_pool": len(q1) / tpe, "pool_processes": P,
        "api": "AbstractEnvironment.is_collision_free / is_edge_collision_free (abstract_env.py:255-354)"}
    w = _pkg("scenes").make_knn_workload(seed=0)
    n_sample = 32
    res["knn"] = {"workload": "200,000 nodes in 28-D, 16 Zipf modes, k = 10; a sample of the 4,096 queries",
                  "api": "batch_config_dist (configuration.py:342-349) + argpartition/argsort (prm_graph.py:446-447)"}
    for metric in ("euclidean", "max_euclidean"):
        _knn_init(root, metric)
        oi, _ = oracle.knn(w["queries"][:n_sample], w["q_mode"][:n_sample], w["nodes"], w["mode_offsets"],
                           w["slices"], metric, w["k"])
        got, t1 = _timed(lambda: [_knn_one(i) for i in range(n_sample)])
        assert np.array_equal(np.array(got), oi), metric
        with ctx.Pool(P, initializer=_knn_init, initargs=(root, metric)) as pool:
            pool.map(_knn_one, range(P))
            pg, tp = _timed(lambda: pool.map(_knn_one, range(4 * P)))
        res["knn"][metric] = {"queries_per_s_1proc": n_sample / t1, "queries_sampled_1proc": n_sample,
                              "queries_per_s_pool": 4 * P / tp, "queries_sampled_pool": 4 * P,
                              "indices_equal_oracle": True}
    (HERE / "reference_timings.json").write_text(json.dumps(res, indent=1))
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: time_reference.py <reference root>")
    main(sys.argv[1])
