#!/usr/bin/env python3
"""Edge checks per second at 0 verdict mismatches on the four-arm scene.

Workload (one step): 100,000 edges of four serial 7-DoF DH arms (168 collision
spheres, 10,584 inter-robot sphere pairs) among 50 boxes; step counts
lognormal (median 40, sigma 0.6) clipped to 5..500 at resolution 0.05 rad;
FP32 endpoints.  Synthetic, seeded (the reference publishes no dataset).

Reported (one JSON line on rank 0):
  value      batched, graph-captured edge check with inputs resident in HBM
  e2e        the same through the public env API from pinned host buffers
             (host->device copy of the endpoints and device->host copy of the
             verdicts inside every timed step)
  plain      one launch per is_edge_collision_free call (extra key)
  roofline   the first-pass edge kernel in full-evaluation mode (every
             interpolated configuration and every sphere pair, no early exit)
             against the measured FP32 FMA peak
  cpu_baseline  the CPU FP64 restatement (OpenMP, all host cores)
Every run compares all verdicts with the CPU oracle and reports mismatches.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
PKG = "multirobot-pathplanning-benchmark_gb300"

METRIC = "edge checks/sec at 0 verdict mismatches: batched vs plain GPU vs host-CPU ref"
UNIT = "edges/s"
RESOLUTION = 0.05
N_EDGES = 100_000
E2E_DEPTH = 4          # edge-check plans in flight in the end-to-end measurement


def pkg(sub=None):
    return importlib.import_module(PKG if sub is None else f"{PKG}.{sub}")


def oracle_mod():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    oracle.build()
    return oracle


def workload(rank: int):
    scenes = pkg("scenes")
    scene = scenes.make_arm_scene(0)
    N = scenes.lognormal_steps(N_EDGES, 7 + 1000 * rank)
    q1, q2 = scenes.edges_with_steps(scene, N, RESOLUTION, 11 + 1000 * rank)
    return scene, q1, q2, N


def config_flops(scene) -> int:
    """Algorithmic FP32 flops of one full configuration evaluation, counted
    as the work-unit table of the hot path fixes them: 63 per DH link
    composition, 18 per sphere centre, 9 per sphere-box test and 9 per
    inter-robot sphere pair test (four arms: 28 x 63 + 168 x 18 + 8,400 x 9 +
    10,584 x 9 = 175,644)."""
    links = int(np.sum(scene.n_links))
    S = len(scene.sphere_radius)
    B = len(scene.box_lo)
    counts = np.bincount(scene.sphere_robot, minlength=scene.n_robots)
    pairs = int((counts.sum() ** 2 - (counts ** 2).sum()) // 2)
    return 63 * links + 18 * S + 9 * S * B + 9 * pairs


def config_ops_with_compares(scene) -> int:
    """The same work with the clamps and compares counted as operations too
    (15 per sphere-box test, 11 per sphere pair): a second, labelled figure,
    not the roofline numerator."""
    links = int(np.sum(scene.n_links))
    S = len(scene.sphere_radius)
    B = len(scene.box_lo)
    counts = np.bincount(scene.sphere_robot, minlength=scene.n_robots)
    pairs = int((counts.sum() ** 2 - (counts ** 2).sum()) // 2)
    return 63 * links + 18 * S + 15 * S * B + 11 * pairs


WORKLOAD_DESC = ("four 7-DoF DH arms on a 1.2 m table (168 spheres r 0.03-0.07 m, 10,584 inter-robot pairs), "
                 "50 boxes; 100,000 edges/step, step counts lognormal(median 40, sigma 0.6) clipped 5..500 at "
                 "0.05 rad; FP32 endpoints, FP64 interpolation")


# ---------------------------------------------------------------------------
class ClockSampler:
    """SM clocks, power and throttle reasons sampled every ~200 ms while a run
    is under way: a thread runs one-shot `nvidia-smi --query-gpu` calls (a
    looping nvidia-smi writing to a file buffers its output and loses it when
    stopped).  The GPU is named by its UUID when torch reports one, so the
    sample is of the device this process uses."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index: int, period_s: float = 0.2):
        import threading

        self.gpu = str(index)
        try:
            import torch

            u = getattr(torch.cuda.get_device_properties(index), "uuid", None)
            if u is not None:
                u = str(u)
                self.gpu = u if u.startswith("GPU-") else f"GPU-{u}"
        except Exception:
            pass
        self.rows, self.errors = [], []
        self.period = period_s
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._loop, daemon=True)
        self._t.start()

    def _query(self):
        r = subprocess.run(["nvidia-smi", "-i", self.gpu, f"--query-gpu={self.FIELDS}",
                            "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) != 7:
                continue
            try:
                self.rows.append((float(p[0]), float(p[1]), float(p[2]), p[3:]))
            except ValueError:
                continue
        if r.returncode != 0 and not self.errors:
            self.errors.append((r.stderr or r.stdout).strip()[:200])

    def _loop(self):
        while not self._stop.is_set():
            try:
                self._query()
            except Exception as e:   # nvidia-smi missing or hung: report, keep the run going
                self.errors.append(repr(e)[:200])
                return
            self._stop.wait(self.period)

    def stop(self) -> dict:
        self._stop.set()
        self._t.join(timeout=15)
        rows = list(self.rows)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                    "errors": self.errors[:1]}
        pmin = min(r[2] for r in rows)
        load = [r for r in rows if r[2] > pmin * 1.15] or rows
        reasons = sorted({self.NAMES[i] for r in load for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in load])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "samples_under_load": len(load),
                "power_w_max": max(r[2] for r in rows),
                "window": "the whole run (headline steps, end-to-end steps and the extra workloads)"}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x: float, world: int) -> float:
    """Max over ranks (the slowest replica sets the job's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---------------------------------------------------------------------------
def cpu_baseline(orc, scene, q1, q2, budget_s: float = 12.0, max_passes: int = 200) -> dict:
    o = orc.OracleScene(scene)
    a, b = np.asarray(q1, np.float64), np.asarray(q2, np.float64)
    o.edges_free(a[:2000], b[:2000], RESOLUTION)   # warm caches / thread pool
    t0 = time.perf_counter()
    passes = 0
    while True:
        o.edges_free(a, b, RESOLUTION)
        passes += 1
        if time.perf_counter() - t0 >= budget_s or passes >= max_passes:
            break
    dt = time.perf_counter() - t0
    return {"value": passes * len(a) / dt, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
            "sample": f"{passes} passes over the 100,000-edge workload ({dt:.1f} s), oracle/oracle.c FP64 "
                      f"restatement, OpenMP {orc.num_threads()} threads, {os.cpu_count()} host cores"}


def bench_config(world: int, n: int) -> dict:
    """The workload's `config`, identical in both arms of the benchmark."""
    return {"workload": WORKLOAD_DESC, "edges_per_step": n, "edges_total": n * world,
            "l2": "GPU arm: flushed between timed steps (256 MB write outside the timed events)",
            "parallelism": f"replicas x{world}",
            "fk_parity": "the four arms' kinematics (standard DH) are defined by this library and checked against "
                         "the oracle's C restatement; the reference delegates robots to external engines"}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    orc = oracle_mod()
    scene, q1, q2, N = workload(0)
    o = orc.OracleScene(scene)
    a, b = np.asarray(q1, np.float64), np.asarray(q2, np.float64)
    for _ in range(args.warmup):
        o.edges_free(a, b, RESOLUTION)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.edges_free(a, b, RESOLUTION)
    dt = time.perf_counter() - t0
    v = args.steps * len(a) / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(world, len(a)),
        "form": f"CPU FP64 restatement (oracle/oracle.c), OpenMP {orc.num_threads()} threads on rank 0",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
                         "sample": f"each step: the full 100,000-edge workload on the CPU FP64 restatement "
                                   f"(oracle/oracle.c), OpenMP {orc.num_threads()} threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    _lib, envm = pkg("_lib"), pkg("env")
    orc = oracle_mod()

    clocks = ClockSampler(dev.index) if rank == 0 else None
    scene, q1, q2, N = workload(rank)
    n = len(q1)
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=RESOLUTION)
    sc = env._gb300
    o = orc.OracleScene(scene)
    ref = o.edges_free(q1, q2, RESOLUTION)

    s = torch.cuda.Stream(device=dev)
    q1_d = torch.from_numpy(q1).to(dev)
    q2_d = torch.from_numpy(q2).to(dev)
    out_d = torch.empty(n, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2

    # correctness of the plain call and reservation of the call's scratch
    with torch.cuda.stream(s):
        sc.is_edge_collision_free_batch(q1_d, q2_d, RESOLUTION, out=out_d, stream=s)
    mism = int((out_d.cpu().numpy() != ref).sum())
    early_stats = sc.last_call_stats()

    # launch and work-shape autotuning (CTAs/SM x warps, obstacle tile, box
    # head, phase-B1 depth) on a separately drawn sample of the same
    # distribution; verdicts never depend on it (checked again after timing)
    tune = None
    if not args.no_tune:
        scn = pkg("scenes")
        Nt = scn.lognormal_steps(N_EDGES, 99 + 1000 * rank)
        t1, t2 = scn.edges_with_steps(scene, Nt, RESOLUTION, 98 + 1000 * rank)
        r = pkg("autotune").autotune(sc, t1, t2, None, RESOLUTION, repeats=3)
        tune = {"best": r["best"], "default_ms": r["default_ms"], "best_ms": r["best_ms"], "trials": len(r["table"]),
                "sample": "100,000 edges of the same distribution, other seeds"}

    def capture(flags):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            sc.is_edge_collision_free_batch(q1_d, q2_d, RESOLUTION, out=out_d, stream=s, flags=flags)
        return g

    g = capture(_lib.MRMG_FLAG_ASYNC)
    with torch.cuda.stream(s):
        for _ in range(args.warmup):
            flush.zero_()
            g.replay()
    s.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    with torch.cuda.stream(s):
        for e0, e1 in evs:
            flush.zero_()
            e0.record(s)
            g.replay()
            e1.record(s)
    s.synchronize()
    t_wall = time.perf_counter() - t_wall0
    torch.cuda.synchronize()
    barrier(world)
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = reduce_max(float(np.sum(step_ms)), world)
    value = world * n * args.steps / (total_ms * 1e-3)
    mism += int((out_d.cpu().numpy() != ref).sum())

    # ---- end to end through the public API: a graph-captured edge-check plan
    # (pinned host buffers; every step copies the endpoints host->device in
    # chunks overlapped with the checks and reads the verdicts back)
    plan = env.edge_check_plan(n, chunks=args.chunks, dtype=torch.float32)   # the workload's FP32 endpoints
    plan.q1_host[:] = q1
    plan.q2_host[:] = q2
    for _ in range(args.warmup):
        plan.run()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vh = plan.run()
    e2e_serial_s = reduce_max(time.perf_counter() - t0, world)
    e2e_serial = world * n * args.steps / e2e_serial_s
    mism += int((vh != ref).sum())

    # the same with E2E_DEPTH plans in flight: later steps' endpoints cross to
    # the device while earlier steps' checks run, and independent steps
    # overlap each other's kernel tails (every step still copies its own
    # inputs and reads its own verdicts back inside the timed region)
    pipe = env.edge_check_pipeline(n, depth=E2E_DEPTH, dtype=torch.float32)
    for p in pipe.plans:
        p.q1_host[:] = q1
        p.q2_host[:] = q2
    for _ in range(args.warmup):
        pipe.result(pipe.submit())
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    inflight = []
    for _ in range(args.steps):
        if len(inflight) == pipe.depth:
            vh = pipe.result(inflight.pop(0))
        inflight.append(pipe.submit())
    for slot in inflight:
        vh = pipe.result(slot)
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    e2e = world * n * args.steps / e2e_s
    mism += int((vh != ref).sum())

    # the plain batched call from pinned torch tensors (no plan), for comparison
    q1_h = torch.from_numpy(q1).pin_memory()
    q2_h = torch.from_numpy(q2).pin_memory()
    for _ in range(args.warmup):
        env.batch_is_edge_collision_free(q1_h, q2_h).cpu()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ncall = max(10, args.steps // 10)
    for _ in range(ncall):
        vc = env.batch_is_edge_collision_free(q1_h, q2_h).cpu()
    call_e2e = n * ncall / (time.perf_counter() - t0)
    mism += int((vc.numpy().astype(np.uint8) != ref).sum())

    # the same call on the caller's numpy arrays: the kernels read the
    # endpoints in place from host memory where the device reads pageable
    # memory (GB300), the verdicts come back in one copy
    for _ in range(args.warmup):
        env.batch_is_edge_collision_free(q1, q2)
    t0 = time.perf_counter()
    for _ in range(ncall):
        vn = env.batch_is_edge_collision_free(q1, q2)
    host_e2e = n * ncall / (time.perf_counter() - t0)
    mism += int((vn.astype(np.uint8) != ref).sum())

    extra = {}
    if rank == 0:
        # ---- plain: one launch (and one host round trip) per edge
        m = min(n, args.plain_edges)
        env.is_edge_collision_free(q1[0], q2[0], None)
        t0 = time.perf_counter()
        plain_v = [env.is_edge_collision_free(q1[i], q2[i], None) for i in range(m)]
        plain = m / (time.perf_counter() - t0)
        mism += int((np.array(plain_v, dtype=np.uint8) != ref[:m]).sum())
        # one is_collision_free call per configuration (the sampler's pattern)
        qc = np.asarray(q1[:m], np.float64)
        ref_c = o.configs_free(qc)
        env.is_collision_free(qc[0], None)
        t0 = time.perf_counter()
        plain_c = [env.is_collision_free(qc[i], None) for i in range(m)]
        plain_cfg = m / (time.perf_counter() - t0)
        mism += int((np.array(plain_c, dtype=np.uint8) != ref_c).sum())

        # ---- roofline: first-pass kernel in full-evaluation mode
        full_flags = _lib.MRMG_FLAG_ASYNC | _lib.MRMG_FLAG_FULL_EVAL
        with torch.cuda.stream(s):
            sc.is_edge_collision_free_batch(q1_d, q2_d, RESOLUTION, out=out_d, stream=s,
                                            flags=_lib.MRMG_FLAG_FULL_EVAL)
        cfgs = sc.last_call_stats()["configs_evaluated"]
        full_mism = int((out_d.cpu().numpy() != ref).sum())
        gf = capture(full_flags)
        with torch.cuda.stream(s):
            gf.replay()
            fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
            for a, b in fev:
                a.record(s)
                gf.replay()
                b.record(s)
        s.synchronize()
        full_ms = float(np.mean([a.elapsed_time(b) for a, b in fev]))
        F1 = config_flops(scene)
        F1c = config_ops_with_compares(scene)
        achieved = cfgs * F1 / (full_ms * 1e-3) / 1e12
        peak = _measure_fp32_peak(_lib)
        traffic = _profile_traffic()
        extra = dict(
            plain={"value": plain, "unit": UNIT, "edges_sampled": m, "us_per_call": 1e6 / plain,
                   "form": "env.is_edge_collision_free per edge: one call, one host round trip"},
            plain_configs={"value": plain_cfg, "unit": "configs/s", "configs_sampled": m,
                           "us_per_call": 1e6 / plain_cfg,
                           "form": "env.is_collision_free per configuration: one call, one host round trip"},
            batched_over_plain=value / plain,
            roofline={"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                      "frac": achieved / peak, "traffic": traffic,
                      "kernel": "first pass (arm_edges_kernel phase A + arm_edges_phase_b), full-evaluation mode",
                      "algorithmic": f"{cfgs} configurations x {F1} flops per launch (per configuration: 28 DH "
                                     f"links x 63 + 168 sphere centres x 18 + 8,400 sphere-box tests x 9 + 10,584 "
                                     f"sphere pairs x 9)",
                      "ms_per_launch": full_ms,
                      "frac_with_compares": cfgs * F1c / (full_ms * 1e-3) / 1e12 / peak,
                      "with_compares": f"{F1c} operations per configuration when the clamps and compares count "
                                       "(15 per sphere-box test, 11 per pair)",
                      "peak_source": "measured FP32 FFMA microbenchmark (mrmg_microbench_fma) in this run; "
                                     "MEASURED_PEAKS.json holds HBM and BF16 only"},
            full_eval_mismatches=full_mism,
            workload_stats={"free_edges": int(ref.sum()), "mean_steps": float(N.mean()),
                            "configs_evaluated_early_exit": early_stats["configs_evaluated"],
                            "configs_rechecked_fp64": early_stats["rechecked_fp64"],
                            "configs_full_evaluation": cfgs},
        )
        if world == 1:
            extra["cpu_baseline"] = cpu_baseline(orc, scene, q1, q2, budget_s=args.cpu_seconds)
            if not args.skip_extra:
                extra["knn"] = bench_knn(orc)
                extra["penetration"] = bench_penetration()
                extra["serving"] = bench_serving(orc)
                extra["prm_lazy"] = bench_prm_lazy()
                extra["abstract"] = bench_abstract(orc)
                extra["sparse_scene"] = bench_sparse_edges(orc)

    mism = int(reduce_max(float(mism), world))
    clk = clocks.stop() if clocks is not None else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": bench_config(world, n),
            "form": "batched, CUDA-graph captured (counter reset, phase A, phase B1, phase B2 + finalize, FP64 "
                    "re-check pass, status copy)",
            "verdict_mismatches": mism,
            "clocks": clk,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(q1.nbytes + q2.nbytes),
                    "d2h_bytes_per_step": int(n),
                    "api": f"Gb300ArmEnvironment.edge_check_pipeline(n, depth={E2E_DEPTH}): one CUDA graph per "
                           f"step (endpoints host->device, checks, verdicts device->host), {E2E_DEPTH} steps in "
                           "flight"},
            "e2e_serial": {"value": e2e_serial, "unit": UNIT,
                           "api": f"Gb300ArmEnvironment.edge_check_plan(n).run(): one step at a time, "
                                  f"{args.chunks} pipelined chunks"},
            "e2e_host_arrays": {"value": host_e2e, "unit": UNIT,
                                "api": "Gb300ArmEnvironment.batch_is_edge_collision_free(numpy arrays): one call per "
                                       "step, endpoints read in place from host memory (pageable access), verdicts "
                                       "copied back"},
            "e2e_batch_call": {"value": call_e2e, "unit": UNIT,
                               "api": "Gb300ArmEnvironment.batch_is_edge_collision_free(pinned tensors)"},
            "gpu_launches": 4 * args.steps,
            "wall_s_timed": t_wall,
            "autotune": tune,
        }
        line.update(extra)
        line["summary"] = _summary(line)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0 if mism == 0 else 3


def bench_knn(orc, steps: int = 20) -> dict:
    """Per-mode k-NN on the 200k-node / 16-mode / 4,096-query workload, k = 10,
    euclidean and max_euclidean: device time of the full query batch (inputs
    resident), indices checked against the oracle, CPU oracle on a sample."""
    import torch

    knn, scenes = pkg("knn"), pkg("scenes")
    w = scenes.make_knn_workload(seed=0)
    sizes = np.diff(w["mode_offsets"])
    pairs = int(sizes[w["q_mode"]].sum())
    qs = torch.from_numpy(w["queries"]).cuda()
    out = {"workload": "200,000 nodes in 28-D (64 Gaussian clusters, sigma 0.3), 16 modes with Zipf(1.1) sizes, "
                       "4,096 uniform queries, k = 10", "pairs_per_batch": pairs}
    for metric in ["euclidean", "max_euclidean"]:
        store = knn.NodeStore(w["nodes"], w["mode_offsets"], w["slices"], metric)
        idx, dist = store.knn(qs, w["q_mode"], w["k"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            idx, dist = store.knn(qs, w["q_mode"], w["k"])
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
        oi, od = orc.knn(w["queries"], w["q_mode"], w["nodes"], w["mode_offsets"], w["slices"], metric, w["k"])
        mism = int((idx.cpu().numpy() != oi).sum())
        # CPU: the oracle on a 256-query sample, scaled
        sub = slice(0, 256)
        t1 = time.perf_counter()
        orc.knn(w["queries"][sub], w["q_mode"][sub], w["nodes"], w["mode_offsets"], w["slices"], metric, w["k"])
        cpu_s = (time.perf_counter() - t1) * len(w["queries"]) / 256
        issued = 2 * (96 if metric == "euclidean" else 128) * pairs
        alg = 2 * 32 * pairs                 # K = 28 padded to 32 (four 8-wide agent blocks for max over agents)
        node_bytes = w["nodes"].shape[0] * w["nodes"].shape[1] * 4
        peaks = _peaks()
        out[metric] = {"queries_per_s": len(w["queries"]) / dt, "ms_per_batch": 1e3 * dt, "index_mismatches": mism,
                       "tensor_core": store.last_stats.get("tensor_core"),
                       "rerun_exact": store.last_stats.get("rerun_exact"),
                       "gemm_tflops_issued": issued / dt / 1e12,
                       "roofline": {"bound": "tensor", "achieved": alg / dt / 1e12, "peak": peaks["bf16_tflops"],
                                    "unit": "TFLOP/s", "frac": alg / dt / 1e12 / peaks["bf16_tflops"],
                                    "algorithmic": f"2 x 32 x {pairs} query-node pairs per batch (K = 28 padded "
                                                   f"to 32)",
                                    "issued_frac": issued / dt / 1e12 / peaks["bf16_tflops"],
                                    "issued": f"split-BF16 operands: K = {96 if metric == 'euclidean' else 128} "
                                              f"per pair on the tensor pipe",
                                    "hbm_achieved_gbs": node_bytes / dt / 1e9, "hbm_peak_gbs": peaks["hbm_gbs"],
                                    "hbm_frac": node_bytes / dt / 1e9 / peaks["hbm_gbs"],
                                    "hbm_bytes": f"{node_bytes} B: the nodes once in FP32",
                                    "peak_source": peaks["source"],
                                    "timing": "host wall clock per synchronous batch call (inputs resident)"},
                       "cpu_queries_per_s": len(w["queries"]) / cpu_s, "cpu_cores": orc.num_threads()}
        # radius queries: each query's radius is its 16th-nearest distance
        _, d16 = store.knn(qs, w["q_mode"], 16)
        r = d16[:, -1].cpu().numpy()
        r = np.where(np.isfinite(r), r, 0.0)
        offs, nidx, ndist = store.near(qs, w["q_mode"], r)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            offs, nidx, ndist = store.near(qs, w["q_mode"], r)
        torch.cuda.synchronize()
        dtn = (time.perf_counter() - t0) / steps
        so = orc.near(w["queries"][sub], w["q_mode"][sub], w["nodes"], w["mode_offsets"], w["slices"], metric, r[sub])
        o = offs.cpu().numpy()
        ok = np.array_equal(o[:257] - o[0], so[0]) and np.array_equal(nidx[:int(o[256])].cpu().numpy(), so[1])
        out[metric]["near"] = {"queries_per_s": len(w["queries"]) / dtn, "ms_per_batch": 1e3 * dtn,
                               "neighbours": int(o[-1]), "sample_256_identical": bool(ok)}
        store.close()
    out["rrt_loop"] = bench_rrt_loop(w)
    out["cpu_baseline_reference_python"] = _ref_block("knn")
    return out


def _ref_block(key: str):
    rt = _reference_timings()
    if not rt or key not in rt:
        return None
    return {**rt[key], "where": rt["where"], "numba": rt["host"].get("numba")}


def bench_rrt_loop(w, iters: int = 2000) -> dict:
    """The RRT* inner loop on a node store that already holds the 200k-node
    workload: per iteration one nearest query (k = 1), one radius query and
    one single-row append, each a synchronous library call from host arrays."""
    knn = pkg("knn")
    store = knn.NodeStore(w["nodes"], w["mode_offsets"], w["slices"], "euclidean")
    rng = np.random.default_rng(1)
    qs = rng.uniform(-np.pi, np.pi, (iters, w["nodes"].shape[1]))
    modes = rng.integers(0, len(w["mode_offsets"]) - 1, iters).astype(np.int32)
    for i in range(20):
        store.knn(qs[i:i + 1], modes[i:i + 1], 1)
        store.near(qs[i:i + 1], modes[i:i + 1], 0.5)
    t = {"nearest": 0.0, "near": 0.0, "append": 0.0}
    n0 = sum(store.size(m) for m in range(store.n_modes))
    for i in range(iters):
        q, m = qs[i:i + 1], modes[i:i + 1]
        t0 = time.perf_counter()
        idx, dist = store.knn(q, m, 1)
        t1 = time.perf_counter()
        store.near(q, m, 0.5)
        t2 = time.perf_counter()
        store.append(int(m[0]), q)
        t3 = time.perf_counter()
        t["nearest"] += t1 - t0
        t["near"] += t2 - t1
        t["append"] += t3 - t2
    grown = sum(store.size(m) for m in range(store.n_modes)) - n0
    store.close()
    return {"iterations": iters, "nodes_appended": grown,
            **{f"{k}_us": 1e6 * v / iters for k, v in t.items()}}


def bench_penetration(steps: int = 10) -> dict:
    """Path-penetration cost and gradient on 512 paths x 256 waypoints x 28
    joints (four-arm scene; straight lines between collision-free endpoints
    plus N(0, 0.05^2) noise): device time of the cost, the gradient and both
    in one launch (inputs resident), accuracy against the float64 oracle on
    two sampled paths, the MUFU roofline, and the float64 torch-autograd CPU
    path on a sample."""
    import torch

    pen, col, scenes, _lib = pkg("penetration"), pkg("collision"), pkg("scenes"), pkg("_lib")
    sys.path.insert(0, str(ROOT / "oracle"))
    import penetration_f64 as orc_pen

    sc = scenes.make_arm_scene(0)
    s = col.Gb300Scene(sc)
    paths = scenes.make_path_workload(sc, seed=0, is_free=lambda q: s.is_collision_free_batch(q).cpu().numpy())
    w = torch.from_numpy(paths).cuda()
    P, T, D = w.shape
    S, B = len(sc.sphere_radius), len(sc.box_lo)
    counts = np.bincount(sc.sphere_robot, minlength=sc.n_robots)
    n_pairs = S * B + int((counts.sum() ** 2 - (counts ** 2).sum()) // 2)
    out = {"workload": f"{P} paths x {T} waypoints x {D} joints, four-arm scene ({S} spheres, {B} boxes, "
                       f"{n_pairs} pairs per waypoint); margin 0.02, scale 0.02, beta 1, smoothness 0.1",
           "pairs_per_waypoint": n_pairs}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(**kw):
        for _ in range(3):
            pen.path_penetration(s, w, **kw)
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(steps):
            pen.path_penetration(s, w, **kw)
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / steps

    ms_cost = timed(cost=True)
    ms_grad = timed(cost=False, grad=True)
    ms_both = timed(cost=True, grad=True)
    res = pen.path_penetration(s, w, cost=True, grad=True)
    errs = []
    for p in (0, P // 2):
        c_ref, g_ref = orc_pen.penetration_grad(sc.arrays(), paths[p:p + 1])
        g = res["grad"][p].cpu().numpy().astype(np.float64)
        errs.append({"path": p, "cost_rel_err": float(abs(res["cost"][p].item() - c_ref[0]) / abs(c_ref[0])),
                     "grad_rel_err": float(np.linalg.norm(g - g_ref[0]) / np.linalg.norm(g_ref[0]))})
    # MUFU operations per pair of the cost kernel: sqrt, 2^x and log2
    import ctypes as C

    mufu = C.c_double(0)
    _lib.check(_lib.load().mrmg_microbench_fma(2, 20000, C.byref(mufu), None))
    wpts = P * T
    ach = 3.0 * n_pairs * wpts / (ms_cost * 1e-3) / 1e12
    out.update({
        "ms_cost": ms_cost, "ms_grad": ms_grad, "ms_cost_and_grad": ms_both,
        "waypoints_per_s_cost_and_grad": wpts / (ms_both * 1e-3),
        "paths_per_s_cost_and_grad": P / (ms_both * 1e-3),
        "accuracy": errs,
        "roofline_cost_kernel": {"bound": "mufu", "achieved": ach, "peak": mufu.value, "unit": "Tops/s",
                                 "frac": ach / mufu.value,
                                 "algorithmic": f"{wpts} waypoints x {n_pairs} pairs x 3 MUFU ops per launch",
                                 "peak_source": "measured ex2.approx microbenchmark (mrmg_microbench_fma precision 2)"},
    })
    # CPU: float64 torch autograd (cost + gradient), all threads, on 2 paths
    n_cpu = 2
    t0 = time.perf_counter()
    orc_pen.penetration_grad(sc.arrays(), paths[:n_cpu])
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": n_cpu * T / cpu_s, "unit": "waypoints/s (cost + gradient)",
                           "cores": torch.get_num_threads(), "kind": "port",
                           "sample": f"{n_cpu} paths x {T} waypoints, float64 torch autograd on the host"}
    s.close()
    return out


def bench_sparse_edges(orc, n: int = 100_000, reps: int = 10) -> dict:
    """The same four arms among 5 boxes, 100,000 edges of up to 0.3 rad per
    joint between collision-free configurations at resolution 0.02: most
    edges are free, so every interpolated position is evaluated (the headline
    scene mostly stops at the first position).  Batched call with inputs
    resident, CUDA events per call, L2 flushed; verdicts against the oracle;
    the oracle's rate on the host cores beside."""
    import torch

    scenes, envm = pkg("scenes"), pkg("env")
    scene = scenes.make_arm_scene(1, n_boxes=5)
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=0.02, tune_samples=1024)
    sc = env._gb300
    q = scenes.uniform_configs(scene, 4 * n, seed=5, dtype=np.float32)
    a = q[env.batch_is_collision_free(q)][:n]
    rng = np.random.default_rng(6)
    b = (a + rng.uniform(-0.3, 0.3, a.shape)).astype(np.float32)
    a_d, b_d = torch.from_numpy(np.ascontiguousarray(a)).cuda(), torch.from_numpy(b).cuda()
    out = torch.empty(len(a), dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    sc.is_edge_collision_free_batch(a_d, b_d, 0.02, out=out)
    ref = orc.OracleScene(scene).edges_free(a, b, 0.02)
    mism = int((out.cpu().numpy() != ref).sum())
    stats = sc.last_call_stats()
    ms = []
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sc.is_edge_collision_free_batch(a_d, b_d, 0.02, out=out)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = float(np.median(ms))
    o = orc.OracleScene(scene)
    t0 = time.perf_counter()
    o.edges_free(a[:20_000], b[:20_000], 0.02)
    cpu = 20_000 / (time.perf_counter() - t0)
    F1 = config_flops(scene)
    return {"workload": f"{len(a)} edges between free configurations of the four arms among 5 boxes, <= 0.3 rad "
                        "per joint, resolution 0.02", "free_edges": int(ref.sum()),
            "configs_evaluated": stats["configs_evaluated"], "ms_per_call": t,
            "edges_per_s": len(a) / (t * 1e-3), "configs_per_s": stats["configs_evaluated"] / (t * 1e-3),
            "effective_tflops": stats["configs_evaluated"] * F1 / (t * 1e-3) / 1e12,
            "effective_note": f"{F1} flops per configuration of this scene (5 boxes), early exit on",
            "verdict_mismatches": mism, "cpu_edges_per_s": cpu, "cpu_cores": orc.num_threads(),
            "timing": "synchronous batched call, CUDA events, L2 flushed before each call"}


def bench_abstract(orc, reps: int = 20) -> dict:
    """The two-disc abstract scene (radius 0.1, 10 boxes; the reference's
    CPU-runnable case): 10,000 uniform configurations, 1,000 uniform edges at
    resolution 0.01 and the 1,000 x 10,000 euclidean distance matrix (FP64).
    Device time per call with inputs resident (CUDA events; L2 flushed
    before each timed matrix launch), results against the oracle, the
    oracle on the host cores beside, and the distance matrix against the
    HBM roofline (80 MB of FP64 written per launch)."""
    import torch

    col, scenes, _lib = pkg("collision"), pkg("scenes"), pkg("_lib")
    sc = scenes.make_disc_scene(0)
    s = col.Gb300Scene(sc)
    o = orc.OracleScene(sc)
    rng = np.random.default_rng(0)
    q = rng.uniform(-1, 1, (10_000, 4))
    q1, q2 = rng.uniform(-1, 1, (1000, 4)), rng.uniform(-1, 1, (1000, 4))
    qd, q1d, q2d = (torch.from_numpy(x).cuda() for x in (q, q1, q2))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(f, flush_l2=False):
        f()
        torch.cuda.synchronize()
        ms = 0.0
        for _ in range(reps):
            if flush_l2:
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            f()
            b.record()
            b.synchronize()
            ms += a.elapsed_time(b)
        return ms / reps

    v = s.is_collision_free_batch(qd)
    e = s.is_edge_collision_free_batch(q1d, q2d, 0.01)
    cfg_ms = timed(lambda: s.is_collision_free_batch(qd))
    edge_ms = timed(lambda: s.is_edge_collision_free_batch(q1d, q2d, 0.01))
    lib = _lib.load()
    sl = np.ascontiguousarray(sc.agent_slices, dtype=np.int64)
    out = torch.empty((1000, 10_000), dtype=torch.float64, device="cuda")

    def dmat():   # asynchronous: the events time the kernel on this stream
        _lib.check(lib.mrmg_config_dist_matrix(q1d.data_ptr(), 1000, qd.data_ptr(), 10_000, 4, sl.ctypes.data,
                                               len(sl), _lib.METRICS["euclidean"], out.data_ptr(),
                                               _lib.stream_handle(None), _lib.MRMG_FLAG_ASYNC), "dist matrix")

    mat_ms = timed(dmat, flush_l2=True)
    ref_v, ref_e = o.configs_free(q), o.edges_free(q1, q2, 0.01)

    # The same calls replayed as CUDA graphs, end to end from pinned host
    # memory (inputs host->device, the checks, verdicts device->host, one
    # graph launch and one wait per call): what a caller that repeats calls
    # of one size pays once the per-call launches and the synchronous status
    # read are gone.  Host wall clock per call, median of `reps * 10` calls.
    plan = col.EdgeCheckPlan(s, 1000, 0.01, dtype=torch.float64, chunks=1)
    plan.q1_host[:] = q1
    plan.q2_host[:] = q2
    g_edges = plan.run().copy()
    st = torch.cuda.Stream()
    q_pin = torch.from_numpy(q).pin_memory()
    q_dev = torch.empty_like(qd)
    v_dev = torch.empty(len(q), dtype=torch.uint8, device="cuda")
    v_pin = torch.empty(len(q), dtype=torch.uint8).pin_memory()
    torch.cuda.synchronize()
    cfg_graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(cfg_graph, stream=st):
        q_dev.copy_(q_pin, non_blocking=True)
        s.is_collision_free_batch(q_dev, out=v_dev, stream=st, flags=_lib.MRMG_FLAG_ASYNC)
        v_pin.copy_(v_dev, non_blocking=True)

    def cfg_run():
        with torch.cuda.stream(st):
            cfg_graph.replay()
        st.synchronize()
        return v_pin.numpy()

    g_cfg = cfg_run().copy()

    def wall(f):
        ts = []
        for _ in range(reps * 10):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)) * 1e3

    edge_graph_ms, cfg_graph_ms = wall(plan.run), wall(cfg_run)
    # the host-pointer calls (numpy in, numpy verdicts out: what the env's
    # batch methods run for host arrays): inputs through mapped pinned memory,
    # one launch, one wait
    h_cfg = s.is_collision_free_host(q)
    h_edge = s.is_edge_collision_free_host(q1, q2, 0.01)
    host_cfg_ms = wall(lambda: s.is_collision_free_host(q))
    host_edge_ms = wall(lambda: s.is_edge_collision_free_host(q1, q2, 0.01))
    t0 = time.perf_counter()
    ref_d = orc.dist_matrix(q1, q, sl, "euclidean")
    cpu_mat_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.configs_free(q)
    cpu_cfg_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.edges_free(q1, q2, 0.01)
    cpu_edge_s = time.perf_counter() - t0
    import ctypes as C
    fp64 = C.c_double(0.0)
    _lib.check(lib.mrmg_microbench_fma(1, 20000, C.byref(fp64), None))
    hbm = _peaks()["hbm_gbs"]
    bytes_out = 1000 * 10_000 * 8
    # FP64 work per distance in the reference's order: 4 subtractions, 4
    # products, 3 sums, 1 square root (counted as one operation; it is an
    # instruction sequence on the FP64 pipe)
    ops = 1000 * 10_000 * 12
    return {
        "workload": "2 discs r = 0.1 in [-1, 1]^4, 10 boxes (centres U[-0.8, 0.8]^2, half extents U[0.05, 0.2]); "
                    "10,000 configurations, 1,000 edges at resolution 0.01, 1,000 x 10,000 euclidean matrix",
        "configs": {"ms_per_call": cfg_ms, "configs_per_s": 1e4 / (cfg_ms * 1e-3),
                    "mismatches": int((v.cpu().numpy() != ref_v).sum()), "cpu_configs_per_s": 1e4 / cpu_cfg_s,
                    "graph_e2e": {"ms_per_call": cfg_graph_ms, "configs_per_s": 1e4 / (cfg_graph_ms * 1e-3),
                                  "mismatches": int((g_cfg != ref_v).sum()),
                                  "h2d_bytes": int(q.nbytes), "d2h_bytes": len(q)}},
        "configs_host_call": {"ms_per_call": host_cfg_ms, "configs_per_s": 1e4 / (host_cfg_ms * 1e-3),
                              "mismatches": int((h_cfg != ref_v).sum()),
                              "api": "Gb300Scene.is_collision_free_host(numpy [10000, 4])"},
        "edges_host_call": {"ms_per_call": host_edge_ms, "edges_per_s": 1e3 / (host_edge_ms * 1e-3),
                            "mismatches": int((h_edge != ref_e).sum()),
                            "api": "Gb300Scene.is_edge_collision_free_host(numpy [1000, 4] x 2, 0.01)"},
        "edges": {"ms_per_call": edge_ms, "edges_per_s": 1e3 / (edge_ms * 1e-3),
                  "mismatches": int((e.cpu().numpy() != ref_e).sum()), "cpu_edges_per_s": 1e3 / cpu_edge_s,
                  "graph_e2e": {"ms_per_call": edge_graph_ms, "edges_per_s": 1e3 / (edge_graph_ms * 1e-3),
                                "mismatches": int((g_edges != ref_e).sum()),
                                "h2d_bytes": int(q1.nbytes + q2.nbytes), "d2h_bytes": len(q1),
                                "api": "collision.EdgeCheckPlan(scene, 1000, 0.01, dtype=float64).run()"}},
        "timing": "synchronous calls: CUDA events around one call with inputs resident (launches, the status "
                  "read and the host's return included); graph_e2e: host wall clock per graph replay and wait",
        "dist_matrix": {"ms_per_launch": mat_ms, "distances_per_s": 1e7 / (mat_ms * 1e-3),
                        "bit_identical": bool(np.array_equal(out.cpu().numpy(), ref_d)),
                        "cpu_distances_per_s": 1e7 / cpu_mat_s,
                        "roofline": {"bound": "fp64", "achieved": ops / (mat_ms * 1e-3) / 1e12,
                                     "peak": fp64.value, "unit": "TFLOP/s",
                                     "frac": ops / (mat_ms * 1e-3) / 1e12 / fp64.value,
                                     "algorithmic": "1e7 distances x 12 FP64 operations per launch (the "
                                                    "reference's order has no fused multiply-add, so a saturated "
                                                    "pipe reads 0.5 against an FMA peak)",
                                     "peak_source": "measured FP64 FMA microbenchmark (mrmg_microbench_fma "
                                                    "precision 1), FMA = 2 flops",
                                     "l2": "flushed before each launch",
                                     "hbm_achieved_gbs": bytes_out / (mat_ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm,
                                     "hbm_note": "80 MB FP64 written per launch, far below the measured copy "
                                                 "bandwidth at this duration: the FP64 pipe is the bound"}},
        "cpu_cores": orc.num_threads(), "cpu_kind": "port (oracle/oracle.c FP64, OpenMP)",
        "cpu_baseline_reference_python": _ref_block("disc_two_agents"),
    }


class _PrmNode:
    def __init__(self, i, q):
        self.id = i
        self.state = type("State", (), {"q": q, "mode": None})()
        self.whitelist, self.blacklist = set(), set()


def bench_prm_lazy(n_nodes: int = 3000, k: int = 10, window: int = 256) -> dict:
    """The composite PRM's lazy A* (prm_graph.py:552-746) on a roadmap of
    about 3,000 collision-free configurations of the four-arm scene with 5
    boxes (k = 10 nearest, node-store k-NN), edges checked at 0.05 rad: one
    device call per popped edge (the reference's call pattern) against
    speculative batches of up to 256 upcoming edges.  Edge costs and the
    heuristic (cost to the goal) are precomputed in one batched call each, so
    the timings isolate the edge checks; both searches give the same path.
    Each timing is the best of three runs."""
    lazy, scenes, envm, knn = pkg("lazy"), pkg("scenes"), pkg("env"), pkg("knn")
    scene = scenes.make_arm_scene(1, n_boxes=5)
    env = envm.Gb300ArmEnvironment(scene, collision_resolution=0.05, tune_samples=1024)
    q = scenes.uniform_configs(scene, 4 * n_nodes, seed=7, dtype=np.float64)
    q = q[env.batch_is_collision_free(q)][:n_nodes]
    q = q[:1] + 0.35 * (q - q[:1])            # a compact roadmap around the first configuration
    q = np.ascontiguousarray(q[env.batch_is_collision_free(q)])
    n = len(q)
    sl = scene.agent_slices()
    store = knn.NodeStore(q, [0, n], sl, "euclidean")
    nbr = store.knn(q, np.zeros(n, dtype=np.int32), k + 1)[0].cpu().numpy()[:, 1:]
    store.close()
    ecost = env.batch_config_cost(np.repeat(q, k, 0), q[nbr.reshape(-1)], sl).reshape(n, k)
    cost_tab = {(i, int(j)): float(ecost[i, c]) for i in range(n) for c, j in enumerate(nbr[i])}
    rows = [q[i].copy() for i in range(n)]
    row_of = {id(r): i for i, r in enumerate(rows)}

    def search(goal, w):
        hc = env.batch_config_cost(np.repeat(q[goal][None], n, 0), q, sl)
        nodes = [_PrmNode(i, rows[i]) for i in range(n)]
        checker = lazy.SpeculativeEdgeChecker(env, resolution=0.05, window=w)
        t0 = time.perf_counter()
        r = lazy.lazy_astar(nodes[0], [nodes[goal]], lambda nd: ([nodes[j] for j in nbr[nd.id]], nbr[nd.id]),
                            lambda a, b: cost_tab[(row_of[id(a)], row_of[id(b)])],
                            lambda a, ids: ecost[row_of[id(a)]], lambda nd: float(hc[nd.id]), checker)
        r["seconds"] = time.perf_counter() - t0
        return r

    goal = None
    for cand in np.argsort(-np.abs(q - q[0]).max(1))[:40]:
        r = search(int(cand), window)
        if len(r["path"]) >= 6:
            goal = int(cand)
            break
    out = {"roadmap_nodes": n, "k": k, "resolution": 0.05, "window": window, "goal_found": goal is not None}
    if goal is None:
        return out
    # best of three runs each: the searches are host-bound, so the host's
    # load on a shared machine shows in single runs
    seq = min((search(goal, 1) for _ in range(3)), key=lambda r: r["seconds"])
    bat = min((search(goal, window) for _ in range(3)), key=lambda r: r["seconds"])
    for tag, r in (("per_edge_calls", seq), ("batched", bat)):
        out[tag] = {"seconds": r["seconds"], "device_calls": r["calls"], "edges_checked": r["edges_checked"],
                    "edge_lookups": r["lookups"], "processed_edges": r["processed_edges"]}
    out["same_path"] = [nd.id for nd in seq["path"]] == [nd.id for nd in bat["path"]]
    out["path_nodes"] = len(bat["path"])
    out["speedup"] = seq["seconds"] / max(bat["seconds"], 1e-12)
    return out


def bench_serving(orc, steps: int = 24, warmup: int = 3) -> dict:
    """Serving-shaped load on eight mobile manipulators (72-D, 304 spheres,
    200 boxes): each step 64 planner instances submit 100-20,000 uniform
    configurations and 10-5,000 edges (N uniform in 5..800) each; one graph
    launch per step after the launch shape is autotuned.  Reports host
    latency p50/p99 (packing + copies + checks + split), device time, items/s,
    verdicts of two instances against the oracle, and the oracle's CPU rate."""
    import torch

    scenes, envm, srv = pkg("scenes"), pkg("env"), pkg("serving")
    sc = scenes.make_mobile_scene(0)
    env = envm.Gb300ArmEnvironment(sc)              # tunes the box test order
    s = env._gb300
    pool = [scenes.make_serving_requests(sc, seed=100 + i) for i in range(3)]
    # autotune the persistent grid on a quarter of the first step
    r0 = pool[0]
    cfg = np.concatenate([r["configs"] for r in r0[:16]])
    q1 = np.concatenate([cfg] + [r["q1"] for r in r0[:16]])
    q2 = np.concatenate([cfg] + [r["q2"] for r in r0[:16]])
    N = np.concatenate([np.full(len(cfg), 3, np.int64)] + [r["N"] for r in r0[:16]])
    tune = srv.autotune_launch(s, q1, q2, N, ctas_per_sm=(1, 2, 3, 4), warps=(4, 8), repeats=3)
    b = srv.ServingBatcher(s)
    for i in range(warmup):
        b.step(pool[i % len(pool)])
    b.latencies.clear()
    b.device_ms.clear()
    items = cfgs = edges = 0
    t0 = time.perf_counter()
    for i in range(steps):
        res = b.step(pool[i % len(pool)])
        cfgs += res.n_configs
        edges += res.n_edges
    wall = time.perf_counter() - t0
    lat = b.latency_percentiles()
    # the same steps through host packing into pinned staging (the path of
    # devices without coherent access to pageable host memory)
    b.latencies.clear()
    b.device_ms.clear()
    for i in range(steps):
        b.step(pool[i % len(pool)], direct=False)
    lat_packed = b.latency_percentiles()
    # zero-copy submission: the instances write their requests straight into
    # the pinned staging views (untimed: that is request production); the
    # latency runs from submit to verdicts on the host
    b.latencies.clear()
    b.device_ms.clear()
    for i in range(steps):
        reqs = pool[i % len(pool)]
        slots = b.prepare([(len(r["configs"]), len(r["q1"])) for r in reqs])
        for k, r in enumerate(reqs):
            slots.configs[k][:] = r["configs"]
            slots.q1[k][:] = r["q1"]
            slots.q2[k][:] = r["q2"]
            slots.N[k][:] = r["N"]
        b.submit(slots, t0=time.perf_counter())
    lat_zc = b.latency_percentiles()
    # verdicts of two instances of the first step against the oracle
    res = b.step(pool[0])
    o = orc.OracleScene(sc)
    mism = 0
    t1 = time.perf_counter()
    for k in (0, 1):
        r = pool[0][k]
        mism += int((res.config_free[k] != o.configs_free(r["configs"])).sum())
        mism += int((res.edge_free[k] != o.edges_free(r["q1"], r["q2"], 0.05, N=r["N"])).sum())
    cpu_s = time.perf_counter() - t1
    cpu_items = sum(len(pool[0][k]["configs"]) + len(pool[0][k]["q1"]) for k in (0, 1))
    items = cfgs + edges
    return {
        "workload": "8 mobile manipulators (planar base + 6-DoF arm, 72-D, 304 spheres), 200 boxes in a 6x6x2 m room; "
                    "64 instances/step, each 100-20,000 configs and 10-5,000 edges (N 5..800)",
        "steps": steps, "configs_per_step": cfgs / steps, "edges_per_step": edges / steps,
        "latency": lat, "step_path": "direct gather from the requests' host arrays" if b.direct else "packed",
        "latency_packed": lat_packed, "latency_zero_copy": lat_zc, "items_per_s": items / wall, "configs_per_s": cfgs / wall, "edges_per_s": edges / wall,
        "graph_launches_per_step": 1, "buckets": [list(k) for k in b.graphs],
        "autotune": tune, "verdict_mismatches_sampled": mism,
        "cpu_baseline": {"value": cpu_items / cpu_s, "unit": "items/s (configs + edges)", "cores": orc.num_threads(),
                         "kind": "port", "sample": "instances 0 and 1 of one step, oracle/oracle.c FP64, OpenMP"},
    }


def _summary(line: dict) -> dict:
    """The figures a reader looks for first, repeated at the end of the line
    (a log that keeps only the tail of the output still shows them)."""
    def g(*keys):
        d = line
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    out = {"edges_per_s": line.get("value"), "e2e_edges_per_s": g("e2e", "value"), "e2e_host_arrays_edges_per_s": g("e2e_host_arrays", "value"),
           "verdict_mismatches": line.get("verdict_mismatches"),
           "plain_us_per_edge_call": g("plain", "us_per_call"),
           "plain_us_per_config_call": g("plain_configs", "us_per_call"),
           "batched_over_plain": line.get("batched_over_plain"),
           "roofline_frac_fp32": g("roofline", "frac"),
           "cpu_port_edges_per_s": g("cpu_baseline", "value")}
    for m in ("euclidean", "max_euclidean"):
        out[f"knn_{m}_ms"] = g("knn", m, "ms_per_batch")
        out[f"knn_{m}_index_mismatches"] = g("knn", m, "index_mismatches")
        out[f"knn_{m}_tensor_frac"] = g("knn", m, "roofline", "frac")
    out["abstract_edges_per_s"] = g("abstract", "edges", "edges_per_s")
    out["abstract_host_call_edges_per_s"] = g("abstract", "edges_host_call", "edges_per_s")
    out["abstract_configs_per_s"] = g("abstract", "configs", "configs_per_s")
    out["abstract_reference_python_edges_per_s_pool"] = g("abstract", "cpu_baseline_reference_python",
                                                          "edges_per_s_pool")
    out["abstract_cpu_configs_per_s"] = g("abstract", "configs", "cpu_configs_per_s")
    out["abstract_cpu_edges_per_s"] = g("abstract", "edges", "cpu_edges_per_s")
    out["serving_p50_p99_ms"] = [g("serving", "latency", "p50_ms"), g("serving", "latency", "p99_ms")]
    out["penetration_ms_cost_and_grad"] = g("penetration", "ms_cost_and_grad")
    out["sparse_scene_edges_per_s"] = g("sparse_scene", "edges_per_s")
    out["sparse_scene_free_edges"] = g("sparse_scene", "free_edges")
    out["sparse_scene_mismatches"] = g("sparse_scene", "verdict_mismatches")
    return out


def _reference_timings() -> dict:
    """The reference's own Python code timed on the CPU-runnable workloads
    (tests/golden/time_reference.py writes the file where the reference's
    checkout is; the reference cannot be installed on the GPU host), or {}."""
    p = ROOT / "tests" / "golden" / "reference_timings.json"
    if not p.exists():
        return {}
    d = json.loads(p.read_text())
    d["where"] = ("measured by tests/golden/time_reference.py on " + d.get("host", {}).get("cpu", "?") + " ("
                  + str(d.get("host", {}).get("cpu_count", "?")) + " cores), not on this host")
    return d


def _peaks() -> dict:
    """HBM copy bandwidth and dense BF16 burst throughput measured on this
    pool's GPUs (MEASURED_PEAKS.json), else the fallback figures."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "source": "of measured (MEASURED_PEAKS.json: burst BF16 GEMM, copy bandwidth)"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "of fallback (6.8 TB/s, 1.9 PFLOP/s BF16)"}


def _measure_fp32_peak(_lib) -> float:
    import ctypes as C

    out = C.c_double(0)
    _lib.check(_lib.load().mrmg_microbench_fma(0, 20000, C.byref(out), None))
    return out.value


def _profile_traffic():
    """DRAM bytes per launch of the full-evaluation kernel from the committed
    ncu summary (profiles/), or None."""
    p = ROOT / "profiles" / "arm_edges_kernel_full_eval.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def run_profile(args):
    """Short run for ncu: the first-pass edge kernel on the benchmark workload,
    early-exit ('early') or full-evaluation ('full') mode, the per-mode k-NN
    batch ('knn', euclidean), radius queries ('near'), the penetration cost
    ('pen') or the two-disc scene's calls ('abstract'), `--steps` times."""
    import torch

    if args.profile == "knn":
        knn, scenes = pkg("knn"), pkg("scenes")
        w = scenes.make_knn_workload(seed=0)
        store = knn.NodeStore(w["nodes"], w["mode_offsets"], w["slices"], "euclidean")
        qs = torch.from_numpy(w["queries"]).cuda()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            idx, _ = store.knn(qs, w["q_mode"], w["k"])
        torch.cuda.synchronize()
        print(json.dumps({"profile": "knn", "launches": args.steps, "s": time.perf_counter() - t0,
                          "stats": store.last_stats}), flush=True)
        return 0

    if args.profile == "near":
        knn, scenes = pkg("knn"), pkg("scenes")
        w = scenes.make_knn_workload(seed=0)
        store = knn.NodeStore(w["nodes"], w["mode_offsets"], w["slices"], "euclidean")
        qs = torch.from_numpy(w["queries"]).cuda()
        _, d16 = store.knn(qs, w["q_mode"], 16)
        r = np.nan_to_num(d16[:, -1].cpu().numpy(), posinf=0.0)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            offs, _, _ = store.near(qs, w["q_mode"], r)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "near", "launches": args.steps, "s": time.perf_counter() - t0,
                          "neighbours": int(offs[-1].item())}), flush=True)
        return 0

    if args.profile == "abstract":
        # the two-disc scene's synchronous calls: 1,000 edges at 0.01 and
        # 10,000 configurations per step (edges_kernel / configs_pass launches)
        col, scenes = pkg("collision"), pkg("scenes")
        s = col.Gb300Scene(scenes.make_disc_scene(0))
        rng = np.random.default_rng(0)
        qd = torch.from_numpy(rng.uniform(-1, 1, (10_000, 4))).cuda()
        q1d = torch.from_numpy(rng.uniform(-1, 1, (1000, 4))).cuda()
        q2d = torch.from_numpy(rng.uniform(-1, 1, (1000, 4))).cuda()
        q1h, q2h, qh = q1d.cpu().numpy(), q2d.cpu().numpy(), qd.cpu().numpy()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e = s.is_edge_collision_free_batch(q1d, q2d, 0.01)
            v = s.is_collision_free_batch(qd)
            s.is_edge_collision_free_host(q1h, q2h, 0.01)
            s.is_collision_free_host(qh)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "abstract", "launches": 4 * args.steps, "s": time.perf_counter() - t0,
                          "free_edges": int(e.sum().item()), "free_configs": int(v.sum().item())}), flush=True)
        return 0

    if args.profile == "dist":
        # the two-disc scene's 1,000 x 10,000 euclidean distance matrix (FP64)
        scenes, _lib = pkg("scenes"), pkg("_lib")
        lib = _lib.load()
        sc = scenes.make_disc_scene(0)
        rng = np.random.default_rng(0)
        qd = torch.from_numpy(rng.uniform(-1, 1, (10_000, 4))).cuda()
        q1d = torch.from_numpy(rng.uniform(-1, 1, (1000, 4))).cuda()
        sl = np.ascontiguousarray(sc.agent_slices, dtype=np.int64)
        out = torch.empty((1000, 10_000), dtype=torch.float64, device="cuda")
        t0 = time.perf_counter()
        for _ in range(args.steps):
            _lib.check(lib.mrmg_config_dist_matrix(q1d.data_ptr(), 1000, qd.data_ptr(), 10_000, 4, sl.ctypes.data,
                                                   len(sl), _lib.METRICS["euclidean"], out.data_ptr(),
                                                   _lib.stream_handle(None), 0), "dist matrix")
        torch.cuda.synchronize()
        print(json.dumps({"profile": "dist", "launches": args.steps, "s": time.perf_counter() - t0}), flush=True)
        return 0

    if args.profile == "configs":
        # 100,000 uniform configurations of the four-arm scene per call
        envm, scenes = pkg("env"), pkg("scenes")
        scene = scenes.make_arm_scene(0)
        sc = envm.Gb300ArmEnvironment(scene, collision_resolution=RESOLUTION)._gb300
        q = torch.from_numpy(scenes.uniform_configs(scene, 100_000, seed=3)).cuda()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            v = sc.is_collision_free_batch(q)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "configs", "launches": 2 * args.steps, "s": time.perf_counter() - t0,
                          "free": int(v.sum().item())}), flush=True)
        return 0

    if args.profile == "pen":
        pen, col, scenes = pkg("penetration"), pkg("collision"), pkg("scenes")
        sc = scenes.make_arm_scene(0)
        s = col.Gb300Scene(sc)
        paths = scenes.make_path_workload(sc, seed=0, n_paths=128)
        w = torch.from_numpy(paths).cuda()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            pen.path_penetration(s, w, cost=True)
            pen.path_penetration(s, w, cost=False, grad=True)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "pen", "launches": 2 * args.steps, "s": time.perf_counter() - t0}), flush=True)
        return 0

    _lib, envm = pkg("_lib"), pkg("env")
    scene, q1, q2, N = workload(0)
    sc = envm.Gb300ArmEnvironment(scene, collision_resolution=RESOLUTION)._gb300
    q1_d, q2_d = torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda()
    out = torch.empty(len(q1), dtype=torch.uint8, device="cuda")
    flags = _lib.MRMG_FLAG_FULL_EVAL if args.profile == "full" else 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sc.is_edge_collision_free_batch(q1_d, q2_d, RESOLUTION, out=out, flags=flags)
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "launches": args.steps, "s": time.perf_counter() - t0,
                      "free": int(out.sum().item()), "stats": sc.last_call_stats()}), flush=True)
    return 0


def run_dry(args):
    """The replica orchestration without a GPU: every rank builds its own
    seeded shard, joins the barrier and the max-over-ranks reduction (gloo),
    and rank 0 prints the line's shape with n_gpus = the world size.  No
    edge is checked, so no value is reported; used to test the host logic."""
    world, rank, _ = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    scene, q1, q2, N = workload(rank)
    barrier(world)
    t0 = time.perf_counter()
    barrier(world)
    t = reduce_max(time.perf_counter() - t0, world)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": None, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "dry_run": True,
                          "config": bench_config(world, len(q1)), "barrier_s_max": t,
                          "shard_first_edge_norm": float(np.linalg.norm(q1[0]))}), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def _free_port() -> int:
    import socket

    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _replica_main(rank: int, args, port: int):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(args.gpus),
                      LOCAL_RANK=str(rank))
    fn = run_dry if args.dry_run else (run_reference if args.impl == "reference" else run_gb300)
    rc = fn(args)
    if rc:
        sys.exit(rc)


def spawn_replicas(args) -> int:
    """`--gpus N` without an external launcher: one process per GPU (replicas,
    rank r on GPU r), rendezvous on 127.0.0.1, the same code path as under
    torchrun."""
    import torch.multiprocessing as mp

    try:
        mp.spawn(_replica_main, args=(args, _free_port()), nprocs=args.gpus, join=True)
    except mp.ProcessExitedException as e:
        return int(e.exit_code or 1)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--plain-edges", type=int, default=2000)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--chunks", type=int, default=1, help="pipelined chunks of the end-to-end plan")
    ap.add_argument("--skip-extra", action="store_true", help="only the headline edge-check workload")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch and work shape")
    ap.add_argument("--profile", choices=["early", "full", "knn", "near", "pen", "abstract", "dist", "configs"],
                    default=None,
                    help="short runs of one workload's kernels for ncu captures")
    ap.add_argument("--dry-run", action="store_true",
                    help="replica orchestration only (gloo, no GPU work, no value): tests the host logic")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_replicas(args)
    if args.dry_run:
        return run_dry(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
