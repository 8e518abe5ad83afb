"""Batched serving of collision requests from many planner instances.

Each planner step, every instance submits a batch of configurations and a
batch of edges (the calls the planners make through ``is_collision_free`` /
``is_edge_collision_free``, planning_env.py:1724-1763, e.g. from PRM's lazy
edge evaluation, prm_graph.py:652-720, or ``is_path_collision_free``'s rounds,
planning_env.py:1826-1874).  ``ServingBatcher.step`` packs all of them into
one CUDA graph launch:

* a configuration q is checked as the edge q -> q with N = 3 interpolation
  points: its only interior point is q itself (q + 0 * 1), so the verdict is
  is_collision_free(q);
* edges keep their own N (given, or ``int(max|q2 - q1| / resolution) + 1``
  with the minimum of 2, abstract_env.py:321-329);
* unused slots of the capacity bucket get N = 2 and no interior point, so
  they cost nothing.

The graph brings the step's endpoints and counts to the device, runs the
persistent edge pipeline once over the whole step, and copies the verdicts
back.  Where the device reads pageable host memory (GB300 over its coherent
host link; ``mrmg_host_access``), the graph's first launch gathers the
requests' own arrays from host memory through a table of their addresses
(``mrmg_serving_gather``): no host packing pass and no staging copy.
Elsewhere the requests are packed into pinned staging buffers on a thread
pool and copied.  The staging buffers hold FP32 endpoints (half the copy of FP64): the
verdicts (and step counts N) are the reference's for the FP32 values, so
FP64 requests are rounded to FP32 first.  Callers that need the FP64
verdicts of FP64 configurations use
``Gb300Scene`` / the env methods, or ``EdgeCheckPlan`` with its default
FP64 buffers.  Graphs are cached per capacity bucket (configurations and edges
rounded up to a quantum).  ``autotune_launch`` picks the persistent grid
(CTAs per SM, warps per CTA) by timing candidates on a sample step; the
verdicts never depend on it.
"""
from __future__ import annotations

import ctypes as C
import os
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .collision import Gb300Scene, _DeviceWord


def edge_steps(q1: np.ndarray, q2: np.ndarray, resolution: float) -> np.ndarray:
    """N = max(2, int(max_k |q2_k - q1_k| / resolution) + 1) per edge, in
    float64 as abstract_env.py:321-329 computes it."""
    d = np.abs(q2.astype(np.float64) - q1.astype(np.float64)).max(axis=1) / float(resolution)
    return np.maximum(d.astype(np.int64) + 1, 2)


class _StepGraph:
    """One capacity bucket: device buffers, one graph, and either pinned
    host staging (packed) or a gather table (direct: the graph's first launch
    reads the requests' own host arrays, mrmg_serving_gather)."""

    def __init__(self, scene: Gb300Scene, ccap: int, ecap: int, include_endpoints: bool, direct: bool = False,
                 max_src: int = 1024):
        self.scene, self.ccap, self.ecap = scene, int(ccap), int(ecap)
        n = self.ccap + self.ecap
        D = scene.q_dim
        self.n = n
        self.direct = bool(direct)
        self.max_src = int(max_src)
        if self.direct:
            # int64 {n_src, n_configs, n_edges, 0}, then rows {address, rows, first row, kind}
            self.table = torch.zeros(4 + 4 * self.max_src, dtype=torch.int64).pin_memory()
            self.gerr = torch.zeros(1, dtype=torch.int32, device="cuda")
            self.gerr_pin = torch.zeros(1, dtype=torch.int32).pin_memory()
        else:
            self.cfg_pin = torch.empty((self.ccap, D), dtype=torch.float32).pin_memory()
            self.e1_pin = torch.empty((self.ecap, D), dtype=torch.float32).pin_memory()
            self.e2_pin = torch.empty((self.ecap, D), dtype=torch.float32).pin_memory()
            self.N_pin = torch.full((n,), 2, dtype=torch.int64).pin_memory()
        self.out_pin = torch.empty(n, dtype=torch.uint8).pin_memory()
        self.err_pin = torch.zeros(1, dtype=torch.int32).pin_memory()
        self.q1 = torch.zeros((n, D), dtype=torch.float32, device="cuda")
        self.q2 = torch.zeros((n, D), dtype=torch.float32, device="cuda")
        self.N = torch.full((n,), 2, dtype=torch.int64, device="cuda")
        self.out = torch.empty(n, dtype=torch.uint8, device="cuda")
        self.err = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.stream = torch.cuda.Stream()
        self.ev0, self.ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        self.device_ms = 0.0
        self.incl = bool(include_endpoints)
        lib = scene.lib
        _lib.check(lib.mrmg_scene_reserve(scene.h, n, self.stream.cuda_stream))
        ew = C.c_void_p()
        _lib.check(lib.mrmg_scene_error_word(scene.h, C.byref(ew)))
        self._err_view = torch.as_tensor(_DeviceWord(ew.value), device="cuda")
        with torch.cuda.stream(self.stream):   # modules load outside the capture
            scene.is_edge_collision_free_batch(self.q1[:1], self.q2[:1], 0.0, self.incl, N=self.N[:1],
                                               out=self.out[:1], stream=self.stream)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._enqueue()

    def _enqueue(self):
        s, c = self.stream, self.ccap
        if self.direct:
            with torch.cuda.stream(s):
                self.gerr.zero_()
            _lib.check(self.scene.lib.mrmg_serving_gather(self.table.data_ptr(), self.max_src, self.scene.q_dim,
                                                          self.ccap, self.ecap, self.q1.data_ptr(), self.q2.data_ptr(),
                                                          self.N.data_ptr(), self.gerr.data_ptr(), s.cuda_stream),
                       "serving gather")
        else:
            with torch.cuda.stream(s):
                self.q1[:c].copy_(self.cfg_pin, non_blocking=True)
                self.q2[:c].copy_(self.q1[:c])
                self.q1[c:].copy_(self.e1_pin, non_blocking=True)
                self.q2[c:].copy_(self.e2_pin, non_blocking=True)
                self.N.copy_(self.N_pin, non_blocking=True)
        self.scene.is_edge_collision_free_batch(self.q1, self.q2, 0.0, self.incl, N=self.N, out=self.out, stream=s,
                                                flags=_lib.MRMG_FLAG_ASYNC)
        with torch.cuda.stream(s):
            self.err.copy_(self._err_view)
            self.out_pin.copy_(self.out, non_blocking=True)
            self.err_pin.copy_(self.err, non_blocking=True)
            if self.direct:
                self.gerr_pin.copy_(self.gerr, non_blocking=True)

    def run(self) -> np.ndarray:
        with torch.cuda.stream(self.stream):
            self.ev0.record(self.stream)
            self.graph.replay()
            self.ev1.record(self.stream)
        self.stream.synchronize()
        self.device_ms = self.ev0.elapsed_time(self.ev1)
        bits = int(self.err_pin.numpy()[0]) | (int(self.gerr_pin.numpy()[0]) if self.direct else 0)
        if bits:
            _lib.check(self.scene.lib.mrmg_status_from_error_bits(bits), "serving step")
        return self.out_pin.numpy()


@dataclass
class StepSlots:
    """Per-instance views into one bucket's pinned staging buffers: an
    instance writes its configurations into ``configs[k]`` and its edges into
    ``q1[k]`` / ``q2[k]`` / ``N[k]`` (no further host copy)."""
    graph: object
    configs: list
    q1: list
    q2: list
    N: list
    n_configs: int
    n_edges: int
    t0: float = 0.0


@dataclass
class StepResult:
    config_free: list          # per instance: uint8 verdicts of its configurations
    edge_free: list            # per instance: uint8 verdicts of its edges
    latency_s: float           # submit -> verdicts on the host
    device_ms: float           # the graph launch alone (copies + checks), CUDA events
    n_configs: int
    n_edges: int
    bucket: tuple = field(default=(0, 0))


class ServingBatcher:
    """Collision requests of many planner instances, one graph launch per step.

    ``step(requests)`` takes a list of dicts with ``configs`` [n, D], ``q1`` /
    ``q2`` [m, D] and optionally ``N`` [m] (else computed from
    ``resolution``) and returns a ``StepResult`` with the verdicts split back
    per instance (1 = collision free)."""

    def __init__(self, scene: Gb300Scene, resolution: float = 0.05, include_endpoints: bool = False,
                 config_quantum: int = 1 << 16, edge_quantum: int = 1 << 14, direct=None, max_sources: int = 1024):
        """``direct`` (default: where the device reads pageable host memory,
        mrmg_host_access): ``step`` hands the graph a table of the requests'
        own arrays, which its first launch reads from host memory, instead of
        packing them into pinned staging on the host first."""
        if scene.kind != 1:
            raise TypeError("the serving batcher drives arm scenes")
        self.scene = scene
        self.res = float(resolution)
        self.incl = bool(include_endpoints)
        self.cq, self.eq = int(config_quantum), int(edge_quantum)
        if direct is None:
            v = C.c_int32(0)
            _lib.check(scene.lib.mrmg_host_access(C.byref(v)))
            direct = bool(v.value)
        self.direct = bool(direct)
        self.max_src = int(max_sources)
        self.graphs: dict = {}
        self.latencies: list = []
        self.device_ms: list = []
        self._pool = ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1)))

    def _graph(self, nc: int, ne: int, direct: bool = False) -> _StepGraph:
        key = (max(1, -(-nc // self.cq)) * self.cq, max(1, -(-ne // self.eq)) * self.eq, bool(direct))
        g = self.graphs.get(key)
        if g is None:
            g = _StepGraph(self.scene, key[0], key[1], self.incl, direct=direct, max_src=self.max_src)
            self.graphs[key] = g
        return g

    def prepare(self, sizes: list) -> StepSlots:
        """Staging views for one step: ``sizes`` holds (configurations, edges)
        per instance.  Fill the views (explicit N for every edge), then call
        ``submit``; the views stay valid until the next ``prepare`` of the
        same capacity bucket."""
        nc = int(sum(int(a) for a, _ in sizes))
        ne = int(sum(int(b) for _, b in sizes))
        g = self._graph(nc, ne)
        cfg_h, e1_h, e2_h, N_h = g.cfg_pin.numpy(), g.e1_pin.numpy(), g.e2_pin.numpy(), g.N_pin.numpy()
        cv, q1v, q2v, nv = [], [], [], []
        oc = oe = 0
        for a, b in sizes:
            a, b = int(a), int(b)
            cv.append(cfg_h[oc:oc + a])
            q1v.append(e1_h[oe:oe + b])
            q2v.append(e2_h[oe:oe + b])
            nv.append(N_h[g.ccap + oe:g.ccap + oe + b])
            oc += a
            oe += b
        return StepSlots(g, cv, q1v, q2v, nv, nc, ne, time.perf_counter())

    def submit(self, slots: StepSlots, t0=None) -> StepResult:
        """Launch a prepared step and split its verdicts per instance; the
        latency is counted from ``t0`` (default: the time of ``prepare``)."""
        g, nc, ne = slots.graph, slots.n_configs, slots.n_edges
        N_h = g.N_pin.numpy()
        N_h[:nc] = 3
        N_h[nc:g.ccap] = 2
        N_h[g.ccap + ne:] = 2
        out = g.run()
        self.device_ms.append(g.device_ms)
        cf, ef = [], []
        o = 0
        for c in slots.configs:
            cf.append(out[o:o + len(c)].copy())
            o += len(c)
        o = g.ccap
        for a in slots.q1:
            ef.append(out[o:o + len(a)].copy())
            o += len(a)
        lat = time.perf_counter() - (slots.t0 if t0 is None else t0)
        self.latencies.append(lat)
        return StepResult(cf, ef, lat, g.device_ms, nc, ne, (g.ccap, g.ecap))

    def step(self, requests: list, direct=None) -> StepResult:
        """Verdicts of one step's requests; ``direct`` overrides the
        batcher's mode for this step (None: the batcher's)."""
        t0 = time.perf_counter()
        D = self.scene.q_dim

        def rows(r, key):
            a = r.get(key)
            if a is None:
                return np.zeros((0, D), np.float32)
            return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, D))

        cs = [rows(r, "configs") for r in requests]
        e1 = [rows(r, "q1") for r in requests]
        e2 = [rows(r, "q2") for r in requests]
        for a, b in zip(e1, e2):
            if a.shape != b.shape:
                raise ValueError("edge endpoints q1 and q2 must have the same shape")
        Ns = []
        for r, a, b in zip(requests, e1, e2):
            N = r.get("N")
            Ns.append(edge_steps(a, b, self.res) if N is None
                      else np.ascontiguousarray(np.asarray(N, dtype=np.int64).reshape(-1)))
            if len(Ns[-1]) != len(a):
                raise ValueError("one step count per edge")
        nc = int(sum(len(c) for c in cs))
        ne = int(sum(len(a) for a in e1))
        n_src = sum(len(c) > 0 for c in cs) + 3 * sum(len(a) > 0 for a in e1)
        if (self.direct if direct is None else bool(direct)) and n_src <= self.max_src:
            return self._step_direct(t0, cs, e1, e2, Ns, nc, ne)
        g = self._graph(nc, ne)
        cfg_h, e1_h, e2_h, N_h = g.cfg_pin.numpy(), g.e1_pin.numpy(), g.e2_pin.numpy(), g.N_pin.numpy()
        # pack into the pinned staging buffers (numpy copies release the GIL:
        # instances are copied in parallel)
        jobs = []
        o = 0
        for c in cs:
            jobs.append((cfg_h, o, c))
            o += len(c)
        o = 0
        for a, b, N in zip(e1, e2, Ns):
            jobs += [(e1_h, o, a), (e2_h, o, b), (N_h, g.ccap + o, N)]
            o += len(a)

        def put(job):
            dst, off, src = job
            dst[off:off + len(src)] = src

        if nc + ne > 50_000:
            list(self._pool.map(put, jobs))
        else:
            for j in jobs:
                put(j)
        N_h[:nc] = 3
        N_h[nc:g.ccap] = 2
        N_h[g.ccap + ne:] = 2
        out = g.run()
        self.device_ms.append(g.device_ms)
        cf, ef = [], []
        o = 0
        for c in cs:
            cf.append(out[o:o + len(c)].copy())
            o += len(c)
        o = g.ccap
        for a in e1:
            ef.append(out[o:o + len(a)].copy())
            o += len(a)
        lat = time.perf_counter() - t0
        self.latencies.append(lat)
        return StepResult(cf, ef, lat, g.device_ms, nc, ne, (g.ccap, g.ecap))

    def _step_direct(self, t0, cs, e1, e2, Ns, nc, ne) -> StepResult:
        """The step through the gather table: no host copy of the requests;
        the graph's first launch reads them where they are."""
        g = self._graph(nc, ne, direct=True)
        tab = g.table.numpy()
        k = 4
        o = 0
        for c in cs:
            if len(c):
                tab[k:k + 4] = (c.ctypes.data, len(c), o, 0)
                k += 4
            o += len(c)
        o = 0
        for a, b, N in zip(e1, e2, Ns):
            if len(a):
                tab[k:k + 12] = (a.ctypes.data, len(a), o, 1, b.ctypes.data, len(b), o, 2, N.ctypes.data, len(N), o, 3)
                k += 12
            o += len(a)
        tab[0:4] = ((k - 4) // 4, nc, ne, 0)
        out = g.run()   # the arrays of cs / e1 / e2 / Ns stay referenced until the graph has finished
        self.device_ms.append(g.device_ms)
        cf, ef = [], []
        o = 0
        for c in cs:
            cf.append(out[o:o + len(c)].copy())
            o += len(c)
        o = g.ccap
        for a in e1:
            ef.append(out[o:o + len(a)].copy())
            o += len(a)
        lat = time.perf_counter() - t0
        self.latencies.append(lat)
        return StepResult(cf, ef, lat, g.device_ms, nc, ne, (g.ccap, g.ecap))

    def latency_percentiles(self) -> dict:
        if not self.latencies:
            return {}
        a = np.asarray(self.latencies) * 1e3
        d = np.asarray(self.device_ms)
        return {"p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)),
                "mean_ms": float(a.mean()), "device_p50_ms": float(np.percentile(d, 50)),
                "device_p99_ms": float(np.percentile(d, 99)), "steps": len(a)}


def autotune_launch(scene: Gb300Scene, q1, q2, N, resolution: float = 0.0, include_endpoints: bool = False,
                    ctas_per_sm=(1, 2, 3, 4), warps=(4, 8), repeats: int = 3) -> dict:
    """Time the edge pipeline on a sample (q1, q2, N) for every launch shape
    (CTAs per SM x warps per CTA), keep the fastest on the scene and return
    the table.  Shapes the scene's shared memory does not allow are skipped."""
    a = torch.as_tensor(np.asarray(q1, np.float32)).cuda()
    b = torch.as_tensor(np.asarray(q2, np.float32)).cuda()
    Nt = torch.as_tensor(np.asarray(N, np.int64)).cuda()
    out = torch.empty(len(a), dtype=torch.uint8, device="cuda")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    table = []
    ref = None
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    shapes = [(cps, w) for cps in ctas_per_sm for w in warps]
    for cps, w in shapes:
        try:
            scene.set_launch(cps * sms, w)
            scene.is_edge_collision_free_batch(a, b, resolution, include_endpoints, N=Nt, out=out)
        except (ValueError, NotImplementedError, RuntimeError):
            continue
        got = out.cpu().numpy()
        if ref is None:
            ref = got.copy()
        elif not np.array_equal(ref, got):
            raise AssertionError("verdicts changed with the launch shape")
        ts = []
        for _ in range(repeats):
            ev0.record()
            scene.is_edge_collision_free_batch(a, b, resolution, include_endpoints, N=Nt, out=out)
            ev1.record()
            torch.cuda.synchronize()
            ts.append(ev0.elapsed_time(ev1))
        table.append({"ctas_per_sm": cps, "warps": w, "ms": float(np.median(ts))})
    if not table:
        scene.set_launch(0, 0)
        return {"best": None, "table": table}
    best = min(table, key=lambda r: r["ms"])
    scene.set_launch(best["ctas_per_sm"] * sms, best["warps"])
    return {"best": best, "table": table}
