"""Launch and work-shape autotuning of the collision kernels.

The reference has no counterpart (its checks run one configuration at a
time on the CPU).  The tuner times a sample of the caller's own workload
(an edge batch, or a configuration batch) on the device for each candidate
value of one dimension at a time, keeping the others at their best so far
(coordinate descent), and leaves the fastest setting on the scene:

* launch shape -- CTAs per SM x warps per CTA of the persistent kernels;
* box_block    -- boxes whose near (sphere group, box) pairs are compacted
                  and tested together: the obstacle tile;
* box_head     -- boxes tested one by one before the blocks on an edge's
                  first position;
* phase_b1     -- positions per surviving edge in the first phase-B launch;
* cfg_chunk    -- configurations a warp takes from the work queue at a time
                  (configuration workloads).

Every trial's verdicts must equal the first trial's (AssertionError
otherwise): none of these settings may change a verdict.
"""
from __future__ import annotations

import numpy as np
import torch

from .collision import Gb300Scene

DEFAULT_SPACE = {
    "launch": [(c, w) for c in (1, 2, 3, 4) for w in (4, 8)],
    "box_block": (4, 8, 16),
    "box_head": (0, 4, 8, 16),
    "phase_b1": (2, 3, 6),
    "cfg_chunk": (2, 4, 8),
}


def autotune(scene: Gb300Scene, q1=None, q2=None, N=None, resolution: float = 0.0, include_endpoints: bool = False,
             configs=None, space: dict | None = None, repeats: int = 3, stream=None) -> dict:
    """Tunes ``scene`` on the edge sample (q1, q2[, N]) or, with
    ``configs``, on a configuration sample.  Returns ``{"best": {...},
    "default_ms", "best_ms", "table": [...]}`` (median of ``repeats`` CUDA
    event timings per trial)."""
    sp = dict(DEFAULT_SPACE)
    sp.update(space or {})
    edges = configs is None
    if edges:
        a = torch.as_tensor(np.asarray(q1, np.float32)).cuda()
        b = torch.as_tensor(np.asarray(q2, np.float32)).cuda()
        Nt = None if N is None else torch.as_tensor(np.asarray(N, np.int64)).cuda()
        out = torch.empty(len(a), dtype=torch.uint8, device="cuda")

        def run():
            scene.is_edge_collision_free_batch(a, b, resolution, include_endpoints, N=Nt, out=out)
    else:
        q = torch.as_tensor(np.asarray(configs, np.float32)).cuda()
        out = torch.empty(len(q), dtype=torch.uint8, device="cuda")

        def run():
            scene.is_collision_free_batch(q, out=out)

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    arm = scene.kind == 1
    cur = {"launch": (0, 0)}
    if arm:
        cur.update(scene.get_tuning())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ref = {}
    table = []

    def apply(setting):
        c, w = setting["launch"]
        scene.set_launch(c * sms, w)
        if arm:
            scene.set_tuning(setting["box_block"], setting["box_head"], setting["cfg_chunk"], setting["phase_b1"])

    def trial(setting):
        try:
            apply(setting)
            run()
        except (ValueError, NotImplementedError, RuntimeError):
            return None
        got = out.cpu().numpy()
        if "v" not in ref:
            ref["v"] = got.copy()
        elif not np.array_equal(ref["v"], got):
            raise AssertionError(f"verdicts changed with the setting {setting}")
        ts = []
        for _ in range(repeats):
            ev0.record()
            run()
            ev1.record()
            torch.cuda.synchronize()
            ts.append(ev0.elapsed_time(ev1))
        ms = float(np.median(ts))
        table.append({**{k: (list(v) if k == "launch" else v) for k, v in setting.items()}, "ms": ms})
        return ms

    best_ms = trial(cur)
    default_ms = best_ms
    dims = ["launch"] + (["box_block", "box_head", "phase_b1"] if arm and edges else []) + \
        (["box_block", "cfg_chunk"] if arm and not edges else [])
    if not arm and not edges:
        dims = ["launch"]
    for dim in dims:
        for v in sp[dim]:
            cand = dict(cur)
            cand[dim] = tuple(v) if dim == "launch" else int(v)
            if cand == cur:
                continue
            ms = trial(cand)
            if ms is not None and (best_ms is None or ms < best_ms):
                best_ms, cur = ms, cand
    apply(cur)
    best = {k: (list(v) if k == "launch" else v) for k, v in cur.items()}
    if best["launch"] != [0, 0]:
        best["ctas"] = best["launch"][0] * sms
    return {"best": best, "default_ms": default_ms, "best_ms": best_ms, "table": table}
