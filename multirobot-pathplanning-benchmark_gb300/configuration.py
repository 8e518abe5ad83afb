"""Configurations, distances and costs on the GB300.

Mirrors problems/core/configuration.py of the reference:

* ``Gb300Configuration`` has NpConfiguration's surface (flat float64 ``q`` +
  ``_array_slice``, ``from_flat`` / ``from_list`` / ``from_numpy``,
  ``robot_state``, ``state``, ``num_agents``); its ``_batch_dist`` runs on the
  device, so the planners' ``batch_config_dist(pt, batch, metric)`` -- which
  dispatches on ``type(pt)._batch_dist`` (configuration.py:342-349) -- is
  routed to the GPU without touching the planners.
* ``batch_config_dist``, ``config_dist``, ``batch_config_cost``,
  ``config_cost``, ``path_cost`` and ``config_dist_matrix`` keep the
  reference's signatures and return bit-identical float64 values.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from . import _lib
from .collision import _dev_tensor


def _slices_arr(slices) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(slices, dtype=np.int64).reshape(-1, 2))


def config_dist_matrix(queries, nodes, slices, metric: str = "euclidean", out=None, stream=None) -> torch.Tensor:
    """d[q, m] = batch_config_dist(queries[q], nodes, metric)[m] on the device (float64)."""
    if metric not in _lib.METRICS:
        raise ValueError(f"unknown metric {metric!r}")
    lib = _lib.load()
    qs = _dev_tensor(queries, dtype=torch.float64)
    nd = _dev_tensor(nodes, dtype=torch.float64, device=qs.device)
    if qs.dim() == 1:
        qs = qs.reshape(1, -1)
    if nd.dim() == 1:
        nd = nd.reshape(1, -1)
    D = qs.shape[1]
    if nd.shape[1] != D:
        raise ValueError("queries and nodes must have the same dimension")
    sl = _slices_arr(slices)
    if out is None:
        out = torch.empty((qs.shape[0], nd.shape[0]), dtype=torch.float64, device=qs.device)
    elif not isinstance(out, torch.Tensor) or out.dtype != torch.float64 or not out.is_cuda \
            or not out.is_contiguous() or out.numel() < qs.shape[0] * nd.shape[0]:
        raise ValueError(f"out must be a contiguous float64 CUDA tensor of {qs.shape[0]} x {nd.shape[0]} elements")
    _lib.check(lib.mrmg_config_dist_matrix(qs.data_ptr(), qs.shape[0], nd.data_ptr(), nd.shape[0], D, sl.ctypes.data,
                                           len(sl), _lib.METRICS[metric], out.data_ptr(), _lib.stream_handle(stream), 0),
               "config_dist_matrix")
    return out


def _cost(starts, ends, slices, metric, reduction, w, mode) -> torch.Tensor:
    if reduction not in _lib.REDUCTIONS:
        raise ValueError(f"unknown reduction {reduction!r}")
    lib = _lib.load()
    a = _dev_tensor(starts, dtype=torch.float64)
    b = None if ends is None else _dev_tensor(ends, dtype=torch.float64, device=a.device)
    if mode == 1 and b.shape != a.shape:
        # diff = starts - batch_other with numpy broadcasting (configuration.py:457-459)
        try:
            a, b = torch.broadcast_tensors(a, b)
        except RuntimeError:
            raise ValueError("operands could not be broadcast together") from None
        a, b = a.contiguous(), b.contiguous()
    D = a.shape[-1]
    if mode == 0:
        if b.shape[-1] != D:
            raise ValueError("operands could not be broadcast together")
        M = b.reshape(-1, D).shape[0]
    else:
        if a.dim() != 2:   # the reference indexes diff[:, s:e]
            raise ValueError(f"cost operands must be [M, D] arrays, got {tuple(a.shape)}")
        M = a.shape[0] if mode == 1 else a.shape[0] - 1
    sl = _slices_arr(slices)
    out = torch.empty(max(M, 0), dtype=torch.float64, device=a.device)
    cm = _lib.COST_METRICS["euclidean" if metric == "euclidean" else "max"]
    _lib.check(lib.mrmg_batch_config_cost(a.data_ptr(), None if b is None else b.data_ptr(), M, D, sl.ctypes.data,
                                          len(sl), cm, _lib.REDUCTIONS[reduction], float(w), mode, out.data_ptr(),
                                          _lib.stream_handle(None), 0), "batch_config_cost")
    return out


class Gb300Configuration:
    """NpConfiguration-compatible configuration whose distances run on the GPU."""

    __slots__ = ("_array_slice", "q", "_num_agents")

    def __init__(self, q, _slice):
        self._array_slice = np.array(_slice)
        self.q = np.asarray(q).astype(np.float64)
        self._num_agents = len(self._array_slice)

    def num_agents(self) -> int:
        return self._num_agents

    def __getitem__(self, ind):
        return self.robot_state(ind)

    def __setitem__(self, ind, data):
        s, e = self._array_slice[ind]
        self.q[s:e] = data

    @classmethod
    def from_list(cls, q_list: Sequence) -> "Gb300Configuration":
        if len(q_list) == 1:
            return cls(np.asarray(q_list[0]), [(0, len(q_list[0]))])
        slices, s = [], 0
        for qi in q_list:
            slices.append((s, s + len(qi)))
            s += len(qi)
        return cls(np.concatenate(q_list), slices)

    def from_flat(self, q) -> "Gb300Configuration":
        q = np.asarray(q)
        assert q.shape == self.q.shape, "Shape mismatch"
        return type(self)(q, self._array_slice.copy())

    @classmethod
    def from_numpy(cls, arr) -> "Gb300Configuration":
        return cls(arr, [(0, len(arr))])

    def robot_state(self, ind: int) -> np.ndarray:
        if self._num_agents == 1:
            return self.q
        s, e = self._array_slice[ind]
        return self.q[s:e]

    def state(self) -> np.ndarray:
        return self.q

    def as_list(self) -> list:
        return [self.robot_state(i) for i in range(self._num_agents)]

    @classmethod
    def _dist(cls, pt, other, metric: str = "euclidean") -> float:
        return float(cls._batch_dist(pt, [other], metric)[0])

    @classmethod
    def _batch_dist(cls, pt, batch_other, metric: str = "euclidean") -> np.ndarray:
        """NpConfiguration._batch_dist (configuration.py:303-329) on the device."""
        if isinstance(batch_other, np.ndarray) or isinstance(batch_other, torch.Tensor):
            arr = batch_other
        else:
            arr = np.array([o.q for o in batch_other], dtype=np.float64)
        m = metric if metric in ("euclidean", "sum_euclidean", "max_euclidean") else "max"
        out = config_dist_matrix(np.asarray(pt.q, dtype=np.float64).reshape(1, -1), arr, pt._array_slice, m)
        return out[0].cpu().numpy()


def config_dist(q_start, q_end, metric: str = "max") -> float:
    """config_dist (configuration.py:332-339)."""
    return type(q_start)._dist(q_start, q_end, metric)


def batch_config_dist(pt, batch_pts, metric: str = "max") -> np.ndarray:
    """batch_config_dist (configuration.py:342-349): dispatches on type(pt)."""
    return type(pt)._batch_dist(pt, batch_pts, metric)


def batch_config_cost(starts, batch_other, metric: str = "max", reduction: str = "max", w: float = 0.01,
                      tmp_agent_slice=None) -> np.ndarray:
    """batch_config_cost (configuration.py:437-489) with the same input forms."""
    if hasattr(starts, "state") and hasattr(starts, "_array_slice") and isinstance(batch_other, np.ndarray):
        return _cost(np.asarray(starts.state(), dtype=np.float64), batch_other, starts._array_slice, metric,
                     reduction, w, 0).cpu().numpy()
    if isinstance(starts, np.ndarray) and isinstance(batch_other, np.ndarray):
        return _cost(starts, batch_other, tmp_agent_slice, metric, reduction, w, 1).cpu().numpy()
    if batch_other is None and tmp_agent_slice is not None:
        if isinstance(starts[0], np.ndarray):
            return _cost(np.array(starts), None, tmp_agent_slice, metric, reduction, w, 2).cpu().numpy()
        raise ValueError
    if isinstance(starts, list) and isinstance(batch_other, list):
        if hasattr(starts[0], "state"):
            a = np.array([s.state() for s in starts])
            b = np.array([o.state() for o in batch_other], dtype=np.float64)
            sl = starts[0]._array_slice
        else:
            a = np.array([s.q.state() for s in starts])
            b = np.array([o.q.state() for o in batch_other], dtype=np.float64)
            sl = starts[0].q._array_slice
        return _cost(a, b, sl, metric, reduction, w, 1).cpu().numpy()
    raise ValueError


def config_cost(q_start, q_end, metric: str = "max", reduction: str = "max") -> float:
    """config_cost (configuration.py:352-363)."""
    return batch_config_cost(q_start, q_end.state()[None, :], metric, reduction)[0]


def path_cost(path, batch_cost_fun, agent_slices=None) -> float:
    """path_cost (problems/util.py:51-67): per-edge costs, then np.sum."""
    if hasattr(path[0], "q") and hasattr(path[0], "mode"):
        pts = [s.q.state() for s in path]
        costs = batch_cost_fun(pts, None, tmp_agent_slice=path[0].q._array_slice)
    elif isinstance(path[0], np.ndarray) and agent_slices is not None:
        costs = batch_cost_fun(path, None, tmp_agent_slice=agent_slices)
    else:
        raise ValueError("Arguments to path cost seem to be wrong.")
    return np.sum(costs)
