"""Per-mode k nearest neighbours on the GB300 (PRM get_neighbors,
planners/prm/prm_graph.py:389-549; RRT nearest, planners/rrtstar_base.py:1228-1254).

Indices are local to the query's mode and bit-identical to the reference's
selection over its FP64 distances (ties, unspecified in the reference, go to
the lower index)."""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .collision import _dev_tensor


def _slices_arr(slices) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(slices, dtype=np.int64).reshape(-1, 2))


def _query_modes(query_mode, Q: int) -> np.ndarray:
    """One int32 mode per query (the library reads exactly Q of them); a
    single mode applies to every query."""
    if isinstance(query_mode, torch.Tensor):
        query_mode = query_mode.detach().cpu().numpy()
    qm = np.asarray(query_mode, dtype=np.int32).reshape(-1)
    if qm.shape[0] == 1 and Q != 1:
        qm = np.repeat(qm, Q)
    if qm.shape[0] != Q:
        raise ValueError(f"one mode per query: {qm.shape[0]} modes for {Q} queries")
    return np.ascontiguousarray(qm, dtype=np.int32)


def knn_exact(queries, query_mode, nodes, mode_offsets, slices, metric: str, k: int, stream=None):
    """Exact FP64 k-NN (warp per query).  Returns (idx int64 [Q, k], dist float64 [Q, k]) on the device."""
    lib = _lib.load()
    qshape, nshape = tuple(np.shape(queries)), tuple(np.shape(nodes))
    if len(qshape) == 1:
        qshape = (1,) + qshape
    if len(qshape) != 2 or len(nshape) != 2 or nshape[1] != qshape[1]:
        raise ValueError(f"queries {qshape} and nodes {nshape} must be [Q, D] and [M, D]")
    Q, D = qshape
    # the kernel reads the offsets of each query's mode without a bound: check
    # modes and offsets here (host copies of device arguments)
    qm_h = _query_modes(query_mode, Q)
    mo_h = np.asarray(mode_offsets.detach().cpu().numpy() if isinstance(mode_offsets, torch.Tensor) else mode_offsets,
                      dtype=np.int64).reshape(-1)
    if mo_h.shape[0] < 2 or mo_h[0] != 0 or mo_h[-1] != nshape[0] or np.any(np.diff(mo_h) < 0):
        raise ValueError("mode_offsets must rise from 0 to the number of nodes")
    if Q and (qm_h.min() < 0 or qm_h.max() >= mo_h.shape[0] - 1):
        raise ValueError("query mode out of range")
    qs = _dev_tensor(queries, dtype=torch.float64).reshape(Q, D)
    nd = _dev_tensor(nodes, dtype=torch.float64, device=qs.device)
    qm = torch.from_numpy(qm_h).to(qs.device)
    mo = torch.from_numpy(np.ascontiguousarray(mo_h)).to(qs.device)
    sl = _slices_arr(slices)
    idx = torch.empty((Q, k), dtype=torch.int64, device=qs.device)
    dist = torch.empty((Q, k), dtype=torch.float64, device=qs.device)
    _lib.check(lib.mrmg_knn_exact(qs.data_ptr(), Q, qm.data_ptr(), nd.data_ptr(), mo.data_ptr(), D, sl.ctypes.data,
                                  len(sl), _lib.METRICS[metric], int(k), idx.data_ptr(), dist.data_ptr(),
                                  _lib.stream_handle(stream), 0), "knn")
    return idx, dist


def selftest_umma(a_bf16: torch.Tensor, b_bf16: torch.Tensor) -> torch.Tensor:
    """C = A @ B^T through the tcgen05 path (A [128, 64], B [n, 64], BF16)."""
    lib = _lib.load()
    n = b_bf16.shape[0]
    c = torch.zeros((128, n), dtype=torch.float32, device="cuda")
    _lib.check(lib.mrmg_selftest_umma(a_bf16.contiguous().data_ptr(), b_bf16.contiguous().data_ptr(), n, c.data_ptr(),
                                      _lib.stream_handle(None)), "umma self-test")
    return c


class NodeStore:
    """Per-mode node arrays resident on the device for repeated k-NN and
    radius queries (the planners' node_array_cache / batch_subtree).  The
    store owns a copy of the nodes and grows by ``append`` / shrinks by
    ``remove`` as SingleTree does (rrtstar_base.py:270-289).  Euclidean and
    max_euclidean queries use the tensor-core candidate path (tcgen05 split-
    BF16 distance GEMM, certified, FP64 re-rank); other metrics the exact one."""

    PATHS = {"auto": 0, "tensor_core": 1, "exact": 2}

    def __init__(self, nodes, mode_offsets, slices, metric: str = "euclidean", stream=None, path: str = "auto"):
        import ctypes as C

        self.lib = _lib.load()
        self.nodes = _dev_tensor(nodes, dtype=torch.float64)
        self.mode_offsets = np.ascontiguousarray(np.asarray(mode_offsets, dtype=np.int64))
        self.slices = _slices_arr(slices)
        self.metric = metric
        self.D = self.nodes.shape[1]
        h = C.c_void_p()
        _lib.check(self.lib.mrmg_node_store_create(self.nodes.data_ptr(), self.nodes.shape[0], self.D,
                                                   self.mode_offsets.ctypes.data, len(self.mode_offsets) - 1,
                                                   self.slices.ctypes.data, len(self.slices), _lib.METRICS[metric],
                                                   C.byref(h), _lib.stream_handle(stream)), "node store")
        self.h = h
        self.nodes = None          # the store holds its own copy
        self.set_path(path)
        self.last_stats = {}

    def set_path(self, path: str):
        """'auto', 'tensor_core' (wherever the metric allows) or 'exact'
        (node-parallel: certified FP32 candidates re-ranked in FP64, or FP64
        throughout); the results are identical."""
        _lib.check(self.lib.mrmg_node_store_set_path(self.h, self.PATHS[path]), "set_path")
        self.path = path

    @classmethod
    def empty(cls, dim: int, n_modes: int, slices, metric: str = "euclidean", stream=None, path: str = "auto"):
        """A store with ``n_modes`` empty modes, filled by ``append``."""
        return cls(np.zeros((0, dim)), np.zeros(n_modes + 1, dtype=np.int64), slices, metric, stream, path)

    def append(self, mode: int, rows, stream=None):
        """Appends rows [n, D] (host or device) to ``mode``; their mode-local
        indices continue the mode's insertion order."""
        if isinstance(rows, torch.Tensor):
            t = rows.detach().to(torch.float64)
            if t.shape[-1] != self.D:
                raise ValueError(f"rows must have {self.D} columns")
            t = t.reshape(-1, self.D).contiguous()
            ptr, n, keep = t.data_ptr(), t.shape[0], t
        else:
            a = np.ascontiguousarray(np.asarray(rows, dtype=np.float64).reshape(-1, self.D))
            ptr, n, keep = a.ctypes.data, a.shape[0], a
        _lib.check(self.lib.mrmg_node_store_append(self.h, int(mode), ptr, int(n), _lib.stream_handle(stream)),
                   "append")
        del keep

    def remove(self, mode: int, idx: int, stream=None):
        """Removes node ``idx`` of ``mode``: the mode's last node takes its index."""
        _lib.check(self.lib.mrmg_node_store_remove(self.h, int(mode), int(idx), _lib.stream_handle(stream)), "remove")

    def _info(self, mode: int = -1):
        o = np.zeros(3, dtype=np.int64)
        _lib.check(self.lib.mrmg_node_store_info(self.h, int(mode), o.ctypes.data))
        return o

    @property
    def n_modes(self) -> int:
        return int(self._info()[0])

    def size(self, mode: int) -> int:
        return int(self._info(mode)[1])

    @property
    def tensor_core(self) -> bool:
        return bool(self._info()[2])

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.mrmg_node_store_destroy(self.h)
            self.h.value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _queries(self, queries):
        """(pointer, Q, keep-alive, device): CUDA tensors pass as they are;
        host arrays go to the library as host memory (it stages them)."""
        if isinstance(queries, torch.Tensor) and queries.is_cuda:
            qs = _dev_tensor(queries, dtype=torch.float64)
            return qs.data_ptr(), qs.shape[0], qs, qs.device
        a = queries.detach().numpy() if isinstance(queries, torch.Tensor) else queries
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, self.D))
        return a.ctypes.data, a.shape[0], a, torch.device("cuda", torch.cuda.current_device())

    def knn(self, queries, query_mode, k: int, stream=None):
        """(idx [Q, k] int64, dist [Q, k] float64) on the device; idx local to the mode."""
        ptr, Q, keep, dev = self._queries(queries)
        qm = _query_modes(query_mode, Q)
        idx = torch.empty((Q, k), dtype=torch.int64, device=dev)
        dist = torch.empty((Q, k), dtype=torch.float64, device=dev)
        st = np.zeros(2, dtype=np.int64)
        _lib.check(self.lib.mrmg_knn(self.h, ptr, Q, qm.ctypes.data, int(k), idx.data_ptr(),
                                     dist.data_ptr(), st.ctypes.data, _lib.stream_handle(stream)), "knn")
        del keep
        self.last_stats = {"tensor_core": bool(st[0]), "rerun_exact": int(st[1])}
        return idx, dist

    def near(self, queries, query_mode, radius, add_eps: float = 1e-10, cap: int | None = None,
             distances: bool = True, stream=None):
        """Radius neighbours, as RRT* near / find_nearest_indices
        (planners/rrtstar_base.py:439-453, 1296-1337): per query every node of
        its mode with distance <= radius + add_eps, ascending mode-local index.
        ``radius`` is a scalar or one value per query.  Returns CSR device
        tensors (offsets [Q + 1], idx [total], dist [total] float64; dist is
        None when ``distances`` is False)."""
        ptr, Q, keep, dev = self._queries(queries)
        qm = _query_modes(query_mode, Q)
        r = np.ascontiguousarray(np.broadcast_to(np.asarray(radius, dtype=np.float64), (Q,)))
        if cap is None:
            cap = max(1024, 64 * Q)
        offs = torch.empty(Q + 1, dtype=torch.int64, device=dev)
        idx = torch.empty(max(cap, 1), dtype=torch.int64, device=dev)
        dist = torch.empty(max(cap, 1), dtype=torch.float64, device=dev) if distances else None
        tot = np.zeros(1, dtype=np.int64)
        _lib.check(self.lib.mrmg_near(self.h, ptr, Q, qm.ctypes.data, r.ctypes.data, float(add_eps),
                                      offs.data_ptr(), idx.data_ptr(), None if dist is None else dist.data_ptr(),
                                      int(cap), tot.ctypes.data, _lib.stream_handle(stream)), "near")
        total = int(tot[0])
        if total > cap:
            idx = torch.empty(total, dtype=torch.int64, device=dev)
            dist = torch.empty(total, dtype=torch.float64, device=dev) if distances else None
            _lib.check(self.lib.mrmg_near_fetch(self.h, idx.data_ptr(), None if dist is None else dist.data_ptr(),
                                                total, _lib.stream_handle(stream)), "near fetch")
        return offs, idx[:total], (dist[:total] if dist is not None else None)
