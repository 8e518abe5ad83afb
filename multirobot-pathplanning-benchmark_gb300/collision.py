"""Device-side scene handles: batched collision checks on the GB300.

``Gb300Scene`` owns one scene of the C library (abstract point agents or
sphere arms) and exposes the batched entry points.  Inputs may be torch CUDA
tensors (used in place) or numpy arrays / host tensors (copied to the device).
Verdicts are uint8 tensors on the device: 1 = collision free.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .scenes import AbstractScene, ArmScene


def _dev_tensor(x, dtype=None, device=None):
    """A contiguous CUDA tensor for x (float32 or float64 kept)."""
    if isinstance(x, torch.Tensor):
        t = x
        if dtype is not None and t.dtype != dtype:
            t = t.to(dtype)
        if not t.is_cuda:
            t = t.to(device or "cuda", non_blocking=t.is_pinned())
        return t.contiguous()
    a = np.asarray(x)
    if dtype is None:
        dtype = torch.float32 if a.dtype == np.float32 else torch.float64
        a = a.astype(np.float32 if dtype == torch.float32 else np.float64, copy=False)
    t = torch.from_numpy(np.ascontiguousarray(a))
    if t.dtype != dtype:
        t = t.to(dtype)
    return t.to(device or "cuda")


def _out_tensor(out, n: int, device) -> torch.Tensor:
    """The verdict buffer: a new one, or the caller's (a contiguous uint8
    device tensor with room for n verdicts; the kernels write n bytes)."""
    if out is None:
        return torch.empty(n, dtype=torch.uint8, device=device)
    if not isinstance(out, torch.Tensor) or out.dtype != torch.uint8 or not out.is_cuda or not out.is_contiguous() \
            or out.numel() < n:
        raise ValueError(f"out must be a contiguous uint8 CUDA tensor of at least {n} elements")
    return out


def _dt_code(t: torch.Tensor) -> int:
    if t.dtype == torch.float32:
        return _lib.MRMG_F32
    if t.dtype == torch.float64:
        return _lib.MRMG_F64
    raise TypeError(f"configurations must be float32 or float64, got {t.dtype}")


def _np_code(a: np.ndarray) -> int:
    return _lib.MRMG_F32 if a.dtype == np.float32 else _lib.MRMG_F64


class Gb300Scene:
    """One scene of libmrmg_gb300 on the current CUDA device."""

    def __init__(self, scene, band: float = 0.0):
        self.lib = _lib.load()
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 backend needs a CUDA device")
        torch.cuda.init()
        self.scene = scene
        h = C.c_void_p()
        keep = []

        def P(a):
            keep.append(a)
            return a.ctypes.data

        if isinstance(scene, AbstractScene):
            t = scene.tables()
            self.kind = 0
            rc = self.lib.mrmg_abstract_scene_create(
                len(scene.agent_radii), scene.dim, scene.q_dim, P(t["agent_offsets"]), P(t["agent_radius"]),
                P(t["pair_threshold"]), P(t["agent_radius_sq"]), len(t["box_lo"]), P(t["box_lo"]), P(t["box_hi"]),
                len(t["sphere_pos"]), P(t["sphere_pos"]), P(t["sphere_radius"]), P(t["sphere_threshold"]), C.byref(h))
        elif isinstance(scene, ArmScene):
            a = scene.arrays()
            self.kind = 1
            rc = self.lib.mrmg_arm_scene_create(
                scene.n_robots, scene.q_dim, P(a["q_offset"]), P(a["base_kind"]), P(a["base_pose"]), P(a["n_links"]),
                P(a["dh"]), len(a["sphere_radius"]), P(a["sphere_robot"]), P(a["sphere_link"]), P(a["sphere_local"]),
                P(a["sphere_radius"]), len(a["box_lo"]), P(a["box_lo"]), P(a["box_hi"]), float(band), C.byref(h))
        else:
            raise TypeError("scene must be an AbstractScene or an ArmScene")
        _lib.check(rc, "scene create")
        self.h = h
        self.q_dim = scene.q_dim
        # single-call buffers and bound entry points (no allocation per call)
        self._one = np.zeros(1, dtype=np.uint8)
        self._one_ptr = self._one.ctypes.data
        self._N1 = np.zeros(1, dtype=np.int64)
        self._N1_ptr = self._N1.ctypes.data
        self._cfg_host = self.lib.mrmg_is_collision_free_host
        self._edge_host = self.lib.mrmg_is_edge_collision_free_host
        self._slot_map = None
        self.mode = -1
        off = getattr(scene, "joint_offset", None) if self.kind == 1 else None
        if off is not None:
            o = np.ascontiguousarray(np.asarray(off, dtype=np.float64).reshape(-1))
            if o.shape != (scene.q_dim,):
                raise ValueError(f"joint_offset must hold {scene.q_dim} values")
            _lib.check(self.lib.mrmg_arm_scene_set_joint_offsets(self.h, o.ctypes.data), "joint offsets")
        if self.kind == 1 and scene.n_modes:
            t = scene.mode_tables()
            _lib.check(self.lib.mrmg_arm_scene_set_modes(
                self.h, scene.n_modes, P(t["sphere_attach"]), P(t["box_off"]), P(t["boxes"]), P(t["attach_off"]),
                P(t["attach"])), "scene modes")

    def set_mode(self, mode: int):
        """Tables of mode ``mode`` for later calls (-1: the scene as created,
        every box and sphere).  Graphs captured earlier keep their tables."""
        _lib.check(self.lib.mrmg_scene_set_mode(self.h, int(mode)), "set_mode")
        self.mode = int(mode)

    def _n_boxes(self) -> int:
        if self.mode >= 0:
            return len(self.scene.mode_boxes[self.mode])
        return len(self.scene.box_lo)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.mrmg_scene_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------
    def info(self) -> dict:
        out = np.zeros(7, dtype=np.int64)
        band = C.c_double(0)
        _lib.check(self.lib.mrmg_scene_info(self.h, out.ctypes.data, C.byref(band)))
        keys = ["kind", "q_dim", "spheres_per_group", "groups", "group_pairs", "ctas", "warps_per_cta"]
        d = {k: int(v) for k, v in zip(keys, out)}
        d["band"] = band.value
        return d

    def set_launch(self, ctas: int = 0, warps_per_cta: int = 0):
        _lib.check(self.lib.mrmg_scene_set_launch(self.h, int(ctas), int(warps_per_cta)))

    def set_tuning(self, box_block: int = 0, box_head: int = 8, cfg_chunk: int = 0, phase_b1: int = 0):
        """Work shape of an arm scene's kernels (0 = default; see
        mrmg_scene_set_tuning).  Never changes a verdict."""
        _lib.check(self.lib.mrmg_scene_set_tuning(self.h, int(box_block), int(box_head), int(cfg_chunk),
                                                  int(phase_b1)))

    def get_tuning(self) -> dict:
        out = np.zeros(4, dtype=np.int32)
        _lib.check(self.lib.mrmg_scene_get_tuning(self.h, out.ctypes.data))
        return dict(zip(("box_block", "box_head", "cfg_chunk", "phase_b1"), map(int, out)))

    def tune_test_order(self, samples, stream=None) -> np.ndarray:
        """Order the boxes so that colliding configurations like `samples`
        (e.g. uniform in the joint limits) stop early; returns the order."""
        if self.kind != 1:
            return np.zeros(0, dtype=np.int32)
        qt = _dev_tensor(samples)
        nb = self._n_boxes()
        order = np.zeros(max(nb, 1), dtype=np.int32)
        _lib.check(self.lib.mrmg_arm_scene_tune_order(self.h, qt.data_ptr(), _dt_code(qt), qt.shape[0],
                                                      order.ctypes.data, _lib.stream_handle(stream)))
        return order[:nb]

    def last_call_stats(self) -> dict:
        out = np.zeros(4, dtype=np.int64)
        _lib.check(self.lib.mrmg_last_call_stats(self.h, out.ctypes.data))
        return {"rechecked_fp64": int(out[0]), "error_bits": int(out[1]), "configs_evaluated": int(out[2])}

    # ------------------------------------------------------------------
    def is_collision_free_batch(self, q, out=None, stream=None, flags: int = 0) -> torch.Tensor:
        """Per-configuration verdicts (1 = free) for q[n, q_dim]."""
        qt = _dev_tensor(q)
        if qt.dim() == 1:
            qt = qt.reshape(1, -1)
        if qt.shape[-1] != self.q_dim:
            raise ValueError(f"configurations must have {self.q_dim} coordinates")
        n = qt.shape[0]
        out = _out_tensor(out, n, qt.device)
        _lib.check(self.lib.mrmg_is_collision_free_batch(self.h, qt.data_ptr(), _dt_code(qt), n, out.data_ptr(),
                                                         _lib.stream_handle(stream), flags), "is_collision_free")
        return out

    def is_collision_free_batch_robots(self, q, robot_mask: int, out=None, stream=None, flags: int = 0) -> torch.Tensor:
        """Per-configuration verdicts for the robots in ``robot_mask`` (bit r =
        robot r): collisions of those robots with boxes and with each other;
        robots outside the mask are ignored (arm scenes)."""
        if self.kind != 1:
            raise NotImplementedError("per-robot checks exist for arm scenes")
        qt = _dev_tensor(q)
        if qt.dim() == 1:
            qt = qt.reshape(1, -1)
        if qt.shape[-1] != self.q_dim:
            raise ValueError(f"configurations must have {self.q_dim} coordinates")
        n = qt.shape[0]
        out = _out_tensor(out, n, qt.device)
        _lib.check(self.lib.mrmg_is_collision_free_batch_robots(self.h, qt.data_ptr(), _dt_code(qt), n,
                                                                int(robot_mask), out.data_ptr(),
                                                                _lib.stream_handle(stream), flags),
                   "is_collision_free_for_robot")
        return out

    def is_edge_collision_free_batch(self, q1, q2, resolution: float, include_endpoints: bool = False, N=None,
                                     N_start: int = 0, N_max=None, out=None, stream=None, flags: int = 0) -> torch.Tensor:
        """Per-edge verdicts (1 = free) for the linear edges q1[n] -> q2[n]."""
        a = _dev_tensor(q1)
        b = _dev_tensor(q2, dtype=a.dtype, device=a.device)
        if a.dim() == 1:
            a, b = a.reshape(1, -1), b.reshape(1, -1)
        if a.shape != b.shape or a.shape[-1] != self.q_dim:
            raise ValueError("edge endpoints must be [n, q_dim] arrays of equal shape")
        n = a.shape[0]
        Nt = None
        if N is not None:
            # one step count per edge (the kernel reads N[e] for every edge); a single one applies to all
            if isinstance(N, torch.Tensor):
                Nt = N.to(device=a.device, dtype=torch.int64).reshape(-1)
                if Nt.numel() == 1 and n != 1:
                    Nt = Nt.expand(n)
                Nt = Nt.contiguous()
            else:
                Nh = np.asarray(N, dtype=np.int64).reshape(-1)
                if Nh.shape[0] == 1 and n != 1:
                    Nh = np.repeat(Nh, n)
                Nt = _dev_tensor(Nh, dtype=torch.int64, device=a.device)
            if Nt.numel() != n:
                raise ValueError(f"N must hold one step count per edge: {Nt.numel()} for {n} edges")
        out = _out_tensor(out, n, a.device)
        rc = self.lib.mrmg_is_edge_collision_free_batch(
            self.h, a.data_ptr(), b.data_ptr(), _dt_code(a), n, float(resolution if resolution is not None else 0.0),
            int(bool(include_endpoints)), None if Nt is None else Nt.data_ptr(), int(N_start),
            -1 if N_max is None else int(N_max), out.data_ptr(), _lib.stream_handle(stream), flags)
        _lib.check(rc, "is_edge_collision_free")
        return out

    # --- host-pointer calls: the planners' one-at-a-time pattern ----------
    # (inputs and verdicts in host memory; one staging copy each way, one
    # launch for small arm batches, synchronous on the scene's own stream)
    def _host_rows(self, x) -> np.ndarray:
        a = np.asarray(x)
        if a.dtype != np.float64 and a.dtype != np.float32:
            a = a.astype(np.float64)
        if a.ndim == 1:
            a = a.reshape(1, -1)
        if a.ndim != 2 or a.shape[1] != self.q_dim:
            raise ValueError(f"configurations must be [n, {self.q_dim}] arrays")
        if not a.flags.c_contiguous:
            a = np.ascontiguousarray(a)
        return a

    def is_collision_free_host(self, q, robot_mask: int = 0, flags: int = 0) -> np.ndarray:
        """Per-configuration verdicts (1 = free) for host configurations
        q[n, q_dim] (numpy); robot_mask as is_collision_free_batch_robots
        (0: every robot)."""
        a = self._host_rows(q)
        out = np.empty(a.shape[0], dtype=np.uint8)
        _lib.check(self.lib.mrmg_is_collision_free_host(self.h, a.ctypes.data, _np_code(a), a.shape[0],
                                                        int(robot_mask), out.ctypes.data, flags), "is_collision_free")
        return out

    def is_edge_collision_free_host(self, q1, q2, resolution: float, include_endpoints: bool = False, N=None,
                                    N_start: int = 0, N_max=None, flags: int = 0) -> np.ndarray:
        """Per-edge verdicts (1 = free) for host endpoint arrays q1, q2 [n, q_dim]."""
        a = self._host_rows(q1)
        b = self._host_rows(q2).astype(a.dtype, copy=False)
        if a.shape != b.shape:
            raise ValueError("edge endpoints must be [n, q_dim] arrays of equal shape")
        n = a.shape[0]
        Nh = None
        if N is not None:
            Nh = np.ascontiguousarray(np.asarray(N, dtype=np.int64).reshape(-1))
            if Nh.shape[0] == 1 and n != 1:
                Nh = np.repeat(Nh, n)
            if Nh.shape[0] != n:
                raise ValueError(f"N must hold one step count per edge: {Nh.shape[0]} for {n} edges")
        out = np.empty(n, dtype=np.uint8)
        rc = self.lib.mrmg_is_edge_collision_free_host(
            self.h, a.ctypes.data, b.ctypes.data, _np_code(a), n, float(resolution if resolution is not None else 0.0),
            int(bool(include_endpoints)), None if Nh is None else Nh.ctypes.data, int(N_start),
            -1 if N_max is None else int(N_max), out.ctypes.data, flags)
        _lib.check(rc, "is_edge_collision_free")
        return out

    def config_free1(self, q, robot_mask: int = 0) -> bool:
        """One configuration (a float64 vector of q_dim values) -> bool."""
        a = q if (type(q) is np.ndarray and q.dtype == np.float64 and q.flags.c_contiguous
                  and q.size == self.q_dim) else self._host_rows(q)
        _lib.check(self._cfg_host(self.h, a.ctypes.data, 1 if a.dtype == np.float64 else 0, 1, robot_mask,
                                  self._one_ptr, 0), "is_collision_free")
        return bool(self._one[0])

    def edge_free1(self, q1, q2, resolution: float, include_endpoints: bool = False, N=None, N_start: int = 0,
                   N_max=None) -> bool:
        """One edge (two float64 vectors of q_dim values) -> bool."""
        ok1 = type(q1) is np.ndarray and q1.dtype == np.float64 and q1.flags.c_contiguous and q1.size == self.q_dim
        ok2 = type(q2) is np.ndarray and q2.dtype == np.float64 and q2.flags.c_contiguous and q2.size == self.q_dim
        a = q1 if ok1 else self._host_rows(q1).astype(np.float64, copy=False)
        b = q2 if ok2 else self._host_rows(q2).astype(np.float64, copy=False)
        Np = None
        if N is not None:
            self._N1[0] = int(N)
            Np = self._N1_ptr
        _lib.check(self._edge_host(self.h, a.ctypes.data, b.ctypes.data, 1, 1, float(resolution),
                                   1 if include_endpoints else 0, Np, int(N_start), -1 if N_max is None else int(N_max),
                                   self._one_ptr, 0), "is_edge_collision_free")
        return bool(self._one[0])

    # ------------------------------------------------------------------
    def slot_map(self) -> np.ndarray:
        if self._slot_map is None:
            info = self.info()
            cap = info["groups"] * info["spheres_per_group"]
            out = np.zeros(cap, dtype=np.int32)
            _lib.check(self.lib.mrmg_arm_slot_map(self.h, out.ctypes.data, cap))
            self._slot_map = out
        return self._slot_map

    def total_penetration(self, q) -> np.ndarray:
        """Total penetration depth (metres, FP64) of each configuration of an
        arm scene: sphere-box and inter-robot sphere-pair overlaps summed
        (mrmg_arm_total_penetration)."""
        if self.kind != 1:
            raise TypeError("total penetration exists for arm scenes only")
        qt = _dev_tensor(q)
        if qt.dim() == 1:
            qt = qt.reshape(1, -1)
        n = qt.shape[0]
        out = torch.empty(n, dtype=torch.float64, device=qt.device)
        _lib.check(self.lib.mrmg_arm_total_penetration(self.h, qt.data_ptr(), _dt_code(qt), n, out.data_ptr(),
                                                       _lib.stream_handle(None)))
        return out.cpu().numpy()

    def sphere_centers(self, q):
        """(FP32, FP64) sphere centres [n, S, 3] of the device kinematics, in
        the scene's sphere order (for the error-bound check)."""
        if self.kind != 1:
            raise TypeError("sphere centres exist for arm scenes only")
        qt = _dev_tensor(q)
        if qt.dim() == 1:
            qt = qt.reshape(1, -1)
        n = qt.shape[0]
        sm = self.slot_map()
        c32 = torch.zeros((n, len(sm), 3), dtype=torch.float32, device=qt.device)
        c64 = torch.zeros((n, len(sm), 3), dtype=torch.float64, device=qt.device)
        _lib.check(self.lib.mrmg_arm_sphere_centers(self.h, qt.data_ptr(), _dt_code(qt), n, c32.data_ptr(),
                                                    c64.data_ptr(), _lib.stream_handle(None)))
        S = int((sm >= 0).sum())
        order = np.argsort(np.where(sm >= 0, sm, 1 << 30))[:S]
        idx = torch.from_numpy(order).to(qt.device)
        return c32[:, idx], c64[:, idx]


class EdgeCheckPlan:
    """A batched edge check of fixed size captured as one CUDA graph.

    The plan owns pinned host buffers for the endpoints and the verdicts and
    device buffers for both.  One ``run()`` replays a graph that copies the
    endpoints host->device in ``chunks`` pieces on a copy stream, checks each
    piece on the compute stream as soon as it has arrived (copies overlap
    checks), copies the verdicts back and records every piece's error bits.
    Fill ``q1_host`` / ``q2_host`` (numpy views of the pinned buffers) and call
    ``run()``; it returns the verdicts (1 = free) as a numpy view.
    """

    def __init__(self, scene: "Gb300Scene", n: int, resolution: float, include_endpoints: bool = False,
                 dtype=torch.float64, chunks: int = 4):
        self.scene = scene
        self.n = int(n)
        D = scene.q_dim
        self.chunks = max(1, min(int(chunks), self.n)) if self.n else 1
        self.q1_pin = torch.empty((self.n, D), dtype=dtype).pin_memory()
        self.q2_pin = torch.empty((self.n, D), dtype=dtype).pin_memory()
        self.out_pin = torch.empty(self.n, dtype=torch.uint8).pin_memory()
        self.err_pin = torch.zeros(self.chunks, dtype=torch.int32).pin_memory()
        self.q1_host = self.q1_pin.numpy()
        self.q2_host = self.q2_pin.numpy()
        self.q1 = torch.empty((self.n, D), dtype=dtype, device="cuda")
        self.q2 = torch.empty((self.n, D), dtype=dtype, device="cuda")
        self.out = torch.empty(self.n, dtype=torch.uint8, device="cuda")
        self.err = torch.zeros(self.chunks, dtype=torch.int32, device="cuda")
        self.compute = torch.cuda.Stream()
        self.copy = torch.cuda.Stream()
        bounds = np.linspace(0, self.n, self.chunks + 1).astype(np.int64)
        self.bounds = [(int(a), int(b)) for a, b in zip(bounds[:-1], bounds[1:])]
        lib = scene.lib
        _lib.check(lib.mrmg_scene_reserve(scene.h, max(b - a for a, b in self.bounds) if self.n else 0,
                                          self.compute.cuda_stream))
        ew = C.c_void_p()
        _lib.check(lib.mrmg_scene_error_word(scene.h, C.byref(ew)))
        self._err_view = torch.as_tensor(_DeviceWord(ew.value), device="cuda")
        self.res, self.incl = float(resolution), bool(include_endpoints)
        # warm-up outside the capture (first launches load modules)
        with torch.cuda.stream(self.compute):
            if self.n:
                scene.is_edge_collision_free_batch(self.q1[:1], self.q2[:1], self.res, self.incl,
                                                   out=self.out[:1], stream=self.compute)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.compute):
            self._enqueue()

    def _enqueue(self):
        sc, cs, cp = self.scene, self.compute, self.copy
        cp.wait_stream(cs)
        events = []
        for a, b in self.bounds:
            with torch.cuda.stream(cp):
                self.q1[a:b].copy_(self.q1_pin[a:b], non_blocking=True)
                self.q2[a:b].copy_(self.q2_pin[a:b], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cp)
            events.append(ev)
        for k, ((a, b), ev) in enumerate(zip(self.bounds, events)):
            cs.wait_event(ev)
            if b > a:
                sc.is_edge_collision_free_batch(self.q1[a:b], self.q2[a:b], self.res, self.incl, out=self.out[a:b],
                                                stream=cs, flags=_lib.MRMG_FLAG_ASYNC)
                with torch.cuda.stream(cs):
                    self.err[k:k + 1].copy_(self._err_view)
        with torch.cuda.stream(cs):
            self.out_pin.copy_(self.out, non_blocking=True)
            self.err_pin.copy_(self.err, non_blocking=True)

    def launch(self):
        """Replay the graph on the plan's stream without waiting."""
        with torch.cuda.stream(self.compute):   # replay() launches on the current stream
            self.graph.replay()

    def wait(self) -> np.ndarray:
        """Wait for the last launch; its verdicts (1 = free) as a numpy view of
        the pinned output buffer."""
        self.compute.synchronize()
        bits = int(np.bitwise_or.reduce(self.err_pin.numpy())) if self.chunks else 0
        if bits:
            _lib.check(self.scene.lib.mrmg_status_from_error_bits(bits), "is_edge_collision_free")
        return self.out_pin.numpy()

    def run(self) -> np.ndarray:
        self.launch()
        return self.wait()


class EdgeCheckPipeline:
    """Several ``EdgeCheckPlan`` slots, each on its own scene handle (own
    per-call scratch) and stream, so consecutive batches overlap: while one
    slot's checks run, the next slot's endpoints are already crossing to the
    device.  ``submit()`` launches the next slot and returns its index;
    ``result(slot)`` waits for that slot and returns its verdicts.  Fill a
    slot's ``q1_host`` / ``q2_host`` only after its previous result was taken.
    Every batch still copies its endpoints host->device and its verdicts back.
    """

    def __init__(self, plans: list):
        if not plans:
            raise ValueError("a pipeline needs at least one plan")
        self.plans = plans
        self.next = 0

    @property
    def depth(self) -> int:
        return len(self.plans)

    def submit(self) -> int:
        slot = self.next
        self.plans[slot].launch()
        self.next = (slot + 1) % len(self.plans)
        return slot

    def result(self, slot: int) -> np.ndarray:
        return self.plans[slot].wait()


class _DeviceWord:
    """__cuda_array_interface__ view of one int32 at a device address."""

    def __init__(self, addr: int):
        self.__cuda_array_interface__ = {"shape": (1,), "typestr": "<i4", "data": (addr, False), "version": 3}


def binary_search_indices(N: int, chunked: bool = False) -> tuple:
    """generate_binary_search_indices(N) computed on the device (closed-form
    position map, or the chunked level iterator)."""
    lib = _lib.load()
    out = torch.zeros(max(int(N), 1), dtype=torch.int64, device="cuda")
    _lib.check(lib.mrmg_binary_search_indices(int(N), out.data_ptr(), int(chunked), _lib.stream_handle(None)))
    return tuple(out[: int(N)].cpu().tolist())
