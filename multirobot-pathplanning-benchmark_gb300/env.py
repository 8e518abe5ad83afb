"""Environment backends with the reference's plugin surface.

``Gb300CollisionBackend`` implements the collision / cost methods of
BaseProblem (problems/planning_env.py:1710-1982) on the device; a planner
environment gets the GB300 backend by mixing it in before its mode logic,
exactly where the reference's AbstractEnvironment / rai_env sit:

    class my_env(SequenceMixin, Gb300CollisionBackend, BaseProblem): ...

Two ready-made backends:

* ``Gb300AbstractEnvironment`` -- AbstractEnvironment's scenes (spherical
  point agents, Rectangle and Sphere obstacles, problems/abstract_env.py).
* ``Gb300ArmEnvironment`` -- sphere-arm robots among boxes.

Semantics (verdicts, N, index order, interpolation arithmetic, exceptions)
follow abstract_env.py:255-354 and planning_env.py:1765-1881; the batched
methods are additive.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np
import torch

from . import _lib
from .collision import Gb300Scene
from .configuration import Gb300Configuration, batch_config_cost as _batch_config_cost, config_cost as _config_cost
from .scenes import AbstractScene, ArmScene


def _tune_all(sc: Gb300Scene, smp) -> np.ndarray:
    """Tunes the box test order of every table set of the scene (the scene as
    created and each mode's); returns the order of the scene as created."""
    if sc.kind != 1 or not sc.scene.n_modes:
        return sc.tune_test_order(smp)
    cur = sc.mode
    for m in range(sc.scene.n_modes):
        sc.set_mode(m)
        sc.tune_test_order(smp)
    sc.set_mode(-1)
    order = sc.tune_test_order(smp)
    sc.set_mode(cur)
    return order


def _state(q) -> np.ndarray:
    if hasattr(q, "state"):
        return np.asarray(q.state(), dtype=np.float64)
    return np.asarray(q, dtype=np.float64)


def _max_dist(q1: np.ndarray, q2: np.ndarray) -> float:
    """config_dist(q1, q2, "max") (compute_abs_max_reduction, configuration.py:174-197)."""
    d = q1 - q2
    m = abs(d[0])
    for v in np.abs(d[1:]):
        if v > m:
            m = v
    return float(m)


def _edge_N(q1: np.ndarray, q2: np.ndarray, resolution: float) -> int:
    return max(2, int(_max_dist(q1, q2) / resolution) + 1)


class Gb300CollisionBackend:
    """Collision, edge, path and cost methods of BaseProblem on the GB300.

    Subclasses set ``self._gb300`` (a Gb300Scene), ``collision_resolution``,
    ``collision_tolerance``, ``cost_metric`` and ``cost_reduction``.
    """

    collision_resolution: float = 0.01
    collision_tolerance: float = 0.01
    cost_metric: str = "euclidean"
    cost_reduction: str = "max"
    _gb300: Gb300Scene

    _mode_index = None
    tolerance_semantics = False

    def _use_mode(self, mode):
        """Per-mode scenes: select the tables of the planner's ``mode``
        (``mode_index(mode)`` gives the table index; None leaves the current
        tables), as the reference envs call set_to_mode before a check."""
        if self._mode_index is None or mode is None:
            return
        idx = int(self._mode_index(mode))
        if idx != self._gb300.mode:
            self._gb300.set_mode(idx)

    # --- mode hooks the planners and the mode logic call ---------------------
    def get_scenegraph_info_for_mode(self, mode, is_start_mode: bool = False) -> dict:
        """Stored with every new mode by the mode logic (planning_env.py:466).
        A sphere-set scene has no scene graph: empty, as the abstract env's
        (abstract_env.py:161-162)."""
        return {}

    def set_to_mode(self, m) -> None:
        """Selects the tables of mode ``m`` on a per-mode scene (the receding-
        horizon wrapper and the prioritized planner call it,
        planners/receding_horizon_wrapper.py:173-178,
        prioritized_planner.py:244); on a scene without modes nothing changes,
        as with the abstract env (abstract_env.py:356-360)."""
        self._use_mode(m)

    # --- the rai engine's penetration tolerance (rai_base_env.py:442-615) ---
    def _tol(self, collision_tolerance):
        """The tolerance a check applies: None (exact verdicts) unless the
        env was made with ``tolerance_semantics``."""
        if not self.tolerance_semantics:
            return None
        return self.collision_tolerance if collision_tolerance is None else collision_tolerance

    def _tolerate_configs(self, qs: np.ndarray, free: np.ndarray, tol) -> np.ndarray:
        """rai's rule (rai_base_env.py:460-512, 535-615): a configuration
        that collides still counts as free while the scene's total
        penetration depth is at most ``tol``."""
        free = np.asarray(free, dtype=bool)
        if tol is None:   # exact verdicts: nothing to re-examine
            return free
        bad = np.nonzero(~free)[0]
        if len(bad) == 0:
            return free
        free = free.copy()
        free[bad] = self._gb300.total_penetration(np.ascontiguousarray(qs[bad], dtype=np.float64)) <= tol
        return free

    def _tolerate_edges(self, q1s, q2s, free, resolution, include_endpoints, N, N_start, N_max, tol) -> np.ndarray:
        """rai's edge check (rai_base_env.py:618-700) under the tolerance:
        an edge whose exact check found a collision is re-examined position
        by position (the checked positions q1 + (q2 - q1) / (N - 1) * i of
        generate_binary_search_indices(N)[N_start:N_max]) with
        _tolerate_configs.  The positions of many edges go to the device
        together, in batches of about 2^20."""
        free = np.asarray(free, dtype=bool)
        if tol is None:   # exact verdicts: nothing to re-examine
            return free
        bad = np.nonzero(~free)[0]
        if len(bad) == 0:
            return free
        from .collision import binary_search_indices

        free = free.copy()
        A = np.asarray(q1s, dtype=np.float64)[bad].reshape(len(bad), -1)
        B = np.asarray(q2s, dtype=np.float64)[bad].reshape(len(bad), -1)
        if N is None:
            n = np.array([_edge_N(a, b, resolution) for a, b in zip(A, B)], dtype=np.int64)
        elif np.ndim(N):
            n = np.asarray(N, dtype=np.int64).reshape(-1)[bad]
        else:
            n = np.full(len(bad), int(N), dtype=np.int64)
        whole = N_start == 0 and N_max is None
        lo = 0 if include_endpoints else 1
        start = 0
        while start < len(bad):
            # a batch of edges whose positions add up to about 2^20
            stop, cnt = start, 0
            while stop < len(bad) and (stop == start or cnt + n[stop] <= (1 << 20)):
                cnt += int(n[stop])
                stop += 1
            owner, pos = [], []
            for k in range(start, stop):
                m = int(n[k])
                if whole:
                    idx = np.arange(lo, m - lo, dtype=np.int64) if m - 2 * lo > 0 else np.zeros(0, np.int64)
                else:
                    idx = np.asarray(binary_search_indices(m)[N_start:m if N_max is None else min(m, int(N_max))],
                                     dtype=np.int64)
                    if not include_endpoints:
                        idx = idx[(idx != 0) & (idx != m - 1)]
                owner.append(np.full(len(idx), k, dtype=np.int64))
                pos.append(idx)
            owner = np.concatenate(owner)
            pos = np.concatenate(pos).astype(np.float64)
            if len(owner):
                d = (B[owner] - A[owner]) / (n[owner] - 1)[:, None].astype(np.float64)
                qs = A[owner] + d * pos[:, None]
                ok = self._tolerate_configs(qs, self._gb300.is_collision_free_host(qs).astype(bool), tol)
                edge_ok = np.ones(stop - start, dtype=bool)
                np.logical_and.at(edge_ok, owner - start, ok)
                free[bad[start:stop]] = edge_ok
            else:
                free[bad[start:stop]] = True
            start = stop
        return free

    # --- single queries (planning_env.py:1724-1763) ------------------------
    def is_collision_free(self, q, mode, collision_tolerance: Optional[float] = None) -> bool:
        """One configuration from host memory: one staged copy each way and,
        on arm scenes, one kernel launch (Gb300Scene.config_free1).  With
        ``tolerance_semantics`` a colliding configuration is free while its
        total penetration is at most the tolerance (rai_base_env.py:442-475)."""
        if q is None:
            raise ValueError
        self._use_mode(mode)
        qs = _state(q)
        ok = self._gb300.config_free1(qs)
        tol = self._tol(collision_tolerance)
        if ok or tol is None:
            return ok
        return bool(self._tolerate_configs(qs[None, :], np.array([ok]), tol)[0])

    def is_edge_collision_free(self, q1, q2, mode, resolution: Optional[float] = None,
                               tolerance: Optional[float] = None, include_endpoints: bool = False,
                               N_start: int = 0, N_max: Optional[int] = None, N: Optional[int] = None) -> bool:
        if resolution is None:
            resolution = self.collision_resolution
        a, b = _state(q1), _state(q2)
        if N is not None and N_start > N:
            raise AssertionError
        self._use_mode(mode)
        ok = self._gb300.edge_free1(a, b, resolution, include_endpoints, N, N_start, N_max)
        tol = self._tol(tolerance)
        if ok or tol is None:
            return ok
        return bool(self._tolerate_edges(a[None, :], b[None, :], np.array([ok]), resolution, include_endpoints, N,
                                         N_start, N_max, tol)[0])

    def is_collision_free_for_robot(self, r, q, m=None, collision_tolerance: Optional[float] = None,
                                    set_mode: bool = True) -> bool:
        """rai_base_env.py:515-615 for arm scenes: free unless a robot of ``r``
        (a name or a list of names) touches a box or another robot of ``r``;
        collisions with robots outside ``r`` are ignored.  Exact, like
        is_collision_free; with ``tolerance_semantics`` such a collision is
        ignored while the scene's total penetration is at most the tolerance
        (rai's ``col > collision_tolerance`` test, :549-551)."""
        self._use_mode(m)
        qs = _state(q)
        ok = self._gb300.config_free1(qs, self._robot_mask(r))
        tol = self._tol(collision_tolerance)
        if ok or tol is None:
            return ok
        return bool(self._tolerate_configs(qs[None, :], np.array([ok]), tol)[0])

    def batch_is_collision_free_for_robot(self, r, qs, mode=None) -> np.ndarray:
        """Per-configuration verdicts of is_collision_free_for_robot."""
        self._use_mode(mode)
        if isinstance(qs, torch.Tensor):
            return self._gb300.is_collision_free_batch_robots(qs, self._robot_mask(r)).bool()
        v = self._gb300.is_collision_free_host(qs, self._robot_mask(r)).view(np.bool_)
        return self._tolerate_configs(np.asarray(qs), v, self._tol(None))

    def _robot_mask(self, r) -> int:
        names = [r] if isinstance(r, str) else list(r)
        mask = 0
        for name in names:
            if name not in self.robots:
                raise ValueError(f"unknown robot {name!r}")
            mask |= 1 << self.robots.index(name)
        if not mask:
            raise ValueError("no robot given")
        return mask

    def _batch_is_collision_free(self, qs: List, mode) -> bool:
        """abstract_env.py:278-299: True iff every configuration is free, with
        Sphere obstacles tested in the arithmetic of the reference's batched
        form (Sphere.batch_collides_with_sphere, abstract_env.py:51-55: the
        axis=1 norm), which differs from the single check's on ties within an
        ulp of the contact distance."""
        if len(qs) == 0:
            return True
        self._use_mode(mode)
        v = self._gb300.is_collision_free_host(np.array([_state(q) for q in qs]), flags=_lib.MRMG_FLAG_BATCH_FORM)
        return bool(v.all())

    # --- batched (additive) ------------------------------------------------
    def batch_is_collision_free(self, qs, mode=None) -> np.ndarray:
        """Per-configuration verdicts for an [n, D] array (host memory: one
        staged call, numpy bools back) or device tensor (checked in place,
        bool tensor back)."""
        self._use_mode(mode)
        if isinstance(qs, torch.Tensor):
            return self._gb300.is_collision_free_batch(qs).bool()
        v = self._gb300.is_collision_free_host(qs).view(np.bool_)
        return self._tolerate_configs(np.asarray(qs), v, self._tol(None))

    def batch_is_edge_collision_free(self, q1s, q2s, mode=None, resolution: Optional[float] = None,
                                     include_endpoints: bool = False, N=None) -> np.ndarray:
        """Per-edge verdicts for [n, D] endpoint arrays (or device tensors)."""
        if resolution is None:
            resolution = self.collision_resolution
        self._use_mode(mode)
        if isinstance(q1s, torch.Tensor):
            return self._gb300.is_edge_collision_free_batch(q1s, q2s, resolution, include_endpoints, N).bool()
        v = self._gb300.is_edge_collision_free_host(q1s, q2s, resolution, include_endpoints, N).view(np.bool_)
        return self._tolerate_edges(q1s, q2s, v, resolution, include_endpoints, N, 0, None, self._tol(None))

    def edge_check_plan(self, n: int, resolution: Optional[float] = None, include_endpoints: bool = False,
                        chunks: int = 1, dtype=torch.float64):
        """A reusable, graph-captured batched edge check for batches of `n`
        edges: fill ``plan.q1_host`` / ``plan.q2_host`` (pinned) and call
        ``plan.run()`` -> verdicts.  One graph launch per call; host->device
        copies overlap the checks.  The endpoint buffers are FP64 by default,
        as the reference's configurations; ``dtype=torch.float32`` halves the
        copies and checks the FP32 endpoints exactly (an FP64 endpoint
        written into an FP32 buffer is rounded first)."""
        from .collision import EdgeCheckPlan

        return EdgeCheckPlan(self._gb300, n, self.collision_resolution if resolution is None else resolution,
                             include_endpoints, dtype=dtype, chunks=chunks)

    def edge_check_pipeline(self, n: int, depth: int = 2, resolution: Optional[float] = None,
                            include_endpoints: bool = False, dtype=torch.float64):
        """``depth`` plans of ``n`` edges on separate scene handles and streams
        (see ``collision.EdgeCheckPipeline``): batch k+1's copies overlap
        batch k's checks."""
        from .collision import EdgeCheckPipeline

        scenes = [self._gb300] + [self._clone_scene() for _ in range(max(1, int(depth)) - 1)]
        res = self.collision_resolution if resolution is None else resolution
        from .collision import EdgeCheckPlan

        return EdgeCheckPipeline([EdgeCheckPlan(sc, n, res, include_endpoints, dtype=dtype, chunks=1)
                                  for sc in scenes])

    def _clone_scene(self):
        """Another handle on the same scene (own scratch), with the same box
        test order as this env's handle."""
        from .collision import Gb300Scene

        sc = Gb300Scene(self.scene)
        smp = getattr(self, "_tune_samples", None)
        if smp is not None:
            _tune_all(sc, smp)
        if sc.kind == 1 and self._gb300.mode >= 0:
            sc.set_mode(self._gb300.mode)
        return sc

    # --- path check (planning_env.py:1765-1881), one batched pass ----------
    def is_path_collision_free(self, path, binary_order: bool = True, resolution: Optional[float] = None,
                               tolerance: Optional[float] = None, check_edges_in_order: bool = False,
                               check_start_and_end: bool = True) -> bool:
        """Same verdict as the reference: the vertices it checks (the first
        only with check_start_and_end; the last always when checking edges in
        order, else only with check_start_and_end) and the interior of every
        edge.  The order of checks does not change a verdict, so all are
        submitted at once."""
        if resolution is None:
            resolution = self.collision_resolution
        P = len(path)
        qs = np.array([_state(s.q) for s in path])
        if self._mode_index is not None and P >= 1 and getattr(path[0], "mode", None) is not None:
            return self._path_free_by_mode(path, qs, resolution, check_edges_in_order, check_start_and_end)
        verts = list(range(1, P - 1))
        if check_start_and_end and P >= 2:
            verts = [0] + verts
        if check_edges_in_order or check_start_and_end:
            verts = verts + [P - 1]
        if P == 1:
            verts = [0] if (check_edges_in_order or check_start_and_end) else []
        if verts and not self.batch_is_collision_free(qs[sorted(set(verts))]).all():
            return False
        if P >= 2 and not self.batch_is_edge_collision_free(qs[:-1], qs[1:], None, resolution, False).all():
            return False
        return True

    def _path_free_by_mode(self, path, qs, resolution, check_edges_in_order, check_start_and_end) -> bool:
        """is_path_collision_free on a per-mode scene: each vertex in its
        state's mode, each edge in the mode of its first state
        (planning_env.py:1805-1816), one batch per mode."""
        P = len(path)
        verts = set(range(1, P - 1))
        if check_start_and_end:
            verts.add(0)
        if check_edges_in_order or check_start_and_end:
            verts.add(P - 1)
        idx = [int(self._mode_index(s.mode)) for s in path]
        for m in sorted(set(idx)):
            vs = [i for i in sorted(verts) if idx[i] == m]
            es = [i for i in range(P - 1) if idx[i] == m]
            if self._gb300.mode != m:
                self._gb300.set_mode(m)
            tol = self._tol(None)
            if vs and not self._tolerate_configs(qs[vs], self._gb300.is_collision_free_host(qs[vs]).astype(bool),
                                                 tol).all():
                return False
            if es:
                a, b = qs[es], qs[[i + 1 for i in es]]
                v = self._gb300.is_edge_collision_free_host(a, b, resolution, False).astype(bool)
                if not self._tolerate_edges(a, b, v, resolution, False, None, 0, None, tol).all():
                    return False
        return True

    # --- costs (abstract_env.py:238-253) -----------------------------------
    def config_cost(self, start, end) -> float:
        return _config_cost(start, end, self.cost_metric, self.cost_reduction)

    def batch_config_cost(self, starts, ends, tmp_agent_slice=None) -> np.ndarray:
        return _batch_config_cost(starts, ends, self.cost_metric, self.cost_reduction, tmp_agent_slice=tmp_agent_slice)

    # --- sampling (planning_env.py:1697-1708) ------------------------------
    def sample_config_uniform_in_limits(self):
        q = np.random.uniform(low=self.limits[0, :], high=self.limits[1, :])
        return self.start_pos.from_flat(q)


class Gb300AbstractEnvironment(Gb300CollisionBackend):
    """AbstractEnvironment (problems/abstract_env.py:112-131) on the GB300:
    spherical agents among Rectangle and Sphere obstacles."""

    def __init__(self, scene: AbstractScene, limits=None, start_pos=None, collision_resolution: float = 0.01,
                 collision_tolerance: float = 0.01):
        self.scene = scene
        self.agent_radii = list(scene.agent_radii)
        self.limits = limits if limits is not None else np.stack([np.full(scene.q_dim, -1.0), np.full(scene.q_dim, 1.0)])
        sl = [tuple(map(int, s)) for s in scene.agent_slices]
        self.start_pos = start_pos if start_pos is not None else Gb300Configuration(np.zeros(scene.q_dim), sl)
        self.robots = [f"a{i + 1}" for i in range(len(sl))]
        self.robot_dims = {r: e - s for r, (s, e) in zip(self.robots, sl)}
        self.robot_idx = {r: list(range(s, e)) for r, (s, e) in zip(self.robots, sl)}
        self.collision_resolution = collision_resolution
        self.collision_tolerance = collision_tolerance
        self.cost_metric = "euclidean"
        self.cost_reduction = "max"
        self._gb300 = Gb300Scene(scene)


class Gb300ArmEnvironment(Gb300CollisionBackend):
    """Sphere-arm robots (DH chains, optional planar bases) among boxes."""

    def __init__(self, scene: ArmScene, collision_resolution: float = 0.05, collision_tolerance: float = 0.01,
                 band: float = 0.0, tune_samples: int = 4096, seed: int = 0, mode_index=None,
                 tolerance_semantics: bool = False):
        """``mode_index`` (per-mode scenes): maps a planner mode to the
        scene's table index; by default an int is its own index and a mode
        object uses its ``id``.  ``tolerance_semantics``: the rai engine's
        rule (rai_base_env.py:442-700) -- a configuration that collides
        still counts as free while the scene's total penetration depth is at
        most ``collision_tolerance`` (or the tolerance a call passes); by
        default the checks are exact."""
        self.scene = scene
        if scene.n_modes:
            self._mode_index = mode_index or (lambda m: m if isinstance(m, (int, np.integer)) else m.id)
        self.limits = scene.limits
        sl = [tuple(map(int, s)) for s in scene.agent_slices()]
        self.start_pos = Gb300Configuration(np.zeros(scene.q_dim), sl)
        self.robots = [f"r{i}" for i in range(scene.n_robots)]
        self.robot_dims = {r: e - s for r, (s, e) in zip(self.robots, sl)}
        self.robot_idx = {r: list(range(s, e)) for r, (s, e) in zip(self.robots, sl)}
        self.collision_resolution = collision_resolution
        self.collision_tolerance = collision_tolerance
        self.tolerance_semantics = bool(tolerance_semantics)
        self.cost_metric = "euclidean"
        self.cost_reduction = "max"
        self._gb300 = Gb300Scene(scene, band=band)
        if tune_samples and self.limits is not None:
            # test-order autotuning from configurations uniform in the joint limits
            rng = np.random.default_rng(seed)
            smp = rng.uniform(self.limits[0], self.limits[1], (tune_samples, scene.q_dim)).astype(np.float32)
            self._tune_samples = smp
            self.box_order = _tune_all(self._gb300, smp)
