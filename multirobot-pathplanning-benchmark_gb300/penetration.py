"""Differentiable path-penetration cost of sphere-arm paths on the GB300.

There is no counterpart in the reference.  The cost feeds gradient-based path
repair (``repair_paths``), which ``shortcutting.batched_robot_mode_shortcut``
applies to straight-line shortcuts (planners/shortcutting.py:87-244) that
collide.

For a path ``w[0..T-1]`` of full joint vectors:

    cost = sum_t sum_pairs softplus(beta * (margin - d)) / (beta * scale)
         + smooth_weight * sum_t |w[t+1] - w[t]|^2

over every sphere-box pair (``d`` = signed box distance of the sphere centre
minus the radius) and every pair of spheres on different robots (``d`` =
centre distance minus both radii).  With the defaults (margin = scale = 0.02,
beta = 1, smooth_weight = 0.1) the pair term is ``softplus(0.02 - d) / 0.02``.

``PathPenetrationCost`` is a ``torch.autograd.Function``: its forward runs the
cost kernel and its backward the hand-written gradient kernel, which
recomputes forward kinematics per 32-waypoint segment instead of storing it.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .collision import Gb300Scene


@dataclass(frozen=True)
class PenetrationParams:
    margin: float = 0.02
    scale: float = 0.02
    beta: float = 1.0
    smooth_weight: float = 0.1

    def array(self) -> np.ndarray:
        return np.array([self.margin, self.scale, self.beta, self.smooth_weight], dtype=np.float64)


def _paths_tensor(scene: Gb300Scene, paths) -> torch.Tensor:
    if not isinstance(paths, torch.Tensor):
        paths = torch.as_tensor(np.asarray(paths, dtype=np.float32))
    t = paths.detach()
    if t.dtype != torch.float32:
        t = t.to(torch.float32)
    if not t.is_cuda:
        t = t.cuda()
    t = t.contiguous()
    if t.dim() == 2:
        t = t.unsqueeze(0)
    if t.dim() != 3 or t.shape[-1] != scene.q_dim:
        raise ValueError(f"paths must be [n_paths, n_waypoints, {scene.q_dim}]")
    if t.shape[1] < 1:
        raise ValueError("paths need at least one waypoint")
    return t


def path_penetration(scene: Gb300Scene, paths, params: PenetrationParams = PenetrationParams(), *,
                     cost: bool = True, waypoint_cost: bool = False, grad: bool = False, grad_cost=None,
                     warps_per_cta: int = 0, stream=None, flags: int = 0) -> dict:
    """Cost per path (FP64), per-waypoint cost (FP32) and/or the gradient
    ``grad_cost[p] * dcost_p / dw`` (FP32, same shape as ``paths``)."""
    if scene.kind != 1:
        raise TypeError("the penetration cost needs an arm scene")
    w = _paths_tensor(scene, paths)
    P, T, D = w.shape
    out = {}
    c = torch.empty(P, dtype=torch.float64, device=w.device) if cost else None
    wc = torch.empty((P, T), dtype=torch.float32, device=w.device) if waypoint_cost else None
    g = torch.empty_like(w) if grad else None
    gc = None
    if grad and grad_cost is not None:
        gc = torch.as_tensor(grad_cost, dtype=torch.float32, device=w.device).reshape(-1).contiguous()
        if gc.numel() != P:
            raise ValueError("grad_cost must have one entry per path")
    prm = params.array()
    rc = scene.lib.mrmg_path_penetration(
        scene.h, w.data_ptr(), P, T, prm.ctypes.data, None if gc is None else gc.data_ptr(),
        None if c is None else c.data_ptr(), None if wc is None else wc.data_ptr(),
        None if g is None else g.data_ptr(), int(warps_per_cta), _lib.stream_handle(stream), int(flags))
    _lib.check(rc, "path_penetration")
    if cost:
        out["cost"] = c
    if waypoint_cost:
        out["waypoint_cost"] = wc
    if grad:
        out["grad"] = g
    return out


def penetration_info(scene: Gb300Scene) -> dict:
    o = np.zeros(4, dtype=np.int64)
    _lib.check(scene.lib.mrmg_penetration_info(scene.h, o.ctypes.data))
    return {"spheres": int(o[0]), "boxes": int(o[1]), "smem_cost": int(o[2]), "smem_grad": int(o[3])}


class PathPenetrationCost(torch.autograd.Function):
    """cost[p] (float32) of paths[p] (float32 CUDA tensor [P, T, D])."""

    @staticmethod
    def forward(ctx, paths: torch.Tensor, scene: Gb300Scene, params: PenetrationParams):
        w = _paths_tensor(scene, paths)
        ctx.scene, ctx.params = scene, params
        ctx.squeeze = paths.dim() == 2
        ctx.save_for_backward(w)
        c = path_penetration(scene, w, params, cost=True)["cost"].to(torch.float32)
        return c[0] if ctx.squeeze else c

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        (w,) = ctx.saved_tensors
        go = grad_out.reshape(-1).to(torch.float32)
        g = path_penetration(ctx.scene, w, ctx.params, cost=False, grad=True, grad_cost=go)["grad"]
        return (g[0] if ctx.squeeze else g), None, None


def penetration_cost(paths: torch.Tensor, scene: Gb300Scene, params: PenetrationParams = PenetrationParams()):
    """Differentiable cost per path (see ``PathPenetrationCost``)."""
    return PathPenetrationCost.apply(paths, scene, params)


def repair_paths(scene: Gb300Scene, paths, params: PenetrationParams = PenetrationParams(), iters: int = 50,
                 step: float = 1e-3, resolution: float = 0.05, max_step_norm: float = 0.05,
                 limits=None, hold=None, move_mask=None) -> dict:
    """Gradient path repair: descent steps on the cost with the held
    waypoints fixed (``hold``, [n_paths, n_waypoints] bools; by default the
    first and the last), only the joints of ``move_mask`` moving ([n_paths,
    D] or [D] bools; by default all), each waypoint's move clipped to
    ``max_step_norm`` and the moving joints clamped to ``limits``.  A step is
    kept per path only where it lowers that path's cost, otherwise the path's
    step size is halved, so the cost never rises.  Every path is then checked
    edge by edge (consecutive waypoints, at ``resolution``, end states
    included) with the exact edge checker.  Returns the repaired paths, the
    cost before and after, and a per-path verdict."""
    w = _paths_tensor(scene, paths).clone()
    P, T, D = w.shape
    if hold is None:
        held = torch.zeros((P, T), dtype=torch.bool, device=w.device)
        held[:, 0] = True
        held[:, -1] = True
    else:
        held = torch.as_tensor(np.asarray(hold, dtype=bool), device=w.device).reshape(P, T)
    if move_mask is None:
        mv = torch.ones((P, D), dtype=torch.bool, device=w.device)
    else:
        mv = torch.as_tensor(np.asarray(move_mask, dtype=bool), device=w.device)
        mv = mv.expand(P, D) if mv.dim() == 1 else mv.reshape(P, D)
    movable = (~held)[:, :, None] & mv[:, None, :]
    lo = hi = None
    if limits is not None:
        lim = torch.as_tensor(np.asarray(limits, dtype=np.float32), device=w.device)
        lo, hi = lim[0], lim[1]
    out = path_penetration(scene, w, params, grad=True)
    c0 = out["cost"].clone()
    c, g = out["cost"], out["grad"]
    lr = torch.full((P, 1, 1), float(step), dtype=torch.float32, device=w.device)
    for _ in range(int(iters)):
        d = lr * torch.where(movable, g, torch.zeros_like(g))
        n = torch.linalg.vector_norm(d, dim=-1, keepdim=True)
        d = d * torch.clamp(max_step_norm / torch.clamp(n, min=1e-30), max=1.0)
        cand = w - d
        if lo is not None:
            cand = torch.maximum(torch.minimum(cand, hi), lo)
        cand = torch.where(movable, cand, w)
        nxt = path_penetration(scene, cand, params, grad=True)
        ok = nxt["cost"] <= c
        okw = ok[:, None, None]
        w = torch.where(okw, cand, w)
        c = torch.where(ok, nxt["cost"], c)
        g = torch.where(okw, nxt["grad"], g)
        lr = torch.where(okw, lr, 0.5 * lr)
    free = path_collision_free(scene, w, resolution)
    return {"paths": w, "cost_before": c0, "cost_after": c, "collision_free": free}


def path_collision_free(scene: Gb300Scene, paths, resolution: float) -> torch.Tensor:
    """Per-path verdict (1 = free): every waypoint and every edge between
    consecutive waypoints, endpoints included, as is_path_collision_free
    (planning_env.py:1765-1881) decides it."""
    w = _paths_tensor(scene, paths)
    P, T, D = w.shape
    if T == 1:
        return scene.is_collision_free_batch(w.reshape(P, D))
    a = w[:, :-1].reshape(-1, D).contiguous()
    b = w[:, 1:].reshape(-1, D).contiguous()
    e = scene.is_edge_collision_free_batch(a, b, resolution, include_endpoints=True)
    return e.reshape(P, T - 1).min(dim=1).values
