"""FP64 torch restatement of the path-penetration cost -- TEST INFRASTRUCTURE ONLY.

This module is the checker for the GB300 penetration kernels: tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline / ``--impl reference``
legs use it; the library never imports it.  The cost has no counterpart in
the reference (its consumer would be robot_mode_shortcut,
planners/shortcutting.py:87-244), so the oracle is this float64 autograd
restatement plus central finite differences of it:

    cost = sum_t sum_pairs softplus(beta (margin - d)) / (beta scale)
         + smooth_weight * sum_t |w[t+1] - w[t]|^2

Pairs: every (sphere, box) with d = signed box distance of the centre minus
the radius, and every pair of spheres on different robots with d = centre
distance minus both radii (the robot-robot rule of
AbstractEnvironment.is_collision_free, abstract_env.py:261-268, extended to
sphere sets; no intra-robot pairs, as in the reference).

Forward kinematics follows the standard-DH chain of oracle.c (arm_frames):
frame k = frame k-1 * Rz(theta) Tz(d) Tx(a) Rx(alpha); a planar base is
T(x, y) Rz(theta) times the mount pose.  tests/test_oracle.py pins this FK to
oracle.c's centres.
"""
from __future__ import annotations

import numpy as np
import torch


def _t(a, dev):
    return torch.as_tensor(np.asarray(a), dtype=torch.float64, device=dev)


def fk_centers(arrays: dict, q: torch.Tensor) -> torch.Tensor:
    """Sphere centres [..., S, 3] (input sphere order) for q[..., D] (float64)."""
    dev = q.device
    base = _t(arrays["base_pose"], dev)
    dh = _t(arrays["dh"], dev)
    loc = _t(arrays["sphere_local"], dev)
    s_robot = np.asarray(arrays["sphere_robot"])
    s_link = np.asarray(arrays["sphere_link"])
    q_off = np.asarray(arrays["q_offset"])
    kinds = np.asarray(arrays["base_kind"])
    nls = np.asarray(arrays["n_links"])
    joff = _t(arrays.get("joint_offset", np.zeros(q.shape[-1])), dev)   # joint j turns by q[j] + offset[j]
    S = len(s_robot)
    out = [None] * S
    for r in range(len(q_off)):
        bp = base[r]
        Rb = bp[:9].reshape(3, 3)
        pb = bp[9:]
        jo = int(q_off[r])
        shape = q.shape[:-1]
        if kinds[r] == 1:
            x, y, th = q[..., jo], q[..., jo + 1], q[..., jo + 2] + joff[jo + 2]
            c, s = torch.cos(th), torch.sin(th)
            row0 = c[..., None] * Rb[0] - s[..., None] * Rb[1]
            row1 = s[..., None] * Rb[0] + c[..., None] * Rb[1]
            row2 = Rb[2].expand(*shape, 3)
            Rm = torch.stack([row0, row1, row2], -2)
            p = torch.stack([x + (c * pb[0] - s * pb[1]), y + (s * pb[0] + c * pb[1]), pb[2].expand(shape)], -1)
            jo += 3
        else:
            Rm = Rb.expand(*shape, 3, 3)
            p = pb.expand(*shape, 3)
        frames = [(Rm, p)]
        for k in range(int(nls[r])):
            a, d, ca, sa = dh[r, k]
            th = q[..., jo + k] + joff[jo + k]
            c, s = torch.cos(th), torch.sin(th)
            z = torch.zeros_like(c)
            o = torch.ones_like(c)
            # Rz(theta) Rx(alpha) and the translation Rz(theta) (a, 0, d)
            A = torch.stack([torch.stack([c, -s * ca, s * sa], -1),
                             torch.stack([s, c * ca, -c * sa], -1),
                             torch.stack([z, o * sa, o * ca], -1)], -2)
            t = torch.stack([a * c, a * s, d * o], -1)
            p = p + (Rm @ t[..., None])[..., 0]
            Rm = Rm @ A
            frames.append((Rm, p))
        for i in np.nonzero(s_robot == r)[0]:
            Rk, pk = frames[int(s_link[i])]
            out[i] = pk + (Rk @ loc[i])
    return torch.stack(out, -2)


def _softplus(x):
    return torch.clamp(x, min=0) + torch.log1p(torch.exp(-torch.abs(x)))


def penetration_cost(arrays: dict, paths: torch.Tensor, margin=0.02, scale=0.02, beta=1.0, smooth_weight=0.1,
                     per_waypoint: bool = False) -> torch.Tensor:
    """cost[P] (or per-waypoint [P, T]) of paths[P, T, D], float64, differentiable."""
    dev = paths.device
    c = fk_centers(arrays, paths)                       # [P, T, S, 3]
    r = _t(arrays["sphere_radius"], dev)
    lo = _t(arrays["box_lo"], dev).reshape(-1, 3)
    hi = _t(arrays["box_hi"], dev).reshape(-1, 3)
    ctr, half = 0.5 * (lo + hi), 0.5 * (hi - lo)
    terms = torch.zeros(paths.shape[:2], dtype=torch.float64, device=dev)
    if len(lo):
        dv = c[..., :, None, :] - ctr                   # [P, T, S, B, 3]
        a = torch.abs(dv) - half
        u2 = (torch.clamp(a, min=0) ** 2).sum(-1)
        mx = a.max(-1).values
        sdf = torch.where(mx > 0, torch.sqrt(torch.clamp(u2, min=1e-300)), mx)
        d = sdf - r[:, None]
        terms = terms + _softplus(beta * (margin - d)).sum((-1, -2)) / (beta * scale)
    s_robot = np.asarray(arrays["sphere_robot"])
    I, J = np.triu_indices(len(s_robot), 1)
    keep = s_robot[I] != s_robot[J]
    I, J = torch.as_tensor(I[keep], device=dev), torch.as_tensor(J[keep], device=dev)
    if len(I):
        v = c[..., I, :] - c[..., J, :]
        dist = torch.sqrt(torch.clamp((v * v).sum(-1), min=1e-300))
        d = dist - r[I] - r[J]
        terms = terms + _softplus(beta * (margin - d)).sum(-1) / (beta * scale)
    if paths.shape[1] > 1:
        sm = ((paths[:, 1:] - paths[:, :-1]) ** 2).sum(-1) * smooth_weight
        terms = terms + torch.cat([sm, torch.zeros_like(sm[:, :1])], 1)
    return terms if per_waypoint else terms.sum(1)


def penetration_grad(arrays: dict, paths_np: np.ndarray, **params):
    """(cost[P], grad[P, T, D]) in float64 by torch autograd."""
    w = torch.tensor(np.asarray(paths_np, dtype=np.float64), requires_grad=True)
    c = penetration_cost(arrays, w, **params)
    (g,) = torch.autograd.grad(c.sum(), w)
    return c.detach().numpy(), g.numpy()


def finite_difference(arrays: dict, paths_np: np.ndarray, coords, h: float = 1e-3, **params) -> np.ndarray:
    """Central differences (cost(w + h e) - cost(w - h e)) / 2h of path p's
    cost for each coordinate (p, t, k) in coords, float64."""
    base = np.asarray(paths_np, dtype=np.float64)
    out = []
    with torch.no_grad():
        for p, t, k in coords:
            wp = base[p:p + 1].copy()
            wm = base[p:p + 1].copy()
            wp[0, t, k] += h
            wm[0, t, k] -= h
            cp = penetration_cost(arrays, torch.from_numpy(wp), **params)[0].item()
            cm = penetration_cost(arrays, torch.from_numpy(wm), **params)[0].item()
            out.append((cp - cm) / (2 * h))
    return np.array(out)
