"""Path shortcutting over the GB300 collision backend.

Two shortcutters, both taking the reference's planner objects (a list of
states with ``.q`` and ``.mode``; modes with ``task_ids``) and an environment
with the BaseProblem surface (``robots``, ``robot_dims``,
``batch_config_cost``, ``is_path_collision_free``; the GB300 envs of env.py
or any other):

* ``robot_mode_shortcut`` -- planners/shortcutting.py:87-244: one robot's
  straight-line shortcut between two random path indices at a time, kept when
  it lowers the path cost and ``env.is_path_collision_free`` accepts it.  The
  random draws (``np.random.randint``), the interpolation arithmetic, the
  mode-switch rule and the cost test are the reference's, so with the same
  global seed and an environment that gives the same verdicts and costs, the
  result and the cost trace are the reference's.

* ``batched_robot_mode_shortcut`` -- the same shortcut moves, proposed
  ``batch`` at a time: the candidates' costs in one cost call, every
  candidate's vertices and edges in one batched collision pass per mode, and
  the improving free candidates accepted greedily (largest gain first) over
  disjoint index ranges.  On sphere-arm scenes (``repair=True``) candidates
  that improve the cost but collide are handed to gradient repair
  (``penetration.repair_paths``, only the shortcut robot's joints moving,
  the candidate's end states held) and accepted if the exact path check then
  passes and the cost still improves.

``remove_interpolated_nodes`` (shortcutting.py:247-283) and
``interpolate_path`` (problems/util.py:70-101) are the reference's
preprocessing steps.
"""
from __future__ import annotations

import copy
import time
from typing import List, Optional

import numpy as np

from .configuration import path_cost


def _qs(s) -> np.ndarray:
    q = s.q
    return np.asarray(q.state() if hasattr(q, "state") else q, dtype=np.float64)


def _with_q(state, q_flat: np.ndarray, mode=None):
    """A new state of the same type as ``state`` with configuration
    ``state.q.from_flat(q_flat)`` (and ``mode`` if given)."""
    s = copy.copy(state)
    s.q = state.q.from_flat(q_flat) if hasattr(state.q, "from_flat") else np.array(q_flat)
    if mode is not None:
        s.mode = mode
    return s


def remove_interpolated_nodes(path: List, tolerance: float = 1e-15) -> List:
    """Drops states that lie on the segment between their kept predecessor
    and their successor in the same mode (shortcutting.py:247-283)."""
    if len(path) < 3:
        return path
    kept = [path[0]]
    for i in range(1, len(path) - 1):
        a, b, c = kept[-1], path[i], path[i + 1]
        ab = _qs(b) - _qs(a)
        ac = _qs(c) - _qs(a)
        if np.linalg.norm(ac) < tolerance:
            continue
        lam = np.dot(ab, ac) / np.dot(ac, ac)
        if np.linalg.norm(ab - lam * ac) > tolerance or a.mode != c.mode:
            kept.append(b)
    kept.append(path[-1])
    return kept


def interpolate_path(path: List, resolution: float = 0.1) -> List:
    """States every ``resolution`` in the max-abs metric along each segment,
    the segment's start included and the path's last state appended
    (problems/util.py:70-101; config_dist "max" is the largest absolute
    coordinate difference, exact in any order)."""
    out = []
    for i in range(len(path) - 1):
        q0, q1 = _qs(path[i]), _qs(path[i + 1])
        n = max(1, int(float(np.max(np.abs(q0 - q1))) / resolution))
        step = (q1 - q0) / n
        for j in range(n):
            out.append(_with_q(path[i], q0 + step * j, path[i].mode))
    last = copy.copy(path[-1])
    out.append(last)
    return out


def _robot_slices(env) -> list:
    sl, s = [], 0
    for r in env.robots:
        d = int(env.robot_dims[r])
        sl.append((s, s + d))
        s += d
    return sl


def _element(Q: np.ndarray, modes: list, i: int, j: int, r: int, sl: list) -> np.ndarray:
    """Robot ``r``'s straight line from state ``i`` to state ``j``, the
    other robots as on the path; a mode switch inside the range repeats the
    previous interpolation step (shortcutting.py:183-214)."""
    s, e = sl[r]
    q0 = Q[i, s:e] * 1
    q1 = Q[j, s:e] * 1
    diff = (q1 - q0) / (j - i)
    el = Q[i:j + 1].copy()
    for k in range(j - i + 1):
        if k != 0 and i + k != j and modes[i + k] != modes[i + k - 1]:
            el[k, s:e] = q0 + diff * (k - 1)
        else:
            el[k, s:e] = q0 + diff * k
    return el


def robot_mode_shortcut(env, path: List, max_iter: int = 1000, resolution: float = 0.001,
                        tolerance: float = 0.01, robot_choice: str = "round_robin",
                        interpolation_resolution: float = 0.5):
    """Returns ``(new_path, [costs, times])`` as robot_mode_shortcut
    (shortcutting.py:87-244) does: ``costs[0]`` is the interpolated path's
    cost and one cost follows every attempted shortcut (those that improve
    the cost), accepted or not."""
    new_path = interpolate_path(remove_interpolated_nodes(path), interpolation_resolution)
    costs = [path_cost(new_path, env.batch_config_cost)]
    times = [0.0]
    t0 = time.time()
    sl = _robot_slices(env)
    n_rob = len(env.robots)
    cnt = 0
    it = 0
    rr = 0
    max_attempts = 2500
    while True:
        it += 1
        if cnt >= max_iter or it >= max_attempts:
            break
        i = np.random.randint(0, len(new_path))
        j = np.random.randint(0, len(new_path))
        if i > j:
            i, j = j, i
        if abs(j - i) < 2:
            continue
        if robot_choice == "round_robin":
            r = rr % n_rob
            rr += 1
        else:
            r = np.random.randint(0, n_rob)
        if new_path[i].mode.task_ids[r] != new_path[j].mode.task_ids[r]:
            continue
        Q = np.array([_qs(s) for s in new_path[i:j + 1]])
        modes = [s.mode for s in new_path[i:j + 1]]
        el = _element(Q, modes, 0, j - i, r, sl)
        element = [_with_q(new_path[i + k], el[k]) for k in range(j - i + 1)]
        if path_cost(element, env.batch_config_cost) >= path_cost(new_path[i:j + 1], env.batch_config_cost):
            continue
        cnt += 1
        if env.is_path_collision_free(element, resolution=resolution, tolerance=tolerance,
                                      check_start_and_end=False):
            for k in range(j - i + 1):
                new_path[i + k].q = element[k].q
        times.append(time.time() - t0)
        costs.append(path_cost(new_path, env.batch_config_cost))
    return new_path, [costs, times]


# --- batched shortcutting ---------------------------------------------------

def _segments_free(env, elements: list, el_modes: list, resolution: float, templates: Optional[list] = None) -> np.ndarray:
    """Verdict per candidate, as ``is_path_collision_free(element,
    check_start_and_end=False)`` gives it (interior states; every edge's
    interior, in the mode of its first state), for all candidates in one
    batched pass per mode.  An env without batched checks (the reference's
    own envs) is asked ``is_path_collision_free`` once per candidate, on
    states made from ``templates`` (the candidate's path states: their type
    and modes) with the candidate's configurations."""
    nc = len(elements)
    ok = np.ones(nc, dtype=bool)
    if nc == 0:
        return ok
    vq, vc, vm, e1, e2, ec, em = [], [], [], [], [], [], []
    for c, (el, md) in enumerate(zip(elements, el_modes)):
        P = len(el)
        if P > 2:
            vq.append(el[1:-1])
            vc.append(np.full(P - 2, c))
            vm.extend(md[1:-1])
        e1.append(el[:-1])
        e2.append(el[1:])
        ec.append(np.full(P - 1, c))
        em.extend(md[:-1])
    vq = np.concatenate(vq) if vq else np.zeros((0, elements[0].shape[1]))
    vc = np.concatenate(vc) if vc else np.zeros(0, dtype=np.int64)
    e1, e2, ec = np.concatenate(e1), np.concatenate(e2), np.concatenate(ec)
    mode_index = getattr(env, "_mode_index", None)
    sc = getattr(env, "_gb300", None)
    if (mode_index is None or sc is None) and not hasattr(env, "batch_is_collision_free"):
        if templates is None:
            raise TypeError("an env without batched checks needs the candidates' path states")
        for c, (el, tpl) in enumerate(zip(elements, templates)):
            states = [_with_q(t, q) for t, q in zip(tpl, el)]
            ok[c] = bool(env.is_path_collision_free(states, resolution=resolution, check_start_and_end=False))
        return ok
    if mode_index is None or sc is None:
        if len(vq):
            v = np.asarray(env.batch_is_collision_free(vq, None), dtype=bool)
            np.logical_and.at(ok, vc, v)
        e = np.asarray(env.batch_is_edge_collision_free(e1, e2, None, resolution, False), dtype=bool)
        np.logical_and.at(ok, ec, e)
        return ok
    vmi = np.array([int(mode_index(m)) for m in vm], dtype=np.int64)
    emi = np.array([int(mode_index(m)) for m in em], dtype=np.int64)
    # the env's own verdict rule on top of the scene's (the rai penetration
    # tolerance, where the env applies it), as in its is_path_collision_free
    tol = env._tol(None) if hasattr(env, "_tol") else None
    for m in sorted(set(vmi.tolist()) | set(emi.tolist())):
        if sc.mode != m:
            sc.set_mode(m)
        sel = vmi == m
        if sel.any():
            v = sc.is_collision_free_host(vq[sel]).astype(bool)
            if tol is not None:
                v = env._tolerate_configs(vq[sel], v, tol)
            np.logical_and.at(ok, vc[sel], v)
        sel = emi == m
        if sel.any():
            v = sc.is_edge_collision_free_host(e1[sel], e2[sel], resolution, False).astype(bool)
            if tol is not None:
                v = env._tolerate_edges(e1[sel], e2[sel], v, resolution, False, None, 0, None, tol)
            np.logical_and.at(ok, ec[sel], v)
    return ok


def _segment_costs(env, segs: list, agent_slice) -> np.ndarray:
    """Cost of each state sequence in ``segs`` (np.sum of its edge costs),
    with one cost call for all of them."""
    a = np.concatenate([s[:-1] for s in segs])
    b = np.concatenate([s[1:] for s in segs])
    per = np.asarray(env.batch_config_cost(a, b, tmp_agent_slice=agent_slice), dtype=np.float64)
    out, o = np.empty(len(segs)), 0
    for c, s in enumerate(segs):
        out[c] = np.sum(per[o:o + len(s) - 1])
        o += len(s) - 1
    return out


def _repair(env, elements: list, rob: list, sl: list, resolution: float, iters: int, params) -> list:
    """Gradient repair of colliding candidates on a sphere-arm scene: the
    candidates are padded to one length by repeating their last state, only
    the shortcut robot's joints move, the first and the (padded) last states
    are held.  Returns the repaired element arrays (FP64 copies of the FP32
    device result, end states exactly as before)."""
    import torch

    from .penetration import PenetrationParams, repair_paths

    sc = env._gb300
    T = max(len(e) for e in elements)
    D = elements[0].shape[1]
    W = np.empty((len(elements), T, D), dtype=np.float32)
    hold = np.zeros((len(elements), T), dtype=bool)
    move = np.zeros((len(elements), D), dtype=bool)
    for c, el in enumerate(elements):
        W[c, :len(el)] = el
        W[c, len(el):] = el[-1]
        hold[c, 0] = True
        hold[c, len(el) - 1:] = True
        s, e = sl[rob[c]]
        move[c, s:e] = True
    res = repair_paths(sc, torch.from_numpy(W), params or PenetrationParams(), iters=iters,
                       resolution=resolution, hold=hold, move_mask=move, limits=getattr(env, "limits", None))
    got = res["paths"].cpu().numpy().astype(np.float64)
    out = []
    for c, el in enumerate(elements):
        r = el.copy()
        s, e = sl[rob[c]]
        r[1:-1, s:e] = got[c, 1:len(el) - 1, s:e]
        out.append(r)
    return out


def batched_robot_mode_shortcut(env, path: List, rounds: int = 20, batch: int = 256, resolution: float = 0.001,
                                robot_choice: str = "round_robin", interpolation_resolution: float = 0.5,
                                rng: Optional[np.random.Generator] = None, repair: bool = False,
                                repair_iters: int = 40, penetration_params=None, stats: Optional[dict] = None):
    """Returns ``(new_path, [costs, times])`` with one cost per round.

    Every round draws ``batch`` candidate moves (i < j with j - i >= 2, a
    robot whose task is the same at i and j), builds their straight-line
    elements as ``robot_mode_shortcut`` does, keeps those that lower the
    cost, checks them all at once and applies the free ones greedily by gain
    over disjoint index ranges.  ``repair`` (sphere-arm scenes) re-routes the
    improving candidates that collide by gradient repair and re-checks them
    with the same exact path check before they can be accepted.  The end
    states never move; every accepted element passed the exact check."""
    rng = rng if rng is not None else np.random.default_rng()
    new_path = interpolate_path(remove_interpolated_nodes(path), interpolation_resolution)
    sl = _robot_slices(env)
    agent_slice = new_path[0].q._array_slice if hasattr(new_path[0].q, "_array_slice") else np.array(sl)
    n_rob = len(env.robots)
    can_repair = repair and getattr(getattr(env, "_gb300", None), "kind", 0) == 1
    st = stats if stats is not None else {}
    for k in ("proposed", "improving", "free", "accepted", "repaired", "repaired_accepted"):
        st.setdefault(k, 0)
    Q = np.array([_qs(s) for s in new_path])
    modes = [s.mode for s in new_path]
    costs = [float(_segment_costs(env, [Q], agent_slice)[0])]
    times = [0.0]
    t0 = time.time()
    rr = 0
    L = len(Q)
    for _ in range(int(rounds)):
        if L < 3:
            break
        ii = rng.integers(0, L, batch)
        jj = rng.integers(0, L, batch)
        i, j = np.minimum(ii, jj), np.maximum(ii, jj)
        if robot_choice == "round_robin":
            rob = (rr + np.arange(batch)) % n_rob
            rr += batch
        else:
            rob = rng.integers(0, n_rob, batch)
        cands = []
        for c in range(batch):
            a, b, r = int(i[c]), int(j[c]), int(rob[c])
            if b - a < 2 or modes[a].task_ids[r] != modes[b].task_ids[r]:
                continue
            cands.append((a, b, r))
        st["proposed"] += len(cands)
        if not cands:
            continue
        els = [_element(Q, modes, a, b, r, sl) for a, b, r in cands]
        for el, (a, b, _) in zip(els, cands):
            el[-1] = Q[b]          # the element ends exactly on the path's state b
        new_c = _segment_costs(env, els, agent_slice)
        old_c = _segment_costs(env, [Q[a:b + 1] for a, b, _ in cands], agent_slice)
        imp = np.nonzero(new_c < old_c)[0]
        st["improving"] += len(imp)
        if len(imp) == 0:
            continue
        els = [els[c] for c in imp]
        cands = [cands[c] for c in imp]
        gain = (old_c - new_c)[imp]
        el_modes = [modes[a:b + 1] for a, b, _ in cands]
        tpls = [new_path[a:b + 1] for a, b, _ in cands]
        free = _segments_free(env, els, el_modes, resolution, tpls)
        st["free"] += int(free.sum())
        repaired = np.zeros(len(cands), dtype=bool)
        if can_repair and not free.all():
            bad = np.nonzero(~free)[0]
            single = [c for c in bad if all(m == el_modes[c][0] for m in el_modes[c])]
            by_mode = {}
            for c in single:
                key = env._mode_index(el_modes[c][0]) if env._mode_index is not None else -1
                by_mode.setdefault(int(key), []).append(c)
            for key, cs in by_mode.items():
                if key >= 0 and env._gb300.mode != key:
                    env._gb300.set_mode(key)
                fixed = _repair(env, [els[c] for c in cs], [cands[c][2] for c in cs], sl, resolution,
                                repair_iters, penetration_params)
                st["repaired"] += len(cs)
                for c, el in zip(cs, fixed):
                    els[c] = el
                    repaired[c] = True
            if repaired.any():
                rc = np.nonzero(repaired)[0]
                ok = _segments_free(env, [els[c] for c in rc], [el_modes[c] for c in rc], resolution,
                                    [tpls[c] for c in rc])
                rn = _segment_costs(env, [els[c] for c in rc], agent_slice)
                ro = _segment_costs(env, [Q[cands[c][0]:cands[c][1] + 1] for c in rc], agent_slice)
                for c, f, n_, o_ in zip(rc, ok, rn, ro):
                    free[c] = bool(f) and n_ < o_
                    gain[c] = o_ - n_
        taken = np.zeros(L, dtype=bool)
        for c in np.argsort(-gain, kind="stable"):
            if not free[c]:
                continue
            a, b, _ = cands[c]
            if taken[a:b + 1].any():
                continue
            taken[a:b + 1] = True
            Q[a:b + 1] = els[c]
            st["accepted"] += 1
            st["repaired_accepted"] += int(repaired[c])
        times.append(time.time() - t0)
        costs.append(float(_segment_costs(env, [Q], agent_slice)[0]))
    for k in range(1, L - 1):
        new_path[k] = _with_q(new_path[k], Q[k])
    return new_path, [costs, times]
