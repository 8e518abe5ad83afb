"""Batched lazy edge evaluation for graph search on the GB300.

The composite PRM's search (``MultimodalGraph.search``,
planners/prm/prm_graph.py:552-744) is an A* over edges whose collision check
is deferred until the edge is popped: one ``env.is_edge_collision_free`` call
per popped edge, in pop order.  On a GPU each such call is a launch and a
synchronisation for a single edge.

``SpeculativeEdgeChecker`` turns those calls into batches: when a popped edge
has no verdict yet, it checks that edge together with the next edges the
queue would pop (up to ``window``, in pop order, skipping edges whose target
is already closed) in one batched call per mode, and caches every verdict.
Verdicts are deterministic, so the search sees exactly the verdicts the
sequential calls would give.  Cached verdicts are keyed by the directed edge
and its mode (the check runs from the popped edge's first node, in that
node's mode, as the reference does), and they are not written into the nodes'
white/blacklists until the search itself would have checked the edge: the
lists, the queue contents and the pop order stay the reference's.

``lazy_astar`` restates the search loop with the same queue discipline
(``DictIndexHeap``, prm_queues.py:205-247: smallest f first, ties in push
order), the same white/blacklist rules, pruning against ``best_cost`` and the
same path reconstruction, with the edge checks routed through the checker.
"""
from __future__ import annotations

import heapq
from typing import Callable, Iterable, List, Optional

import numpy as np


def _q(state_q) -> np.ndarray:
    if hasattr(state_q, "state"):
        return np.asarray(state_q.state(), dtype=np.float64)
    return np.asarray(state_q, dtype=np.float64)


class SpeculativeEdgeChecker:
    """Edge verdicts for a search, checked ``window`` edges per batched call.

    ``check(edges, mode)`` must return one verdict per (q0, q1) pair; by
    default it is ``env.batch_is_edge_collision_free(q0s, q1s, mode,
    resolution)``.  ``mode_key(mode)`` groups edges whose checks may share a
    call (default: the mode object itself)."""

    def __init__(self, env=None, resolution: Optional[float] = None, window: int = 256,
                 check: Optional[Callable] = None, mode_key: Callable = lambda m: m):
        if check is None:
            if env is None:
                raise ValueError("an env or a check function is needed")
            res = env.collision_resolution if resolution is None else resolution

            def check(q0s, q1s, mode):
                return np.asarray(env.batch_is_edge_collision_free(q0s, q1s, mode, res), dtype=bool)

        self._check = check
        self.window = max(1, int(window))
        self.mode_key = mode_key
        self.cache = {}
        self.calls = 0          # batched calls made
        self.edges_checked = 0  # edges sent to the device
        self.lookups = 0        # verdicts asked for by the search

    def _key(self, n0, n1):
        return (n0.id, n1.id, self.mode_key(n0.state.mode))

    def is_free(self, n0, n1, upcoming: Iterable = ()) -> bool:
        """Verdict of the edge n0 -> n1 (checked in n0's mode); on a miss the
        edge is checked with up to window - 1 further edges from
        ``upcoming`` ((n0, n1) pairs in the order the search will pop them)."""
        self.lookups += 1
        k = self._key(n0, n1)
        hit = self.cache.get(k)
        if hit is not None:
            return hit
        batch = [(n0, n1)]
        seen = {k}
        for a, b in upcoming:
            if len(batch) >= self.window:
                break
            kk = self._key(a, b)
            if kk in seen or kk in self.cache:
                continue
            seen.add(kk)
            batch.append((a, b))
        groups = {}
        for a, b in batch:
            groups.setdefault(self.mode_key(a.state.mode), []).append((a, b))
        for _, edges in groups.items():
            q0 = np.array([_q(a.state.q) for a, _ in edges])
            q1 = np.array([_q(b.state.q) for _, b in edges])
            v = self._check(q0, q1, edges[0][0].state.mode)
            self.calls += 1
            self.edges_checked += len(edges)
            for (a, b), ok in zip(edges, v):
                self.cache[self._key(a, b)] = bool(ok)
        return self.cache[k]

    def stats(self) -> dict:
        return {"calls": self.calls, "edges_checked": self.edges_checked, "lookups": self.lookups}


class _Heap:
    """(f, push index) heap with items by index: DictIndexHeap's order."""

    __slots__ = ["queue", "items", "idx"]

    def __init__(self):
        self.queue = []
        self.items = {}
        self.idx = 0

    def __bool__(self):
        return bool(self.queue)

    def push(self, item):
        self.items[self.idx] = item
        heapq.heappush(self.queue, (item[0], self.idx))
        self.idx += 1

    def pop(self):
        _, i = heapq.heappop(self.queue)
        return self.items.pop(i)

    def upcoming(self, n: int):
        """The next n items in pop order (for the current contents)."""
        return [self.items[i] for _, i in heapq.nsmallest(n, self.queue)]


def lazy_astar(start, goal_nodes, get_neighbors: Callable, config_cost: Callable, batch_config_cost: Callable,
               h: Callable, checker: SpeculativeEdgeChecker, best_cost: Optional[float] = None) -> dict:
    """The lazy A* of prm_graph.py:615-744 with edge checks from ``checker``.

    ``get_neighbors(node) -> (nodes, [n, D] array)`` (prm_graph.py:389-549),
    ``config_cost(q0, q1)`` and ``batch_config_cost(q, qs)`` the env's costs,
    ``h(node)`` the heuristic.  Nodes carry ``id``, ``state.q``,
    ``state.mode`` and the ``whitelist`` / ``blacklist`` id sets, which are
    updated as the reference updates them.  Returns the path (reconstructed
    as the reference does, start to goal; empty if no goal was reached) and
    the search counters."""
    if best_cost is None:
        best_cost = np.inf
    try:
        goal_set = goal_nodes if isinstance(goal_nodes, (set, frozenset)) else set(goal_nodes)
    except TypeError:   # unhashable nodes: membership as the reference tests it, in the list
        goal_set = list(goal_nodes)
    parents = {start: None}
    gs = {start.id: 0}
    queue = _Heap()
    start_neighbors, _ = get_neighbors(start)
    for n in start_neighbors:
        if start != n:
            ec = config_cost(start.state.q, n.state.q)
            queue.push((gs[start.id] + ec + h(n), ec, (start, n)))
    wasted_pops = 0
    processed_edges = 0
    goal = None
    win = checker.window

    def upcoming():
        for _, _, (a, b) in queue.upcoming(2 * win):
            if b.id in gs or a.id in b.whitelist or b.id in a.blacklist:
                continue
            yield a, b

    while queue:
        _, edge_cost, (n0, n1) = queue.pop()
        if n1.id in gs:
            wasted_pops += 1
            continue
        if n0.id not in n1.whitelist:
            if n1.id in n0.blacklist:
                continue
            if not checker.is_free(n0, n1, upcoming()):
                n1.blacklist.add(n0.id)
                n0.blacklist.add(n1.id)
                continue
            n1.whitelist.add(n0.id)
            n0.whitelist.add(n1.id)
        processed_edges += 1
        g = gs[n0.id] + edge_cost
        gs[n1.id] = g
        parents[n1] = n0
        if n1 in goal_set:
            goal = n1
            break
        neighbors, qs = get_neighbors(n1)
        if not neighbors:
            continue
        costs = batch_config_cost(n1.state.q, qs)
        for n, ec in zip(neighbors, costs):
            if n.id in n1.blacklist:
                continue
            if n.id not in gs:
                f = g + ec + h(n)
                if f > best_cost:
                    continue
                queue.push((f, ec, (n1, n)))
    path: List = []
    if goal is not None:
        path.append(goal)
        n = goal
        while n is not None and parents[n] is not None:
            path.append(parents[n])
            n = parents[n]
        path.append(n)
        path = path[::-1]
    return {"path": path, "cost": gs.get(goal.id) if goal is not None else None, "wasted_pops": wasted_pops,
            "processed_edges": processed_edges, **checker.stats()}
