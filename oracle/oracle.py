"""CPU FP64 oracle for the collision / distance path -- TEST INFRASTRUCTURE ONLY.

This module is the checker: tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / ``--impl reference`` legs use it.  The GB300 library never
imports it.  It binds oracle.c (a C restatement of the reference's arithmetic,
built with -ffp-contract=off) and adds small numpy / pure-Python mirrors.

Pinning: tests/golden/ holds vectors generated by importing the reference
itself (tests/golden/make_golden.py); tests/test_oracle.py checks this module
against every one of them before any GPU result is compared with it.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from collections import deque
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"

vp = C.c_void_p
i32, i64, f64 = C.c_int32, C.c_int64, C.c_double


def build(force: bool = False) -> Path:
    """Compile oracle.c (gcc -O2 -ffp-contract=off, OpenMP when available)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("gcc is required to build the oracle")
    base = [cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", str(SRC), "-o", str(LIB) + ".tmp", "-lm"]
    r = subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True, text=True)
    if r.returncode != 0:
        r = subprocess.run(base, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_abstract_new.restype = vp
        L.orc_abstract_new.argtypes = [i32, i32, vp, vp, vp, i32, vp, vp, i32, vp, vp]
        L.orc_abstract_free.argtypes = [vp]
        L.orc_arm_new.restype = vp
        L.orc_arm_new.argtypes = [i32, i32, vp, vp, vp, vp, vp, i32, vp, vp, vp, vp, i32, vp, vp]
        L.orc_arm_free.argtypes = [vp]
        L.orc_arm_set_offsets.argtypes = [vp, vp]
        L.orc_arm_total_penetration.argtypes = [vp, vp, i64, i32, vp]
        L.orc_abstract_config_free.argtypes = [vp, vp]
        L.orc_arm_config_free.argtypes = [vp, vp]
        L.orc_arm_fk.argtypes = [vp, vp, vp]
        L.orc_edge_free.argtypes = [i32, vp, vp, vp, i32, f64, i32, i64, i64, i64, vp, vp]
        L.orc_configs_free.argtypes = [i32, vp, vp, i64, i32, vp]
        L.orc_arm_configs_free_mask.argtypes = [vp, vp, i64, i32, C.c_uint32, vp]
        L.orc_edges_free.argtypes = [i32, vp, vp, vp, i64, i32, f64, i32, vp, i64, i64, vp, vp]
        L.orc_binary_indices.argtypes = [i64, vp]
        L.orc_sincos.argtypes = [f64, vp, vp]
        L.orc_np_sum.restype = f64
        L.orc_np_sum.argtypes = [vp, i64]
        L.orc_batch_dist.argtypes = [vp, vp, i64, i32, vp, i32, i32, vp]
        L.orc_dist_matrix.argtypes = [vp, i64, vp, i64, i32, vp, i32, i32, vp]
        L.orc_batch_cost.argtypes = [vp, vp, i64, i32, vp, i32, i32, i32, f64, i32, vp]
        L.orc_knn.argtypes = [vp, i64, vp, vp, vp, i32, vp, i32, i32, i32, vp, vp]
        L.orc_num_threads.restype = i32
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


METRICS = {"euclidean": 0, "sum_euclidean": 1, "max_euclidean": 2, "max": 3}


class OracleScene:
    """Owns an oracle-side scene (abstract point agents or sphere arms)."""

    def __init__(self, scene):
        L = lib()
        self._keep = []
        if hasattr(scene, "tables"):   # abstract point-agent scene
            t = scene.tables()
            self.kind = 0
            self.D = scene.q_dim
            arrs = [_c(t[k], np.int64 if k == "agent_offsets" else np.float64) for k in
                    ("agent_offsets", "pair_threshold", "agent_radius_sq", "box_lo", "box_hi", "sphere_pos", "sphere_threshold")]
            self._keep += arrs
            self.h = L.orc_abstract_new(len(scene.agent_radii), scene.dim, _p(arrs[0]), _p(arrs[1]), _p(arrs[2]),
                                        len(arrs[3]), _p(arrs[3]), _p(arrs[4]), len(arrs[5]), _p(arrs[5]), _p(arrs[6]))
        else:
            a = scene.arrays()
            self.kind = 1
            self.D = scene.q_dim
            self.S = len(a["sphere_radius"])
            self._keep.append(a)
            self.h = L.orc_arm_new(scene.n_robots, scene.q_dim, _p(a["q_offset"]), _p(a["base_kind"]), _p(a["base_pose"]),
                                   _p(a["n_links"]), _p(a["dh"]), self.S, _p(a["sphere_robot"]), _p(a["sphere_link"]),
                                   _p(a["sphere_local"]), _p(a["sphere_radius"]), len(a["box_lo"]), _p(a["box_lo"]),
                                   _p(a["box_hi"]))
            off = getattr(scene, "joint_offset", None)
            if self.h and off is not None:
                o = _c(np.asarray(off, dtype=np.float64).reshape(-1), np.float64)
                self._keep.append(o)
                if L.orc_arm_set_offsets(self.h, _p(o)) != 0:
                    raise ValueError("oracle rejected the joint offsets")
        if not self.h:
            raise ValueError("oracle rejected the scene")

    def __del__(self):
        try:
            if self.h:
                (lib().orc_abstract_free if self.kind == 0 else lib().orc_arm_free)(self.h)
        except Exception:
            pass

    # per-configuration / per-edge verdicts -------------------------------
    def config_free(self, q) -> bool:
        q = _c(q, np.float64)
        fn = lib().orc_abstract_config_free if self.kind == 0 else lib().orc_arm_config_free
        return bool(fn(self.h, _p(q)))

    def configs_free(self, qs) -> np.ndarray:
        qs = _c(qs, np.float64).reshape(-1, self.D)
        out = np.zeros(len(qs), dtype=np.uint8)
        lib().orc_configs_free(self.kind, self.h, _p(qs), len(qs), self.D, _p(out))
        return out

    def total_penetration(self, qs) -> np.ndarray:
        """Total penetration depth per configuration (arm scenes; the
        library's mrmg_arm_total_penetration)."""
        qs = _c(qs, np.float64).reshape(-1, self.D)
        out = np.zeros(len(qs))
        if lib().orc_arm_total_penetration(self.h, _p(qs), len(qs), self.D, _p(out)) != 0:
            raise ValueError("total penetration needs an arm scene")
        return out

    def configs_free_for_robots(self, qs, robot_mask: int) -> np.ndarray:
        """is_collision_free_for_robot for the robots in robot_mask (arm scenes)."""
        qs = _c(qs, np.float64).reshape(-1, self.D)
        out = np.zeros(len(qs), dtype=np.uint8)
        lib().orc_arm_configs_free_mask(self.h, _p(qs), len(qs), self.D, int(robot_mask), _p(out))
        return out

    def edge_free(self, q1, q2, resolution, include_endpoints=False, N_start=0, N_max=None, N=None, count=False):
        q1 = _c(q1, np.float64)
        q2 = _c(q2, np.float64)
        st = C.c_int(0)
        cnt = C.c_int64(0)
        r = lib().orc_edge_free(self.kind, self.h, _p(q1), _p(q2), self.D, float(resolution), int(include_endpoints),
                                0 if N is None else int(N), int(N_start), -1 if N_max is None else int(N_max),
                                C.addressof(st), C.addressof(cnt))
        if st.value == -1:
            raise ValueError("bad edge")
        return (bool(r), cnt.value) if count else bool(r)

    def edges_free(self, q1, q2, resolution, include_endpoints=False, N=None, N_start=0, N_max=None, count=False):
        q1 = _c(q1, np.float64).reshape(-1, self.D)
        q2 = _c(q2, np.float64).reshape(-1, self.D)
        Nn = None if N is None else _c(N, np.int64)
        out = np.zeros(len(q1), dtype=np.uint8)
        tot = C.c_int64(0)
        rc = lib().orc_edges_free(self.kind, self.h, _p(q1), _p(q2), len(q1), self.D, float(resolution),
                                  int(include_endpoints), _p(Nn), int(N_start), -1 if N_max is None else int(N_max),
                                  _p(out), C.addressof(tot))
        if rc != 0:
            raise ValueError("bad edge in batch")
        return (out, tot.value) if count else out

    def sphere_centers(self, q) -> np.ndarray:
        assert self.kind == 1
        q = _c(q, np.float64)
        out = np.zeros((self.S, 3))
        lib().orc_arm_fk(self.h, _p(q), _p(out))
        return out


# ---------------------------------------------------------------------------
# integer / ordering helpers
# ---------------------------------------------------------------------------
def binary_search_indices(N: int) -> tuple:
    """generate_binary_search_indices (problems/planning_env.py:34-51), C."""
    out = np.zeros(max(N, 0), dtype=np.int64)
    lib().orc_binary_indices(int(N), _p(out))
    return tuple(int(x) for x in out)


def binary_search_indices_py(N: int) -> tuple:
    """Pure-Python mirror of planning_env.py:34-51 (small N only)."""
    seq = [0] * N
    dq = deque([(0, N - 1)])
    i = 0
    while dq:
        s, e = dq.popleft()
        m = (s + e) // 2
        seq[i] = m
        i += 1
        if s <= m - 1:
            dq.append((s, m - 1))
        if m + 1 <= e:
            dq.append((m + 1, e))
    return tuple(seq)


def sincos(x: float):
    s = C.c_double(0)
    c = C.c_double(0)
    lib().orc_sincos(float(x), C.addressof(s), C.addressof(c))
    return s.value, c.value


def np_sum(a) -> float:
    a = _c(a, np.float64)
    return lib().orc_np_sum(_p(a), len(a))


# ---------------------------------------------------------------------------
# distances / costs (problems/core/configuration.py)
# ---------------------------------------------------------------------------
def _slices(slices):
    return _c(np.asarray(slices).reshape(-1, 2), np.int64)


def batch_dist(pt, batch, slices, metric) -> np.ndarray:
    pt = _c(pt, np.float64)
    batch = _c(batch, np.float64).reshape(-1, len(pt))
    sl = _slices(slices)
    out = np.zeros(len(batch))
    lib().orc_batch_dist(_p(pt), _p(batch), len(batch), len(pt), _p(sl), len(sl), METRICS[metric], _p(out))
    return out


def dist_matrix(qs, nodes, slices, metric) -> np.ndarray:
    qs = _c(qs, np.float64)
    nodes = _c(nodes, np.float64)
    sl = _slices(slices)
    out = np.zeros((len(qs), len(nodes)))
    lib().orc_dist_matrix(_p(qs), len(qs), _p(nodes), len(nodes), qs.shape[1], _p(sl), len(sl), METRICS[metric], _p(out))
    return out


def batch_cost(starts, ends, slices, metric="euclidean", reduction="max", w=0.01, mode=None) -> np.ndarray:
    """mode 0: one start vs many ends; 1: row-wise; 2: path (consecutive)."""
    starts = _c(starts, np.float64)
    sl = _slices(slices)
    if mode is None:
        mode = 2 if ends is None else (0 if starts.ndim == 1 else 1)
    D = starts.shape[-1]
    if mode == 2:
        M = starts.shape[0] - 1
        ends_a = None
    else:
        ends_a = _c(ends, np.float64).reshape(-1, D)
        M = len(ends_a)
    out = np.zeros(max(M, 0))
    rc = lib().orc_batch_cost(_p(starts), _p(ends_a), M, D, _p(sl), len(sl), {"euclidean": 0, "max": 1}[metric],
                              {"max": 0, "sum": 1}[reduction], float(w), mode, _p(out))
    if rc != 0:
        raise ValueError("unsupported cost shape")
    return out


def knn(qs, q_mode, nodes, mode_off, slices, metric, k):
    qs = _c(qs, np.float64)
    q_mode = _c(q_mode, np.int32)
    nodes = _c(nodes, np.float64)
    mode_off = _c(mode_off, np.int64)
    sl = _slices(slices)
    idx = np.zeros((len(qs), k), dtype=np.int64)
    dist = np.zeros((len(qs), k))
    lib().orc_knn(_p(qs), len(qs), _p(q_mode), _p(nodes), _p(mode_off), qs.shape[1], _p(sl), len(sl), METRICS[metric],
                  int(k), _p(idx), _p(dist))
    return idx, dist


def near(qs, q_mode, nodes, mode_off, slices, metric, radius, add_eps=1e-10):
    """Radius neighbours per mode as RRT* near (planners/rrtstar_base.py:1296-1337)
    selects them: batch_config_dist of the query against its mode's nodes, then
    find_nearest_indices (rrtstar_base.py:439-453): r += 1e-10 in FP64 and
    np.nonzero(dists <= r), ascending.  CSR result (offsets, idx, dist)."""
    qs = _c(qs, np.float64)
    q_mode = np.asarray(q_mode).reshape(-1)
    nodes = _c(nodes, np.float64)
    mode_off = np.asarray(mode_off, dtype=np.int64)
    radius = np.broadcast_to(np.asarray(radius, dtype=np.float64), (len(qs),))
    offs, idx, dist = [0], [], []
    for i in range(len(qs)):
        lo, hi = mode_off[q_mode[i]], mode_off[q_mode[i] + 1]
        d = batch_dist(qs[i], nodes[lo:hi], slices, metric) if hi > lo else np.zeros(0)
        r = radius[i] + add_eps
        sel = np.nonzero(d <= r)[0]
        idx.append(sel.astype(np.int64))
        dist.append(d[sel])
        offs.append(offs[-1] + len(sel))
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
    return np.array(offs, dtype=np.int64), cat(idx, np.int64), cat(dist, np.float64)


def batch_free_batched_form(scene, qs) -> bool:
    """AbstractEnvironment._batch_is_collision_free (abstract_env.py:278-299):
    True iff no configuration of qs [n, D] collides, with the obstacle tests
    in their batched numpy forms -- Rectangle.batch_collides_with_sphere
    (:86-104: clip, np.sum of squares along axis 1, <= r^2) and
    Sphere.batch_collides_with_sphere (:52-55: np.linalg.norm along axis 1,
    i.e. rounded squares, numpy's sum and sqrt, < r_o + r) -- and the agent
    pairs as the single check tests them (np.linalg.norm of one vector, < r_i +
    r_j).  numpy restatement: it computes what the reference's numpy calls
    compute on this host."""
    t = scene.tables()
    qs = np.asarray(qs, dtype=np.float64).reshape(len(qs), -1)
    A, dim = len(scene.agent_radii), scene.dim
    off = t["agent_offsets"]
    for i in range(A):
        c = qs[:, off[i]:off[i] + dim]
        r = scene.agent_radii[i]
        for o in range(len(scene.sphere_radius)):
            if (np.linalg.norm(t["sphere_pos"][o] - c, axis=1) < scene.sphere_radius[o] + r).any():
                return False
        for b in range(len(t["box_lo"])):
            closest = np.clip(c, t["box_lo"][b], t["box_hi"][b])
            if (np.sum((closest - c) ** 2, axis=1) <= r ** 2).any():
                return False
    for k in range(len(qs)):
        for i in range(A):
            for j in range(i + 1, A):
                if np.linalg.norm(qs[k, off[i]:off[i] + dim] - qs[k, off[j]:off[j] + dim]) < \
                        scene.agent_radii[i] + scene.agent_radii[j]:
                    return False
    return True


def num_threads() -> int:
    return int(lib().orc_num_threads())
