"""CPU property test of the tensor-core k-NN path's certificate: a numpy
restatement of the candidate kernel's kept lists (packed distance/index
keys, the row filter, the threshold shared between the chunks of a query and
the per-chunk bound) and of the merge's certification (tau from the k-th
smallest upper key end plus twice the error bound, FP64 re-rank of the
candidates whose lower key end is within tau).  Whenever the merge
certifies a query, its answer must be the exact top-k by (distance, index)
over all nodes -- the property the device path relies on before it skips
the exact kernels.  Approximate distances carry errors up to the bound."""
import numpy as np
import pytest

KEEP = 16
EMPTY = np.uint32(0x7F7FFFFF)


def _mask(chunk_nodes: int) -> np.uint32:
    b = 1
    while (1 << b) <= chunk_nodes:
        b += 1
    return np.uint32((1 << b) - 1)


def _f(u) -> np.float32:
    return np.array([u], dtype=np.uint32).view(np.float32)[0]


def _u(x) -> np.uint32:
    return np.array([x], dtype=np.float32).view(np.uint32)[0]


def _lower(key, m):
    return _f(np.uint32(key) & ~m)


def _upper(key, m):
    return _f(np.uint32(key) | m)


def _insert(kk: list, key: np.uint32):
    """The kernel's branch-free insert: one unsigned max and min per slot."""
    for i in range(KEEP - 1, 0, -1):
        kk[i] = min(kk[i], max(kk[i - 1], key))
    kk[0] = min(kk[0], key)


def _candidates(approx: np.ndarray, chunk_nodes: int, tile: int, rng, extra_marks: float):
    """Every chunk's kept list, scanned tile by tile in round-robin order
    over the chunks (as concurrent CTAs would), each chunk reading the
    shared threshold one tile late.  Returns per chunk (lower ends, indices,
    bound)."""
    n = len(approx)
    m = _mask(chunk_nodes)
    chunks = [(c0, min(n, c0 + chunk_nodes)) for c0 in range(0, n, chunk_nodes)]
    st = []
    for c0, c1 in chunks:
        st.append({"kk": [EMPTY] * KEEP, "bound": np.float32(np.inf), "gcur": np.float32(np.inf),
                   "gnext": np.float32(np.inf), "pub": np.float32(np.inf), "t": c0, "end": c1, "c0": c0})
    g = np.float32(np.inf)
    live = True
    while live:
        live = False
        for s in st:
            if s["t"] >= s["end"]:
                continue
            live = True
            s["gnext"] = g                               # read one tile ahead
            t0, t1 = s["t"], min(s["end"], s["t"] + tile)
            for c in range(t0, t1, 32):
                thr = min(_lower(s["kk"][-1], m), s["gcur"])
                vals = approx[c:min(t1, c + 32)]
                marks = vals < thr
                marks |= rng.random(len(vals)) < extra_marks   # the dot-space marks are a superset
                for i in np.nonzero(marks)[0]:
                    d = np.float32(max(vals[i], np.float32(0.0)))
                    key = np.uint32((_u(d) & ~m) | np.uint32(c - s["c0"] + i))
                    if key < s["kk"][-1]:
                        _insert(s["kk"], key)
            s["t"] = t1
            s["bound"] = min(s["bound"], s["gcur"])
            up = _upper(s["kk"][-1], m)
            if up < s["pub"]:
                s["pub"] = up
                g = min(g, up)
            s["gcur"] = min(s["gcur"], s["gnext"])
    out = []
    for s in st:
        kk = s["kk"]
        lows = np.array([np.inf if (k & m) == m else _lower(k, m) for k in kk], dtype=np.float32)
        idx = np.array([-1 if (k & m) == m else s["c0"] + int(k & m) for k in kk], dtype=np.int64)
        e15 = (kk[-1] & m) == m
        out.append((lows, idx, np.float32(min(s["bound"], np.inf if e15 else _lower(kk[-1], m)))))
    return out, m


def _merge(lists, m, eps: np.float32, exact: np.ndarray, k: int):
    """The merge: None when uncertified, else the top-k indices."""
    heads = [0] * len(lists)
    kth = np.float32(np.inf)
    for _ in range(k):
        best, who = np.float32(np.inf), -1
        for c, (lows, _, _) in enumerate(lists):
            if heads[c] < KEEP and lows[heads[c]] != np.inf:
                v = _upper(_u(lows[heads[c]]), m)
                if v < best:
                    best, who = v, c
        kth = best
        if who < 0:
            break
        heads[who] += 1
    tau = np.float32(np.inf) if kth == np.inf else np.float32(kth + np.float32(2.0) * eps)
    if any(not (b > tau) for _, _, b in lists):
        return None
    cand = [int(i) for lows, idx, _ in lists for lo, i in zip(lows, idx) if lo <= tau and i >= 0]
    cand.sort(key=lambda i: (exact[i], i))
    return cand[:k]


@pytest.mark.parametrize("seed", range(40))
def test_certified_answers_are_exact(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(300, 2500))
    kind = seed % 5
    if kind == 0:      # spread distances
        exact = rng.uniform(0.5, 40.0, n)
    elif kind == 1:    # clustered near the minimum: ties within the error bound
        exact = 4.0 + rng.uniform(0, 1e-3, n)
    elif kind == 2:    # exact duplicates
        exact = np.repeat(rng.uniform(1.0, 9.0, n // 20 + 1), 20)[:n]
    elif kind == 3:    # near ties below the key truncation
        exact = 2.0 * (1.0 + 1e-6 * rng.permutation(n))
    else:              # distances near 0: approximate values below 0 (clamped in the keys)
        exact = rng.uniform(0.0, 2e-3, n)
    eps = np.float32(10 ** rng.uniform(-6, -2))
    approx = (exact + rng.uniform(-1, 1, n) * float(eps)).astype(np.float32)
    chunk_nodes = int(rng.choice([128, 384, 1024, 4096]))
    k = int(rng.choice([1, 5, 10, 16]))
    lists, m = _candidates(approx, chunk_nodes, 128, rng, extra_marks=float(rng.choice([0.0, 0.05])))
    got = _merge(lists, m, eps, exact, k)
    want = sorted(range(n), key=lambda i: (exact[i], i))[:k]
    if got is not None:
        assert got == want
    else:   # uncertified: the device hands the query to the exact kernels
        assert kind in (1, 2, 3, 4) or eps > 1e-3


def test_spread_distances_certify():
    """On well separated distances the certificate holds (the fast path is
    taken), so the property above is not satisfied vacuously."""
    rng = np.random.default_rng(99)
    n = 2000
    exact = rng.uniform(0.5, 40.0, n)
    eps = np.float32(1e-5)
    approx = (exact + rng.uniform(-1, 1, n) * float(eps)).astype(np.float32)
    lists, m = _candidates(approx, 512, 128, rng, extra_marks=0.0)
    got = _merge(lists, m, eps, exact, 10)
    assert got == sorted(range(n), key=lambda i: (exact[i], i))[:10]
