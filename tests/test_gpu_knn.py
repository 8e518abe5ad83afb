"""GPU parity for per-mode nearest neighbours: indices bit-identical to the
reference's selection (golden vectors) and to the oracle; distances are the
reference's FP64 values."""
import numpy as np
import pytest
import torch

from conftest import golden, pkg

pytestmark = pytest.mark.gpu


def test_umma_selftest(gpu):
    knn = pkg("knn")
    g = torch.Generator().manual_seed(0)
    for n in (32, 128, 256):
        a = (torch.rand((128, 64), generator=g) * 4 - 2).to(torch.bfloat16).cuda()
        b = (torch.rand((n, 64), generator=g) * 4 - 2).to(torch.bfloat16).cuda()
        c = knn.selftest_umma(a, b).double().cpu()
        ref = a.double().cpu() @ b.double().cpu().T
        bound = 64 * 2.0 ** -23 * (a.double().abs().cpu() @ b.double().abs().cpu().T) + 1e-30
        assert torch.all((c - ref).abs() <= bound), float((c - ref).abs().max())


def test_knn_exact_golden(gpu, oracle):
    knn = pkg("knn")
    g = golden("knn.npz")
    for metric in ["euclidean", "max_euclidean"]:
        idx, dist = knn.knn_exact(g["queries"], g["q_mode"], g["nodes"], g["mode_off"], g["slices"], metric,
                                  int(g["k"]))
        assert np.array_equal(idx.cpu().numpy(), g[f"idx_{metric}"]), metric
        oi, od = oracle.knn(g["queries"], g["q_mode"], g["nodes"], g["mode_off"], g["slices"], metric, int(g["k"]))
        assert np.array_equal(idx.cpu().numpy(), oi) and np.array_equal(dist.cpu().numpy(), od)


def test_knn_exact_all_metrics_vs_oracle(gpu, oracle):
    knn = pkg("knn")
    rng = np.random.default_rng(8)
    D, sl = 12, [[0, 5], [5, 9], [9, 12]]
    nodes = rng.uniform(-3, 3, (3000, D))
    off = np.array([0, 1200, 1200, 2990, 3000])          # an empty mode and a 10-node mode
    qs = rng.uniform(-3, 3, (200, D))
    qm = rng.integers(0, 4, 200).astype(np.int32)
    for metric in ["euclidean", "sum_euclidean", "max_euclidean", "max"]:
        for k in (1, 10, 40):
            idx, dist = knn.knn_exact(qs, qm, nodes, off, sl, metric, k)
            oi, od = oracle.knn(qs, qm, nodes, off, sl, metric, k)
            assert np.array_equal(idx.cpu().numpy(), oi), (metric, k)
            assert np.array_equal(dist.cpu().numpy(), od), (metric, k)


@pytest.mark.parametrize("path", ["tensor_core", "exact", "auto"])
def test_knn_store_golden(gpu, path):
    knn = pkg("knn")
    g = golden("knn.npz")
    for metric in ["euclidean", "max_euclidean"]:
        store = knn.NodeStore(g["nodes"], g["mode_off"], g["slices"], metric, path=path)
        idx, dist = store.knn(g["queries"], g["q_mode"], int(g["k"]))
        assert store.last_stats["tensor_core"] == (path == "tensor_core")
        assert np.array_equal(idx.cpu().numpy(), g[f"idx_{metric}"]), metric


@pytest.mark.parametrize("path", ["auto", "exact"])
@pytest.mark.parametrize("metric", ["euclidean", "max_euclidean"])
def test_knn_workload_vs_oracle(gpu, oracle, metric, path):
    """The per-mode workload (Zipf modes, clustered nodes) at reduced size:
    indices and FP64 distances identical to the oracle's exact selection
    (the automatic path takes the tensor cores at this size)."""
    knn, scenes = pkg("knn"), pkg("scenes")
    w = scenes.make_knn_workload(seed=3, n_nodes=40_000, n_queries=1024)
    store = knn.NodeStore(w["nodes"], w["mode_offsets"], w["slices"], metric, path=path)
    for k in (1, 10, 16):
        idx, dist = store.knn(w["queries"], w["q_mode"], k)
        oi, od = oracle.knn(w["queries"], w["q_mode"], w["nodes"], w["mode_offsets"], w["slices"], metric, k)
        assert np.array_equal(idx.cpu().numpy(), oi), (metric, k)
        assert np.array_equal(dist.cpu().numpy(), od), (metric, k)
        assert store.last_stats["tensor_core"] == (path == "auto")
        assert store.last_stats["rerun_exact"] < 0.05 * len(w["queries"])


@pytest.mark.parametrize("path", ["auto", "tensor_core", "exact"])
def test_knn_store_other_metrics_and_edge_modes(gpu, oracle, path):
    """Metrics outside the tensor-core shapes and k > 16 use the exact kernels;
    empty and tiny modes pad with index -1 / +inf like the oracle."""
    knn = pkg("knn")
    rng = np.random.default_rng(9)
    nodes = rng.uniform(-2, 2, (2000, 14))
    off = np.array([0, 0, 5, 1990, 2000])
    qs = rng.uniform(-2, 2, (100, 14))
    qm = rng.integers(0, 4, 100).astype(np.int32)
    sl = [[0, 7], [7, 14]]
    for metric, k in [("sum_euclidean", 10), ("max", 10), ("euclidean", 20), ("euclidean", 10), ("max_euclidean", 12),
                      ("max", 40)]:
        store = knn.NodeStore(nodes, off, sl, metric, path=path)
        idx, dist = store.knn(qs, qm, k)
        oi, od = oracle.knn(qs, qm, nodes, off, sl, metric, k)
        assert np.array_equal(idx.cpu().numpy(), oi), (metric, k)
        assert np.array_equal(dist.cpu().numpy(), od), (metric, k)


def _csr_equal(got, want):
    offs, idx, dist = (x.cpu().numpy() for x in got)
    wo, wi, wd = want
    return np.array_equal(offs, wo) and np.array_equal(idx, wi) and np.array_equal(dist, wd)


@pytest.mark.parametrize("path", ["tensor_core", "exact"])
def test_near_golden(gpu, oracle, path):
    """Radius neighbours against the reference's find_nearest_indices (radii
    on, just inside and just outside node distances by less than the added
    1e-10; an empty and a one-node mode)."""
    knn = pkg("knn")
    g = golden("near.npz")
    for metric in ["euclidean", "max_euclidean"]:
        store = knn.NodeStore(g["nodes"], g["mode_off"], g["slices"], metric, path=path)
        offs, idx, dist = store.near(g["queries"], g["q_mode"], g[f"radius_{metric}"])
        assert np.array_equal(offs.cpu().numpy(), g[f"offsets_{metric}"]), metric
        assert np.array_equal(idx.cpu().numpy(), g[f"idx_{metric}"]), metric
        want = oracle.near(g["queries"], g["q_mode"], g["nodes"], g["mode_off"], g["slices"], metric,
                           g[f"radius_{metric}"])
        assert _csr_equal((offs, idx, dist), want), metric


@pytest.mark.parametrize("path", ["auto", "exact"])
@pytest.mark.parametrize("metric", ["euclidean", "max_euclidean"])
def test_near_workload_vs_oracle(gpu, oracle, metric, path):
    """The per-mode workload at reduced size, radii at the 24th-nearest
    distance (some lowered by 0.5e-10, so that only the added epsilon keeps the
    node), a tiny output capacity (the fetch path) and r = 0."""
    knn, scenes = pkg("knn"), pkg("scenes")
    w = scenes.make_knn_workload(seed=4, n_nodes=40_000, n_queries=512)
    _, od = oracle.knn(w["queries"], w["q_mode"], w["nodes"], w["mode_offsets"], w["slices"], metric, 24)
    r = od[:, -1].copy()
    r[::3] -= 0.5e-10
    r[~np.isfinite(r)] = 1.0
    store = knn.NodeStore(w["nodes"], w["mode_offsets"], w["slices"], metric, path=path)
    want = oracle.near(w["queries"], w["q_mode"], w["nodes"], w["mode_offsets"], w["slices"], metric, r)
    assert want[0][-1] > 0
    assert _csr_equal(store.near(w["queries"], w["q_mode"], r), want)
    assert _csr_equal(store.near(w["queries"], w["q_mode"], r, cap=7), want)
    offs, idx, dist = store.near(w["queries"], w["q_mode"], r, distances=False)
    assert dist is None and np.array_equal(offs.cpu().numpy(), want[0]) and np.array_equal(idx.cpu().numpy(), want[1])
    z = oracle.near(w["queries"], w["q_mode"], w["nodes"], w["mode_offsets"], w["slices"], metric, 0.0)
    assert _csr_equal(store.near(w["queries"], w["q_mode"], 0.0), z)


@pytest.mark.parametrize("path", ["auto", "tensor_core", "exact"])
def test_near_other_metrics_and_edge_modes(gpu, oracle, path):
    """Metrics outside the tensor-core shapes check every node in FP64; empty
    and tiny modes, negative and infinite radii, and no queries at all."""
    knn = pkg("knn")
    rng = np.random.default_rng(10)
    nodes = rng.uniform(-2, 2, (2000, 14))
    off = np.array([0, 0, 5, 1990, 2000])
    qs = rng.uniform(-2, 2, (100, 14))
    qm = rng.integers(0, 4, 100).astype(np.int32)
    sl = [[0, 7], [7, 14]]
    r = rng.uniform(0.5, 4.0, 100)
    r[5], r[6] = -1.0, np.inf
    for metric in ["sum_euclidean", "max", "euclidean", "max_euclidean"]:
        store = knn.NodeStore(nodes, off, sl, metric, path=path)
        want = oracle.near(qs, qm, nodes, off, sl, metric, r)
        assert _csr_equal(store.near(qs, qm, r), want), metric
        offs, idx, dist = store.near(qs[:0], qm[:0], 1.0)
        assert offs.cpu().tolist() == [0] and idx.numel() == 0


class _HostModes:
    """Host mirror of a growing per-mode node store (insertion order, removal
    by moving the last node into the freed slot, as SingleTree does)."""

    def __init__(self, dim):
        self.dim = dim
        self.modes = []

    def append(self, m, rows):
        while len(self.modes) <= m:
            self.modes.append(np.zeros((0, self.dim)))
        self.modes[m] = np.concatenate([self.modes[m], np.asarray(rows).reshape(-1, self.dim)])

    def remove(self, m, i):
        a = self.modes[m]
        a[i] = a[-1]
        self.modes[m] = a[:-1]

    def arrays(self):
        off = np.concatenate([[0], np.cumsum([len(a) for a in self.modes])]).astype(np.int64)
        return np.concatenate(self.modes), off


@pytest.mark.parametrize("metric,path", [("euclidean", "tensor_core"), ("max_euclidean", "tensor_core"),
                                         ("sum_euclidean", "auto"), ("euclidean", "exact")])
def test_node_store_incremental(gpu, oracle, metric, path):
    """A store grown by appends (single rows across tile boundaries and
    capacity doublings, batches, modes created past the last) and shrunk by
    removals answers k-NN and radius queries like the oracle over the same
    per-mode arrays."""
    knn, scenes = pkg("knn"), pkg("scenes")
    w = scenes.make_knn_workload(seed=6, n_nodes=12_000, n_modes=4, n_queries=256)
    nodes, off, sl = w["nodes"], w["mode_offsets"], w["slices"]
    rng = np.random.default_rng(11)
    host = _HostModes(nodes.shape[1])
    half = [off[m] + (off[m + 1] - off[m]) // 2 for m in range(4)]
    first = np.concatenate([nodes[off[m]:half[m]] for m in range(4)])
    first_off = np.concatenate([[0], np.cumsum([half[m] - off[m] for m in range(4)])])
    store = knn.NodeStore(first, first_off, sl, metric, path=path)
    for m in range(4):
        host.append(m, nodes[off[m]:half[m]])
    # RRT-style single rows into mode 1, PRM-style batches elsewhere, a new mode 6
    for r in nodes[half[1]:half[1] + 700]:
        store.append(1, r)
        host.append(1, r)
    for m in (0, 2, 3):
        rows = nodes[half[m]:off[m + 1]]
        for chunk in np.array_split(rows, 3):
            store.append(m, torch.from_numpy(chunk).cuda())
            host.append(m, chunk)
    extra = rng.normal(0, 1.0, (300, nodes.shape[1]))
    store.append(6, extra)
    host.append(6, extra)
    for m, i in [(1, 0), (1, 5), (0, 17), (6, 299), (2, 3)]:
        store.remove(m, i)
        host.remove(m, i)
    assert store.n_modes == 7 and store.size(5) == 0
    assert [store.size(m) for m in range(7)] == [len(a) for a in host.modes]
    allnodes, alloff = host.arrays()
    qm = rng.integers(0, 7, 256).astype(np.int32)
    qs = w["queries"][:256]
    for k in (1, 10):
        idx, dist = store.knn(qs, qm, k)
        oi, od = oracle.knn(qs, qm, allnodes, alloff, sl, metric, k)
        assert np.array_equal(idx.cpu().numpy(), oi), (metric, k)
        assert np.array_equal(dist.cpu().numpy(), od), (metric, k)
    _, od = oracle.knn(qs, qm, allnodes, alloff, sl, metric, 12)
    r = np.where(np.isfinite(od[:, -1]), od[:, -1], 1.0)
    assert _csr_equal(store.near(qs, qm, r), oracle.near(qs, qm, allnodes, alloff, sl, metric, r))


def test_node_store_grow_from_empty(gpu, oracle):
    """An empty store filled one node at a time, queried as it grows (the RRT
    loop: nearest, near, add)."""
    knn = pkg("knn")
    rng = np.random.default_rng(12)
    D, sl = 8, [[0, 4], [4, 8]]
    store = knn.NodeStore.empty(D, 2, sl, "euclidean")
    host = _HostModes(D)
    for step in range(300):
        m = int(rng.integers(0, 2))
        q = rng.uniform(-1, 1, (1, D))
        if store.size(m) > 0:
            allnodes, alloff = host.arrays()
            idx, dist = store.knn(q, [m], 1)
            oi, od = oracle.knn(q, [m], allnodes, alloff, sl, "euclidean", 1)
            assert np.array_equal(idx.cpu().numpy(), oi) and np.array_equal(dist.cpu().numpy(), od), step
            got = store.near(q, [m], 0.6)
            assert _csr_equal(got, oracle.near(q, [m], allnodes, alloff, sl, "euclidean", 0.6)), step
        store.append(m, q)
        host.append(m, q)
    assert store.size(0) + store.size(1) == 300
    # a mode index past the last creates the modes between, empty; one at or
    # beyond the store's mode limit is refused and leaves the store as it was
    store.append(5, rng.uniform(-1, 1, (2, D)))
    assert store.n_modes == 6 and store.size(3) == 0 and store.size(5) == 2
    with pytest.raises(ValueError):
        store.append(pkg("_lib").MRMG_MAX_STORE_MODES, np.zeros((1, D)))
    assert store.n_modes == 6 and store.size(0) + store.size(1) == 300
    allnodes, alloff = host.arrays()
    q = rng.uniform(-1, 1, (4, D))
    oi, _ = oracle.knn(q, [0, 1, 0, 1], allnodes, alloff, sl, "euclidean", 3)
    assert np.array_equal(store.knn(q, [0, 1, 0, 1], 3)[0].cpu().numpy(), oi)


@pytest.mark.parametrize("path", ["tensor_core", "exact"])
def test_knn_uncertified_queries_rerun(gpu, oracle, path):
    """Nodes repeated many times fill the kept candidate lists with ties, so
    the certificate (of the tensor-core path, or of the node-parallel FP32
    candidate pass) fails and those queries are answered by the node-parallel
    FP64 kernels; the result is still the oracle's (ties to the lower index)."""
    knn = pkg("knn")
    rng = np.random.default_rng(13)
    base = rng.uniform(-1, 1, (40, 28))
    nodes = np.concatenate([np.repeat(base, 150, axis=0), rng.uniform(-1, 1, (3000, 28))])
    off = np.array([0, 6000, len(nodes)])
    qs = np.concatenate([base[:20] + 1e-3, rng.uniform(-1, 1, (200, 28))])
    qm = np.concatenate([np.zeros(20, np.int32), rng.integers(0, 2, 200).astype(np.int32)])
    sl = [[0, 7], [7, 14], [14, 21], [21, 28]]
    store = knn.NodeStore(nodes, off, sl, "euclidean", path=path)
    for k in (10, 16):
        idx, dist = store.knn(qs, qm, k)
        oi, od = oracle.knn(qs, qm, nodes, off, sl, "euclidean", k)
        assert np.array_equal(idx.cpu().numpy(), oi), k
        assert np.array_equal(dist.cpu().numpy(), od), k
        assert store.last_stats["rerun_exact"] >= 20


def test_knn_near_ties_below_key_resolution(gpu, oracle):
    """Nodes on shells around each query whose squared distances differ by a
    relative 1e-6, far below the truncated distance in the tensor-core
    path's packed keys (the low bits of a key hold the node's index): the
    certificate widens tau by the truncation and the FP64 re-rank (or the
    exact rerun) orders them, so indices and distances are the oracle's."""
    knn = pkg("knn")
    rng = np.random.default_rng(21)
    D, Q, per = 28, 64, 200
    qs = rng.uniform(-1, 1, (Q, D))
    dirs = rng.normal(size=(Q, per, D))
    dirs /= np.linalg.norm(dirs, axis=2, keepdims=True)
    radii = 0.5 * (1.0 + 1e-6 * rng.permutation(per))[None, :, None]
    shell = (qs[:, None, :] + dirs * radii).reshape(-1, D)
    nodes = np.concatenate([shell, rng.uniform(-1, 1, (20_000, D))])
    off = np.array([0, len(nodes)])
    qm = np.zeros(Q, np.int32)
    sl = [[0, 7], [7, 14], [14, 21], [21, 28]]
    store = knn.NodeStore(nodes, off, sl, "euclidean", path="tensor_core")
    for k in (10, 16):
        idx, dist = store.knn(qs, qm, k)
        assert store.last_stats["tensor_core"]
        oi, od = oracle.knn(qs, qm, nodes, off, sl, "euclidean", k)
        assert np.array_equal(idx.cpu().numpy(), oi), k
        assert np.array_equal(dist.cpu().numpy(), od), k


def test_knn_large_chunks_match_the_exact_kernel(gpu):
    """A batch large enough that each work item scans 64+ node tiles (14
    index bits in the candidate keys, 9 mantissa bits left for the distance):
    indices and distances equal the exact FP64 kernel's (which is
    bit-identical to the oracle), for both metrics."""
    knn = pkg("knn")
    rng = np.random.default_rng(22)
    D, sl = 8, [[0, 4], [4, 8]]
    nodes = np.concatenate([rng.normal(size=(48_000, D)), rng.uniform(-2, 2, (8_000, D))])
    off = np.array([0, 48_000, len(nodes)])
    qs = rng.uniform(-2, 2, (12_000, D))
    qm = (rng.uniform(size=12_000) < 0.9).astype(np.int32) ^ 1
    for metric in ("euclidean", "max_euclidean"):
        store = knn.NodeStore(nodes, off, sl, metric, path="tensor_core")
        idx, dist = store.knn(qs, qm, 10)
        assert store.last_stats["tensor_core"]
        ei, ed = knn.knn_exact(qs, qm, nodes, off, sl, metric, 10)
        assert torch.equal(idx.cpu(), ei.cpu()), metric
        assert torch.equal(dist.cpu(), ed.cpu()), metric
        store.close()
