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
