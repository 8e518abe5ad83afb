"""The edge check that allocates nothing, for callers that cannot allocate
device memory while checking edges (a planner step recorded into a CUDA
graph, a real-time loop that forbids allocation after start-up, a process
whose memory pool owns the device).  It is called through the C ABI and must
return exactly the verdicts of the regular entry point, on two calls in a
row (the shared static scratch keeps the previous call's contents)."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import pkg

pytestmark = pytest.mark.gpu


def _call(lib, fn, scene, q1, q2, res, out, N_start=0, N_max=-1):
    return fn(scene.h, q1.data_ptr(), q2.data_ptr(), 0 if q1.dtype == torch.float32 else 1, q1.shape[0], res, 0,
              None, N_start, N_max, out.data_ptr(), torch.cuda.current_stream().cuda_stream, 0)


def _cases():
    scenes = pkg("scenes")
    dense = scenes.make_arm_scene(0)
    w = scenes.make_arm_workload(dense, seed=21, n_configs=10, n_edges=12000)
    sparse = scenes.make_arm_scene(1, n_boxes=5)
    rng = np.random.default_rng(4)
    a = scenes.uniform_configs(sparse, 6000, seed=22, dtype=np.float32)
    b = (a + rng.uniform(-0.2, 0.2, a.shape)).astype(np.float32)
    disc = scenes.make_disc_scene(0)
    dw = scenes.make_disc_workload(0, n_configs=10, n_edges=3000)
    return [(dense, w["q1"], w["q2"], 0.05), (sparse, a, b, 0.02), (disc, dw["q1"], dw["q2"], 0.01)]


def test_noalloc_matches_regular_entry_point(gpu):
    lib = pkg("_lib").load()
    col = pkg("collision")
    for scene, q1, q2, res in _cases():
        sc = col.Gb300Scene(scene)
        d1 = torch.from_numpy(np.ascontiguousarray(q1)).cuda()
        d2 = torch.from_numpy(np.ascontiguousarray(q2)).cuda()
        ref = torch.empty(d1.shape[0], dtype=torch.uint8, device="cuda")
        assert _call(lib, lib.mrmg_is_edge_collision_free_batch, sc, d1, d2, res, ref) == 0
        ref_np = ref.cpu().numpy()
        for _ in range(2):   # two calls in a row on the shared scratch
            out = torch.full((d1.shape[0],), 7, dtype=torch.uint8, device="cuda")
            rc = _call(lib, lib.mrmg_is_edge_collision_free_batch_noalloc, sc, d1, d2, res, out)
            assert rc == 0, lib.mrmg_last_error()
            assert np.array_equal(out.cpu().numpy(), ref_np)
        # a windowed call (N_start / N_max) as well
        ref2 = torch.empty_like(ref)
        out2 = torch.empty_like(ref)
        assert _call(lib, lib.mrmg_is_edge_collision_free_batch, sc, d1, d2, res, ref2, 1, 7) == 0
        assert _call(lib, lib.mrmg_is_edge_collision_free_batch_noalloc, sc, d1, d2, res, out2, 1, 7) == 0
        assert np.array_equal(out2.cpu().numpy(), ref2.cpu().numpy())


def test_noalloc_rejects_batches_over_the_limit(gpu):
    lib = pkg("_lib").load()
    scenes, col = pkg("scenes"), pkg("collision")
    sc = col.Gb300Scene(scenes.make_disc_scene(0))
    n = pkg("_lib").MRMG_NOALLOC_MAX_EDGES + 1
    d = torch.zeros((n, 4), dtype=torch.float64, device="cuda")
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    rc = _call(lib, lib.mrmg_is_edge_collision_free_batch_noalloc, sc, d, d, 0.01, out)
    assert rc == pkg("_lib").MRMG_ERR_ARG
    assert b"no-allocation limit" in lib.mrmg_last_error()


def test_noalloc_recorded_in_a_graph(gpu):
    """The case the entry point exists for: a call recorded into a CUDA graph
    with MRMG_FLAG_ASYNC (after one ordinary call has looked up the scratch
    address), replayed twice on new endpoints; each replay's verdicts equal
    the regular entry point's on the same endpoints."""
    lib = pkg("_lib").load()
    L = pkg("_lib")
    scenes, col = pkg("scenes"), pkg("collision")
    scene = scenes.make_arm_scene(1, n_boxes=5)
    sc = col.Gb300Scene(scene)
    n = 4000
    rng = np.random.default_rng(31)
    sets = []
    for seed in (41, 42):
        a = scenes.uniform_configs(scene, n, seed=seed, dtype=np.float32)
        b = (a + rng.uniform(-0.2, 0.2, a.shape)).astype(np.float32)
        sets.append((a, b))
    d1 = torch.empty((n, scene.q_dim), dtype=torch.float32, device="cuda")
    d2 = torch.empty_like(d1)
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    d1.copy_(torch.from_numpy(sets[0][0]))
    d2.copy_(torch.from_numpy(sets[0][1]))
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        assert _call(lib, lib.mrmg_is_edge_collision_free_batch_noalloc, sc, d1, d2, 0.02, out) == 0
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = lib.mrmg_is_edge_collision_free_batch_noalloc(
            sc.h, d1.data_ptr(), d2.data_ptr(), L.MRMG_F32, n, 0.02, 0, None, 0, -1, out.data_ptr(), s.cuda_stream,
            L.MRMG_FLAG_ASYNC)
    assert rc == 0, lib.mrmg_last_error()
    for a, b in sets:
        d1.copy_(torch.from_numpy(a))
        d2.copy_(torch.from_numpy(b))
        out.fill_(7)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        ref = torch.empty_like(out)
        assert _call(lib, lib.mrmg_is_edge_collision_free_batch, sc, d1, d2, 0.02, ref) == 0
        assert np.array_equal(got, ref.cpu().numpy())
        assert 0 < int(got.sum()) < n


def test_noalloc_reports_device_errors(gpu):
    """N_start > N: the synchronous call returns MRMG_ERR_N_START, and a
    recorded asynchronous call leaves the same bits in the scene's error
    word after each replay, cleared again by a valid call."""
    lib = pkg("_lib").load()
    L = pkg("_lib")
    scenes, col = pkg("scenes"), pkg("collision")
    sc = col.Gb300Scene(scenes.make_disc_scene(0))
    w = scenes.make_disc_workload(0, n_configs=10, n_edges=64)
    d1 = torch.from_numpy(np.ascontiguousarray(w["q1"])).cuda()
    d2 = torch.from_numpy(np.ascontiguousarray(w["q2"])).cuda()
    n = d1.shape[0]
    Nt = torch.full((n,), 3, dtype=torch.int64, device="cuda")
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()

    def call(N_start, flags, stream):
        return lib.mrmg_is_edge_collision_free_batch_noalloc(
            sc.h, d1.data_ptr(), d2.data_ptr(), L.MRMG_F64, n, 0.01, 0, Nt.data_ptr(), N_start, -1, out.data_ptr(),
            stream.cuda_stream, flags)

    with torch.cuda.stream(s):
        assert call(5, 0, s) == L.MRMG_ERR_N_START
        assert call(0, 0, s) == 0
    s.synchronize()
    ew = C.c_void_p()
    assert lib.mrmg_scene_error_word(sc.h, C.byref(ew)) == 0
    word = torch.as_tensor(col._DeviceWord(ew.value), device="cuda")
    assert int(word.item()) == 0
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        assert call(5, L.MRMG_FLAG_ASYNC, s) == 0
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        bits = int(word.item())
        assert lib.mrmg_status_from_error_bits(bits) == L.MRMG_ERR_N_START
        with torch.cuda.stream(s):
            assert call(0, 0, s) == 0
        s.synchronize()
        assert int(word.item()) == 0
