"""Host-side logic that needs no GPU: the edge step-count formula of the
serving batcher, the workload generators, the penetration parameter record,
the C library's export of the new entry points, and the FP32 error bounds
the kernels rely on (radius pre-test band, step-count certificate,
double-float edge positions), restated with numpy FP32 arithmetic."""
import math

import numpy as np
import pytest

from conftest import golden, pkg


def test_edge_steps_matches_reference_formula():
    """N = max(2, int(max|q2 - q1| / res) + 1) in float64
    (abstract_env.py:321-329), row by row."""
    import importlib

    scenes = pkg("scenes")
    # serving.py imports torch at module level; the formula itself is numpy
    srv = importlib.import_module("multirobot-pathplanning-benchmark_gb300.serving")
    sc = scenes.make_arm_scene(0)
    rng = np.random.default_rng(0)
    q1 = rng.uniform(-3, 3, (500, 28)).astype(np.float32)
    q2 = (q1 + rng.normal(0, 0.4, q1.shape)).astype(np.float32)
    q2[:5] = q1[:5]                      # zero-length edges: N = 2
    for res in (0.05, 0.01, 0.3):
        want = [max(2, int(max(abs(float(b) - float(a)) for a, b in zip(x, y)) / res) + 1) for x, y in zip(q1, q2)]
        assert np.array_equal(srv.edge_steps(q1, q2, res), np.array(want))
    N = scenes.lognormal_steps(2000, 3)
    a, b = scenes.edges_with_steps(sc, N, 0.05, 4)
    assert np.array_equal(srv.edge_steps(a, b, 0.05), N)


def test_serving_requests_shapes():
    scenes = pkg("scenes")
    sc = scenes.make_mobile_scene(0)
    reqs = scenes.make_serving_requests(sc, seed=1, n_instances=5, configs=(3, 9), edges=(0, 4), steps=(5, 800))
    assert len(reqs) == 5
    for r in reqs:
        assert r["configs"].shape[1] == 72 and 3 <= len(r["configs"]) <= 9
        assert r["q1"].shape == r["q2"].shape and len(r["N"]) == len(r["q1"]) <= 4
        assert r["configs"].dtype == np.float32 and r["N"].dtype == np.int64
        if len(r["N"]):
            assert r["N"].min() >= 5 and r["N"].max() <= 800
        lo, hi = sc.limits
        assert np.all(r["configs"] >= lo.astype(np.float32) - 1e-6) and np.all(r["configs"] <= hi.astype(np.float32) + 1e-6)


def test_penetration_params_record():
    pen = pkg("penetration")
    p = pen.PenetrationParams()
    assert list(p.array()) == [0.02, 0.02, 1.0, 0.1]
    q = pen.PenetrationParams(margin=0.05, beta=40.0)
    assert q.array()[0] == 0.05 and q.array()[2] == 40.0
    with pytest.raises(Exception):
        p.margin = 1.0                   # frozen


def test_new_entry_points_exported(cuda_lib):
    for name in ("mrmg_path_penetration", "mrmg_penetration_info", "mrmg_microbench_fma"):
        assert hasattr(cuda_lib, name)


def test_radius_fp32_band():
    """The FP32 pre-test of radius queries assumes the FP32 sum of squared
    coordinate differences lies within 2.4e-6 (|q| + |x|)^2 of the exact
    squared distance (the kernel decides outside 7.7e-6 of that).  Checked
    with numpy FP32 arithmetic (separate multiply and add: more rounding than
    the kernel's fused chain) on 28-D inputs from 1e-3 to 1e4 in scale,
    including near-duplicate pairs and mixed signs."""
    rng = np.random.default_rng(0)
    worst = 0.0
    for scale in (1e-3, 1.0, 3.14, 1e2, 1e4):
        q = rng.uniform(-scale, scale, (4000, 28))
        x = np.where(rng.random((4000, 1)) < 0.3, q + rng.normal(0, 1e-5 * scale, q.shape),
                     rng.uniform(-scale, scale, q.shape))
        qf, xf = q.astype(np.float32), x.astype(np.float32)
        m = np.zeros(len(q), dtype=np.float32)
        for k in range(28):
            d = qf[:, k] - xf[:, k]
            m = (m + d * d).astype(np.float32)
        exact = np.array([float(sum((a - b) ** 2 for a, b in zip(map(np.longdouble, qi), map(np.longdouble, xi))))
                          for qi, xi in zip(q[:400], x[:400])])
        e = np.linalg.norm(q[:400], axis=1) + np.linalg.norm(x[:400], axis=1)
        ratio = np.abs(m[:400].astype(np.float64) - exact) / (e * e)
        worst = max(worst, float(ratio.max()))
    assert worst <= 2.4e-6, worst


def test_fp32_step_count_certificate():
    """The edge kernels take N = int(m / res) + 1 from the FP32 quotient
    fl32(m) / fl32(res) when its fractional part is farther than
    4.8e-7 * max(t, 1) from an integer (`steps_fp32`); the integer part is
    then the FP64 quotient's.  Checked with numpy FP32 division on random
    lengths and on lengths a few ulps around every multiple of res."""
    rng = np.random.default_rng(5)
    f32 = np.float32
    for res in (0.01, 0.05, 0.003, 0.1, 1.0 / 3.0, 0.0125):
        k = rng.integers(1, 4_000_000, 20_000).astype(np.float64)
        near = k * res
        m = np.concatenate([
            np.exp(rng.uniform(np.log(1e-6), np.log(2e4 * res), 40_000)),
            near, np.nextafter(near, 0.0), np.nextafter(near, np.inf),
            near * (1 + 3e-16), near * (1 - 3e-16), near * (1 + 2e-7), near * (1 - 2e-7)])
        t64 = m / res
        t32 = (m.astype(f32) / f32(res)).astype(f32)
        fl = np.floor(t32).astype(f32)
        fr = (t32 - fl).astype(f32)
        tol = (f32(4.8e-7) * np.maximum(t32, f32(1.0))).astype(f32)
        cert = (t32 < f32(4194304.0)) & (m.astype(f32) >= f32(2.0 ** -60)) & (fr > tol) & (fr < f32(1.0) - tol)
        assert cert[:40_000].mean() > 0.99         # random lengths: the certificate decides
        assert cert[40_000:60_000].sum() == 0      # exact multiples of res: it declines
        assert np.array_equal(np.floor(t32[cert]).astype(np.int64), np.floor(t64[cert]).astype(np.int64)), res


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fp32_step_count_certificate_near_integers(dtype):
    """The certificate on whole edges: FP64 or FP32 endpoints in 6-D, edge
    lengths of 1 to 5,000 steps, half of them within 1e-12 .. 1e-4 steps of
    an integer multiple of the resolution; the device rounds each FP64
    coordinate difference to FP32 and takes the largest.  Every certified
    N is the reference's max(2, int(max|q1 - q2| / res) + 1)."""
    f32 = np.float32
    for res in (0.01, 0.05, 0.001, 0.0123456789, 1e-5):
        rng = np.random.default_rng(int(res * 1e6) + (dtype == np.float32))
        n, D = 150_000, 6
        a = rng.uniform(-3, 3, (n, D)).astype(dtype)
        k = np.floor(10.0 ** rng.uniform(0, 3.7, n))
        near = rng.random(n) < 0.5
        frac = np.where(near, rng.choice([0.0, 1.0, -1.0], n) * 10.0 ** rng.uniform(-12, -4, n), rng.random(n))
        m = (k + frac) * res
        lead = rng.integers(0, D, n)
        b = a.astype(np.float64) + rng.uniform(-1, 1, (n, D)) * m[:, None] * 0.5
        b[np.arange(n), lead] = a[np.arange(n), lead] + m * rng.choice([-1.0, 1.0], n)
        b = b.astype(dtype)
        diff = np.abs(b.astype(np.float64) - a.astype(np.float64))
        N_ref = np.maximum(2, (np.max(diff, axis=1) / res).astype(np.int64) + 1)
        m32 = np.max(diff.astype(f32), axis=1)
        t32 = (m32 / f32(res)).astype(f32)
        fl = np.floor(t32).astype(f32)
        fr = (t32 - fl).astype(f32)
        tol = (f32(4.8e-7) * np.maximum(t32, f32(1.0))).astype(f32)
        cert = (t32 < f32(4194304.0)) & (m32 >= f32(2.0 ** -60)) & (fr > tol) & (fr < f32(1.0) - tol)
        N = np.maximum(2, fl.astype(np.int64) + 1)
        assert np.array_equal(N[cert], N_ref[cert]), res
        assert cert[~near].mean() > 0.99, res


def _interp_df(ah, al, dh, dl, fi, nm1, rn):
    """numpy FP32 restatement of interp_df (fused multiply-adds emulated in
    FP64, then rounded to FP32)."""
    f32 = np.float32

    def fma(a, b, c):
        return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)

    def two_sum(a, b):
        t = (a + b).astype(f32)
        bb = (t - a).astype(f32)
        return t, ((a - (t - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)

    th = (fi * rn).astype(f32)
    tl = (fma(-th, nm1, fi) * rn).astype(f32)
    ph = (dh * th).astype(f32)
    pl = fma(dh, th, -ph)
    pl = fma(dh, tl, fma(dl, th, pl))
    sh, sl = two_sum(ah, ph)
    return sh, (((sl + pl).astype(f32)) + al).astype(f32)


def test_double_float_edge_positions_within_band():
    """Abstract-scene edge positions q1 + (q2 - q1) * i / (N - 1), formed in
    double-float FP32 and rounded once, lie within 2^-24 |Q| + 2^-42 (|q1| +
    |q2|) of the reference's FP64 position Q = q1 + ((q2 - q1) / (N - 1)) * i;
    the kernel's band adds 2^-30 (|q1| + |q2|) per coordinate for the second
    term.  FP64 and FP32-valued endpoints."""
    rng = np.random.default_rng(6)
    f32 = np.float32
    n = 200_000
    q1 = rng.uniform(-4, 4, n)
    q2 = q1 + rng.normal(0, 1.5, n)
    half = rng.random(n) < 0.5
    q1 = np.where(half, q1.astype(f32).astype(np.float64), q1)
    q2 = np.where(half, q2.astype(f32).astype(np.float64), q2)
    res = rng.choice([0.01, 0.05, 0.003], n)
    N = np.maximum(2, (np.abs(q2 - q1) / res).astype(np.int64) + 1)
    i = (rng.random(n) * N).astype(np.int64)
    d = q2 - q1
    ah = q1.astype(f32)
    al = (q1 - ah.astype(np.float64)).astype(f32)
    dh = d.astype(f32)
    dl = (d - dh.astype(np.float64)).astype(f32)
    nm1 = (N - 1).astype(f32)
    rn = (f32(1.0) / nm1).astype(f32)
    h, l = _interp_df(ah, al, dh, dl, i.astype(f32), nm1, rn)
    x = (h + l).astype(f32).astype(np.float64)
    Q = q1 + (d / (N - 1)) * i
    S = np.abs(q1) + np.abs(q2)
    err = np.abs(x - Q)
    assert np.all(err <= 2.0 ** -24 * np.abs(Q) + 2.0 ** -42 * S)
    assert np.all(err <= 2.0 ** -24 * np.abs(Q) + 2.0 ** -30 * S)


@pytest.mark.parametrize("scale,nmax", [(np.pi, 10_000), (50.0, 1 << 20), (1e3, 1 << 24)])
def test_double_float_edge_positions_large_scales(scale, nmax):
    """The same bound for 4-D endpoints up to 10^3 apart from the origin and
    step counts up to 2^24 (the largest the FP32 position path takes), with
    edge lengths from 10^-6 to 1 times the coordinate scale; the bound's
    second term uses the largest |q1_k| + |q2_k| of the edge, as the band."""
    rng = np.random.default_rng(int(scale) + nmax)
    f32 = np.float32
    n, D = 100_000, 4
    q1 = rng.uniform(-scale, scale, (n, D))
    q2 = q1 + rng.uniform(-scale, scale, (n, D)) * 10.0 ** rng.uniform(-6, 0, (n, 1))
    N = rng.integers(2, nmax + 1, n)
    i = np.minimum((rng.random(n) * N).astype(np.int64), N - 1)
    d = q2 - q1
    ah = q1.astype(f32)
    al = (q1 - ah.astype(np.float64)).astype(f32)
    dh = d.astype(f32)
    dl = (d - dh.astype(np.float64)).astype(f32)
    nm1 = (N - 1).astype(f32)[:, None]
    rn = (f32(1.0) / nm1).astype(f32)
    h, l = _interp_df(ah, al, dh, dl, i.astype(f32)[:, None], nm1, rn)
    x = (h + l).astype(f32).astype(np.float64)
    Q = q1 + (d / (N - 1)[:, None]) * i[:, None]
    M = np.max(np.abs(ah.astype(np.float64)) + np.abs(ah.astype(np.float64) + dh.astype(np.float64)), axis=1)
    assert np.all(np.abs(x - Q) <= 2.0 ** -24 * np.abs(x) + 2.0 ** -30 * M[:, None])


def test_query_modes_one_per_query():
    """NodeStore queries hand the library exactly Q int32 modes: a single
    mode applies to every query, any other count is refused (the library
    would read past a short array)."""
    qmodes = pkg("knn")._query_modes
    assert qmodes([2, 0, 1], 3).tolist() == [2, 0, 1] and qmodes([2, 0, 1], 3).dtype == np.int32
    assert qmodes(4, 3).tolist() == [4, 4, 4] and qmodes([4], 2).tolist() == [4, 4]
    assert qmodes(np.array([1, 2], dtype=np.int64), 2).flags["C_CONTIGUOUS"]
    assert qmodes([], 0).shape == (0,) and qmodes(3, 0).shape == (0,)
    import torch

    assert qmodes(torch.tensor([1, 0]), 2).tolist() == [1, 0]
    for bad, Q in (([1, 2], 3), ([1, 2, 3], 2), ([], 1)):
        with pytest.raises(ValueError):
            qmodes(bad, Q)


def test_knn_exact_refuses_bad_modes_on_the_host(cuda_lib):
    """knn_exact's kernel reads the offsets of each query's mode without a
    bound, so modes and offsets are checked before anything reaches the
    device (these raise without a GPU)."""
    knn = pkg("knn")
    nodes, qs, sl = np.zeros((10, 4)), np.zeros((3, 4)), [[0, 2], [2, 4]]
    for qm, off in (([0, 1, 2], [0, 5, 10]), ([0, -1, 1], [0, 5, 10]), ([0, 0], [0, 5, 10]),
                    ([0, 0, 0], [0, 5, 9]), ([0, 0, 0], [1, 5, 10]), ([0, 0, 0], [0, 6, 5, 10]), ([0, 0, 0], [0])):
        with pytest.raises(ValueError):
            knn.knn_exact(qs, qm, nodes, off, sl, "euclidean", 1)
    with pytest.raises(ValueError):
        knn.knn_exact(np.zeros((3, 5)), [0, 0, 0], nodes, [0, 10], sl, "euclidean", 1)


def test_path_check_covers_the_reference_calls():
    """tests/test.py:93-122 of the reference counts the is_collision_free calls
    of is_path_collision_free on a three-state path: 5 at resolution 0.5 and
    21 at 0.1, with and without check_edges_in_order.  The batched path check
    submits the same configurations at once: the checked vertices and the
    interior of every edge.  A stand-in for the device scene counts them."""
    import torch

    envm = pkg("env")
    ka = golden("known_answers.json")

    class CountingScene:
        mode = -1

        def __init__(self):
            self.configs = 0

        def is_collision_free_host(self, qs):
            self.configs += len(qs)
            return np.ones(len(qs), dtype=np.uint8)

        def is_edge_collision_free_host(self, q1s, q2s, resolution, include_endpoints=False, N=None):
            assert not include_endpoints and N is None
            self.configs += sum(envm._edge_N(a, b, resolution) - 2 for a, b in zip(q1s, q2s))
            return np.ones(len(q1s), dtype=np.uint8)

    env = object.__new__(envm.Gb300AbstractEnvironment)

    class S:
        def __init__(self, q):
            self.q, self.mode = np.array(q, dtype=np.float64), None

    path = [S([-1, 0, 1, 1]), S([-1, 1, 1, 0]), S([-1, 2, 1, -1])]
    counts = []
    for res, in_order in ((0.5, True), (0.5, False), (0.1, True), (0.1, False)):
        env._gb300 = CountingScene()
        assert env.is_path_collision_free(path, resolution=res, check_edges_in_order=in_order)
        counts.append(env._gb300.configs)
    assert counts == ka["path_calls"]


def test_env_mode_hooks():
    """The reference's mode logic stores get_scenegraph_info_for_mode(mode)
    with every new mode (planning_env.py:466) and planners call
    set_to_mode: both exist on the backend.  A scene without modes keeps its
    tables; a per-mode scene switches to the mode's table set."""
    envm = pkg("env")

    class Switches:
        def __init__(self):
            self.mode, self.calls = -1, []

        def set_mode(self, m):
            self.mode = m
            self.calls.append(m)

    plain = object.__new__(envm.Gb300AbstractEnvironment)
    plain._gb300 = Switches()
    assert plain.get_scenegraph_info_for_mode(object()) == {} and plain.get_scenegraph_info_for_mode(None, True) == {}
    plain.set_to_mode(3)
    assert plain._gb300.calls == []

    class Mode:
        def __init__(self, i):
            self.id = i

    per_mode = object.__new__(envm.Gb300ArmEnvironment)
    per_mode._gb300 = Switches()
    per_mode._mode_index = lambda m: m if isinstance(m, (int, np.integer)) else m.id
    per_mode.set_to_mode(Mode(2))
    per_mode.set_to_mode(Mode(2))          # already selected: no switch
    per_mode.set_to_mode(0)
    per_mode.set_to_mode(None)             # None leaves the tables as they are
    assert per_mode._gb300.calls == [2, 0] and per_mode._gb300.mode == 0


def test_verdict_buffer_is_checked():
    """A caller's verdict buffer must be a contiguous uint8 CUDA tensor with
    room for every verdict (the kernels write n bytes); anything else is
    refused before a launch."""
    import torch

    out_tensor = pkg("collision")._out_tensor
    for bad in (np.zeros(4, dtype=np.uint8), torch.zeros(4, dtype=torch.uint8),
                torch.zeros(4, dtype=torch.int32), torch.zeros((4, 2), dtype=torch.uint8)[:, 0]):
        with pytest.raises(ValueError):
            out_tensor(bad, 4, None)


def test_scene_arrays_refuse_inconsistent_shapes():
    """The library reads exactly the robot, sphere and box counts it is given:
    scene arrays whose shapes disagree with those counts are refused on the
    host with ValueError, before any library call."""
    import copy

    scenes = pkg("scenes")
    arm = scenes.make_arm_scene(0)
    a = arm.arrays()
    assert a["base_pose"].shape == (4, 12) and a["dh"].shape == (4, scenes.MAX_LINKS, 4)
    assert a["sphere_local"].shape == (168, 3) and a["box_lo"].shape == (50, 3)
    for field, value in (("base_pose", arm.base_pose[:, :9]), ("dh", arm.dh[:, :7]),
                         ("sphere_local", arm.sphere_local[:-1]), ("sphere_robot", arm.sphere_robot[:-1]),
                         ("sphere_link", arm.sphere_link[:, None].repeat(2, 1)), ("base_kind", arm.base_kind[:3]),
                         ("box_hi", arm.box_hi[:-1]), ("box_lo", arm.box_lo[:, :2])):
        bad = copy.deepcopy(arm)
        setattr(bad, field, value)
        with pytest.raises(ValueError):
            bad.arrays()
    modes = scenes.make_arm_mode_scene(1, n_objects=4, n_modes=3)
    modes.mode_tables()
    bad = copy.deepcopy(modes)
    bad.mode_attach = bad.mode_attach[:2]
    with pytest.raises(ValueError):
        bad.mode_tables()
    bad = copy.deepcopy(modes)
    bad.sphere_attach = np.asarray(bad.sphere_attach)[:-1]
    with pytest.raises(ValueError):
        bad.mode_tables()
    no_attach = copy.deepcopy(modes)
    no_attach.sphere_attach, no_attach.mode_attach = None, None
    t = no_attach.mode_tables()
    assert t["attach_off"].tolist() == [0, 0, 0, 0] and (t["sphere_attach"] == -1).all()

    disc = scenes.make_disc_scene(0)
    assert disc.tables()["box_lo"].shape == (10, 2)
    for field, value in (("box_bounds", disc.box_bounds[:-1]), ("box_center", disc.box_center[:, :1]),
                         ("agent_slices", disc.agent_slices[:1]), ("sphere_pos", np.zeros((1, 2)))):
        bad = copy.deepcopy(disc)
        setattr(bad, field, value)
        with pytest.raises(ValueError):
            bad.tables()


def test_mode_tables_and_views():
    """Per-mode scene declarations: the flat arrays the library receives and
    the reduced scene a mode sees (its boxes, robot spheres plus the attached
    objects it lists)."""
    scenes = pkg("scenes")
    sc = scenes.make_arm_mode_scene(0, n_objects=5, n_modes=6)
    t = sc.mode_tables()
    assert t["box_off"][0] == 0 and t["box_off"][-1] == len(t["boxes"]) and len(t["box_off"]) == 7
    assert t["attach_off"][-1] == len(t["attach"]) and t["sphere_attach"].shape == (len(sc.sphere_radius),)
    for m in range(sc.n_modes):
        v = sc.for_mode(m)
        assert len(v.box_lo) == len(sc.mode_boxes[m])
        n_robot = int((sc.sphere_attach < 0).sum())
        assert len(v.sphere_radius) == n_robot + 3 * len(sc.mode_attach[m])
        held = {j % sc.n_robots for j in sc.mode_attach[m]}
        assert len(held) == len(sc.mode_attach[m])          # one object per gripper
        lo = np.asarray(sc.box_lo)[np.asarray(sc.mode_boxes[m], dtype=np.int64)]
        assert np.array_equal(v.box_lo, lo)


def test_speculative_checker_batches_by_mode():
    """The checker sends a missed edge with the upcoming ones, at most
    `window` edges, one call per mode, and answers later lookups from its
    cache without further calls."""
    lazy = pkg("lazy")
    calls = []

    def check(q0, q1, mode):
        calls.append((mode, len(q0)))
        return q0[:, 0] < 0.5

    class N:
        def __init__(self, i, mode):
            self.id = i
            self.state = type("S", (), {"q": np.array([i / 20.0, 0.0]), "mode": mode})()

    nodes = [N(i, i % 2) for i in range(20)]
    ck = lazy.SpeculativeEdgeChecker(check=check, window=6)
    up = [(nodes[i], nodes[i + 1]) for i in range(1, 19)]
    assert ck.is_free(nodes[0], nodes[1], up) is True
    assert sum(n for _, n in calls) == 6 and {m for m, _ in calls} == {0, 1}
    assert len(calls) == 2
    before = len(calls)
    assert ck.is_free(nodes[3], nodes[4]) is True          # speculated: from the cache
    assert len(calls) == before
    assert ck.is_free(nodes[11], nodes[12]) is False      # a miss: one more batch
    assert len(calls) == before + 1
    assert ck.stats()["lookups"] == 3


def test_importer_options():
    imp = pkg("importers")
    base = """<mujoco>{comp}<worldbody>
      <body name="r" pos="0 0 0.1">
        <joint type="slide" axis="1 0 0" range="-1 1"/>
        <joint type="slide" axis="0 1 0" range="-1 1"/>
        <joint type="hinge" axis="0 0 1" range="-1.5 1.5"/>
        {geom}
      </body>
      <body name="s" pos="0 0 0.1">
        <joint type="slide" axis="1 0 0" range="-1 1"/>
        <joint type="slide" axis="0 1 0" range="-1 1"/>
        <joint type="hinge" axis="0 0 1" range="-90 90"/>
        <geom type="sphere" size="0.1"/>
      </body>
      <geom type="box" pos="0.5 0 0.1" size="0.1 0.1 0.1"/>
    </worldbody></mujoco>"""
    sc = imp.load_mjcf_planar(base.format(comp='<compiler angle="radian"/>', geom='<geom type="capsule" size="0.07 0.1"/>'))
    np.testing.assert_allclose(sc.limits[:, 2], [-1.5, 1.5])           # radians as given
    np.testing.assert_allclose(sc.limits[:, 5], [-90.0, 90.0])         # radian compiler: no conversion
    assert sc.sphere_radius.tolist() == [0.07, 0.1] and len(sc.box_lo) == 1
    sc = imp.load_mjcf_planar(base.format(comp="", geom='<geom type="sphere" size="0.2"/>'), robots=["s", "r"])
    assert sc.sphere_radius.tolist() == [0.1, 0.2]                     # configuration order as asked
    np.testing.assert_allclose(sc.limits[:, 2], np.deg2rad([-90.0, 90.0]))
    with pytest.raises(NotImplementedError):
        imp.load_mjcf_planar(base.format(comp="", geom='<geom type="capsule" fromto="0 0 0 0.2 0 0" size="0.05"/>'))
    with pytest.raises(ValueError):
        imp.load_mjcf_planar(base.format(comp="", geom="<geom type='sphere' size='0.1'/>").replace(' range="-1 1"', "", 1))
    with pytest.raises(ValueError):
        imp.load_mjcf_planar(base.format(comp="", geom="<geom type='sphere' size='0.1'/>"), robots=["nobody"])


def _bfs_at32(N: int, p: int) -> int:
    """Python restatement of the kernels' 32-bit closed-form BFS position map
    (bfs_at32 in csrc/mrmg_common.cuh)."""
    L = (N + 1).bit_length() - 1
    full = (1 << L) - 1
    if p < full:
        lv = (p + 1).bit_length() - 1
        slot = p + 1 - (1 << lv)
        s, e = 0, N - 1
        for b in range(lv - 1, -1, -1):
            mid = (s + e) >> 1
            if (slot >> b) & 1:
                s = mid + 1
            else:
                e = mid - 1
        return (s + e) >> 1
    r, a, b = p - full, 0, N - 1
    for d in range(L):
        m = (a + b) >> 1
        cnt = (m - a) - ((1 << (L - d - 1)) - 1)
        if r < cnt:
            b = m - 1
        else:
            r -= cnt
            a = m + 1
    return a


def test_bfs_at32_matches_reference_order():
    """The closed-form position map equals generate_binary_search_indices
    (planning_env.py:34-51) position by position (golden vectors of the
    reference, N = 1..300 and larger)."""
    g = golden("binary_indices.npz")
    off = 0
    for N in g["Ns"]:
        N = int(N)
        ref = g["flat"][off:off + N]
        off += N
        assert [_bfs_at32(N, p) for p in range(N)] == ref.tolist(), N
