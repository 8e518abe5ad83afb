"""GPU parity: the CUDA collision path against the golden vectors of the
reference and against the oracle.  Verdicts and indices must be bit-exact."""
import json

import numpy as np
import pytest
import torch

from conftest import golden, pkg

pytestmark = pytest.mark.gpu


def _disc_scene(g):
    return pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["centers"],
        box_bounds=2.0 * g["half"], sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)


def test_binary_order_on_device(gpu):
    col = pkg("collision")
    g = golden("binary_indices.npz")
    off = 0
    for N in g["Ns"]:
        ref = tuple(int(x) for x in g["flat"][off:off + N])
        off += N
        assert col.binary_search_indices(int(N)) == ref, N
        assert col.binary_search_indices(int(N), chunked=True) == ref, N


def test_disc_configs_golden(gpu):
    g = golden("abstract_disc.npz")
    sc = pkg("collision").Gb300Scene(_disc_scene(g))
    for dt in (np.float64,):
        v = sc.is_collision_free_batch(g["configs"].astype(dt)).cpu().numpy()
        assert np.array_equal(v, g["config_free"])


def test_disc_edges_golden_all_variants(gpu):
    g = golden("abstract_disc.npz")
    sc = pkg("collision").Gb300Scene(_disc_scene(g))
    variants = json.loads(str(g["variants"]))
    for vi, v in enumerate(variants):
        ref = g["edge_free"][vi]
        ok = ref != 255
        out = sc.is_edge_collision_free_batch(g["q1"][ok], g["q2"][ok], v["resolution"],
                                              v.get("include_endpoints", False), None, v.get("N_start", 0),
                                              v.get("N_max")).cpu().numpy()
        assert np.array_equal(out, ref[ok]), vi
        if (~ok).any():
            with pytest.raises(AssertionError):
                sc.is_edge_collision_free_batch(g["q1"][~ok], g["q2"][~ok], v["resolution"],
                                                v.get("include_endpoints", False), None, v.get("N_start", 0),
                                                v.get("N_max"))


def test_disc_edges_graph_plan_golden(gpu):
    """The graph-captured plan over the abstract scene (FP64 endpoints, as the
    reference's configurations) gives the golden verdicts of the reference's
    own edge check, replay after replay and for new endpoints."""
    g = golden("abstract_disc.npz")
    col = pkg("collision")
    sc = col.Gb300Scene(_disc_scene(g))
    v = json.loads(str(g["variants"]))[0]
    assert v.get("N_start", 0) == 0 and v.get("N_max") is None and not v.get("include_endpoints", False)
    ref = g["edge_free"][0]
    assert (ref != 255).all()
    half = len(ref) // 2
    plan = col.EdgeCheckPlan(sc, half, v["resolution"], dtype=torch.float64, chunks=2)
    for lo in (0, half, 0):
        plan.q1_host[:] = g["q1"][lo:lo + half]
        plan.q2_host[:] = g["q2"][lo:lo + half]
        assert np.array_equal(plan.run(), ref[lo:lo + half]), lo


def test_disc_env_api_golden(gpu):
    g = golden("abstract_disc.npz")
    env = pkg("env").Gb300AbstractEnvironment(_disc_scene(g))
    for i in range(0, 400, 37):
        q = env.start_pos.from_flat(g["configs"][i])
        assert env.is_collision_free(q, None) == bool(g["config_free"][i])
    for e in range(0, 800, 53):
        a, b = env.start_pos.from_flat(g["q1"][e]), env.start_pos.from_flat(g["q2"][e])
        assert env.is_edge_collision_free(a, b, None) == bool(g["edge_free"][0, e])
    with pytest.raises(ValueError):
        env.is_collision_free(None, None)


def test_abstract_test_scene_golden(gpu):
    g = golden("abstract_test.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["box_center"],
        box_bounds=g["box_bounds"], sphere_pos=g["sphere_pos"], sphere_radius=[float(g["sphere_radius"][0])], q_dim=4)
    sc = pkg("collision").Gb300Scene(scene)
    assert np.array_equal(sc.is_collision_free_batch(g["configs"]).cpu().numpy(), g["config_free"])
    assert np.array_equal(sc.is_edge_collision_free_batch(g["q1"], g["q2"], float(g["resolution"])).cpu().numpy(),
                          g["edge_free"])


def test_known_answers_path(gpu):
    """tests/test.py:50-58 and :93-105 of the reference: free edge and path."""
    ka = golden("known_answers.json")
    g = golden("abstract_test.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["box_center"],
        box_bounds=g["box_bounds"], sphere_pos=g["sphere_pos"], sphere_radius=[float(g["sphere_radius"][0])], q_dim=4)
    env = pkg("env").Gb300AbstractEnvironment(scene, limits=np.array([[-2.0] * 4, [2.0] * 4]))
    q1 = env.start_pos.from_flat(np.array([-1.0, 0, 1, 1]))
    q2 = env.start_pos.from_flat(np.array([-1.0, 1, 1, 0]))
    q3 = env.start_pos.from_flat(np.array([-1.0, 2, 1, -1]))
    assert env.is_edge_collision_free(q1, q2, None) == ka["edge_free"]

    class S:
        def __init__(self, q):
            self.q, self.mode = q, None

    assert env.is_path_collision_free([S(q1), S(q2), S(q3)], resolution=0.5) == ka["path_free"]


def test_abstract_10d_golden(gpu):
    g = golden("abstract_10d.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 10], [10, 20]]), agent_radii=[0.1, 0.1], box_center=g["box_center"][None],
        box_bounds=g["box_bounds"][None], sphere_pos=np.zeros((0, 10)), sphere_radius=[], q_dim=20)
    sc = pkg("collision").Gb300Scene(scene)
    assert np.array_equal(sc.is_collision_free_batch(g["configs"]).cpu().numpy(), g["config_free"])
    assert np.array_equal(sc.is_edge_collision_free_batch(g["q1"], g["q2"], 0.05).cpu().numpy(), g["edge_free"])


def test_primitives_3d_golden(gpu):
    g = golden("primitives3d.npz")
    scenes, col = pkg("scenes"), pkg("collision")
    for i in list(range(0, 200)) + list(range(4000, 4100)):
        s = scenes.AbstractScene(np.array([[0, 3]]), [float(g["sphere_r"][i])], g["box_center"][i][None],
                                 2.0 * g["box_half"][i][None], np.zeros((0, 3)), [], 3)
        v = col.Gb300Scene(s).is_collision_free_batch(g["sphere_c"][i][None]).item()
        assert v == (0 if g["rect_hit"][i] else 1), i
        s2 = scenes.AbstractScene(np.array([[0, 3]]), [float(g["rb"][i])], np.zeros((0, 3)), np.zeros((0, 3)),
                                  g["pa"][i][None], [float(g["ra"][i])], 3)
        v2 = col.Gb300Scene(s2).is_collision_free_batch(g["pb"][i][None]).item()
        assert v2 == (0 if g["sphere_hit"][i] else 1), i


def test_disc_workload_vs_oracle(gpu, oracle):
    scenes = pkg("scenes")
    scene = scenes.make_disc_scene(0)
    w = scenes.make_disc_workload(0)
    sc = pkg("collision").Gb300Scene(scene)
    o = oracle.OracleScene(scene)
    assert np.array_equal(sc.is_collision_free_batch(w["configs"]).cpu().numpy(), o.configs_free(w["configs"]))
    assert np.array_equal(sc.is_edge_collision_free_batch(w["q1"], w["q2"], 0.01).cpu().numpy(),
                          o.edges_free(w["q1"], w["q2"], 0.01))


BOUNDARY_EPS = [-1e-6, -1e-9, -1e-12, -1e-15, 0.0, 1e-15, 1e-12, 1e-9, 1e-8, 1e-7, 1e-6, 1e-5]


def _face_edges(scene, r):
    """Edges that slide along each face of each box at distance r + eps from
    it (their positions over the face are that far from the box), for every
    eps of BOUNDARY_EPS: inside the FP32 band, so the exact pass decides."""
    lo = scene.box_center - scene.box_bounds / 2
    hi = scene.box_center + scene.box_bounds / 2
    q1, q2 = [], []
    for b in range(len(lo)):
        for e in BOUNDARY_EPS:
            y = hi[b, 1] + r + e
            q1.append([lo[b, 0] - 0.3, y]); q2.append([hi[b, 0] + 0.3, y])
            y = lo[b, 1] - r - e
            q1.append([hi[b, 0] + 0.3, y]); q2.append([lo[b, 0] - 0.3, y])
            x = hi[b, 0] + r + e
            q1.append([x, lo[b, 1] - 0.3]); q2.append([x, hi[b, 1] + 0.3])
            x = lo[b, 0] - r - e
            q1.append([x, hi[b, 1] + 0.3]); q2.append([x, lo[b, 1] - 0.3])
    return np.array(q1), np.array(q2)


def test_near_boundary_cases_vs_oracle(gpu, oracle):
    """Configurations and edges placed at distance r + eps from box faces
    and agent pairs at distance r_i + r_j + eps, eps from -1e-6 to 1e-5
    (exact contact included): the verdicts of the FP32 band and the FP64
    re-check equal the oracle's, for FP64 inputs as the reference's."""
    scenes, col = pkg("scenes"), pkg("collision")
    base = scenes.make_disc_scene(0)
    one = scenes.AbstractScene(agent_slices=np.array([[0, 2]]), agent_radii=[0.1], box_center=base.box_center,
                               box_bounds=base.box_bounds, sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=2)
    q1, q2 = _face_edges(one, 0.1)
    o, sc = oracle.OracleScene(one), col.Gb300Scene(one)
    for incl in (False, True):
        want = o.edges_free(q1, q2, 0.01, include_endpoints=incl)
        assert 0.05 < want.mean() < 0.95
        assert np.array_equal(sc.is_edge_collision_free_batch(q1, q2, 0.01, incl).cpu().numpy(), want), incl
    cfg = np.concatenate([0.5 * (q1 + q2), q1])
    want = o.configs_free(cfg)
    assert 0.05 < want.mean() < 0.95
    assert np.array_equal(sc.is_collision_free_batch(cfg).cpu().numpy(), want)

    pair = scenes.AbstractScene(agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1],
                                box_center=np.zeros((0, 2)), box_bounds=np.zeros((0, 2)),
                                sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)
    rng = np.random.default_rng(3)
    c, p1, p2 = [], [], []
    for e in BOUNDARY_EPS:
        for ang in rng.uniform(0, 2 * np.pi, 8):
            u = np.array([np.cos(ang), np.sin(ang)])
            nrm = np.array([-u[1], u[0]])
            a0 = rng.uniform(-0.5, 0.5, 2)
            a1 = a0 + nrm * (0.2 + e)
            c.append(np.concatenate([a0, a1]))
            p1.append(np.concatenate([a0, a1 - 0.4 * u]))
            p2.append(np.concatenate([a0, a1 + 0.4 * u]))
    c, p1, p2 = np.array(c), np.array(p1), np.array(p2)
    op, sp = oracle.OracleScene(pair), col.Gb300Scene(pair)
    want = op.configs_free(c)
    assert 0.05 < want.mean() < 0.95
    assert np.array_equal(sp.is_collision_free_batch(c).cpu().numpy(), want)
    want = op.edges_free(p1, p2, 0.01, include_endpoints=True)
    assert np.array_equal(sp.is_edge_collision_free_batch(p1, p2, 0.01, True).cpu().numpy(), want)


def test_edge_errors(gpu):
    g = golden("abstract_disc.npz")
    sc = pkg("collision").Gb300Scene(_disc_scene(g))
    q1 = np.array([[0.0, 0.0, 0.5, 0.5]])
    q2 = np.array([[np.nan, 0.0, 0.5, 0.5]])
    with pytest.raises(ValueError):          # int(nan) in the reference
        sc.is_edge_collision_free_batch(q1, q2, 0.01)
    with pytest.raises(AssertionError):      # N_start > N
        sc.is_edge_collision_free_batch(q1, q1 + 0.001, 0.01, N_start=5)
    # empty batch
    assert sc.is_edge_collision_free_batch(np.zeros((0, 4)), np.zeros((0, 4)), 0.01).numel() == 0


def test_path_check_golden(gpu):
    """is_path_collision_free through the env on the device: the reference's
    own verdicts on 400 disc-scene paths under four flag variants
    (tests/golden/paths.npz)."""
    g = golden("paths.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=g["centers"],
        box_bounds=2.0 * g["half"], sphere_pos=np.zeros((0, 2)), sphere_radius=[], q_dim=4)
    env = pkg("env").Gb300AbstractEnvironment(scene)
    off = g["offsets"]

    class S:
        def __init__(self, q):
            self.q, self.mode = env.start_pos.from_flat(q), None

    for vi, v in enumerate(json.loads(str(g["variants"]))):
        got = [int(env.is_path_collision_free([S(q) for q in g["states"][off[i]:off[i + 1]]], **v))
               for i in range(len(off) - 1)]
        assert got == g["free"][vi].tolist(), v


def test_sphere_obstacle_ties_golden(gpu):
    """Configurations within 2e-16 of a Sphere obstacle's contact distance on
    the reference's 'abstract.test' scene: the device's verdicts are the
    reference's own is_collision_free verdicts (batch_forms.npz)."""
    g, a = golden("batch_forms.npz"), golden("abstract_test.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=a["box_center"],
        box_bounds=a["box_bounds"], sphere_pos=a["sphere_pos"], sphere_radius=[float(a["sphere_radius"][0])], q_dim=4)
    sc = pkg("collision").Gb300Scene(scene)
    assert np.array_equal(sc.is_collision_free_batch(g["configs"]).cpu().numpy(), g["single"])


def test_batched_form_ties_golden(gpu):
    """The same near-contact configurations through the batched form: the
    device's MRMG_FLAG_BATCH_FORM verdicts are the reference's own
    _batch_is_collision_free answers, per configuration and for 200 groups
    of 8 (batch_forms.npz), through the C ABI flag and through the env
    method; on these ties they differ from the single form."""
    g, a = golden("batch_forms.npz"), golden("abstract_test.npz")
    scene = pkg("scenes").AbstractScene(
        agent_slices=np.array([[0, 2], [2, 4]]), agent_radii=[0.1, 0.1], box_center=a["box_center"],
        box_bounds=a["box_bounds"], sphere_pos=a["sphere_pos"], sphere_radius=[float(a["sphere_radius"][0])], q_dim=4)
    lib = pkg("_lib")
    env = pkg("env").Gb300AbstractEnvironment(scene)
    v = env._gb300.is_collision_free_batch(g["configs"], flags=lib.MRMG_FLAG_BATCH_FORM).cpu().numpy()
    assert np.array_equal(v, g["batch1"])
    assert not np.array_equal(v, g["single"])
    got8 = np.array([v[grp].all() for grp in g["groups"]], dtype=np.uint8)
    assert np.array_equal(got8, g["batch8"])
    S = pkg("configuration").Gb300Configuration
    sl = [(0, 2), (2, 4)]
    for i in range(0, len(g["configs"]), 97):
        assert env._batch_is_collision_free([S(g["configs"][i], sl)], None) == bool(g["batch1"][i])
    for j, grp in enumerate(g["groups"][:40]):
        assert env._batch_is_collision_free([S(g["configs"][k], sl) for k in grp], None) == bool(g["batch8"][j])


def test_table_staging_never_timed_out(gpu):
    """The kernels stage their scene tables with one bulk asynchronous copy
    on an mbarrier with a bounded wait; none of this process's launches (the
    arm and abstract checks run above and here) fell back to loads."""
    import ctypes

    col, scenes, lib = pkg("collision"), pkg("scenes"), pkg("_lib")
    rng = np.random.default_rng(1)
    for sc in (scenes.make_arm_scene(0), scenes.make_disc_scene(0)):
        s = col.Gb300Scene(sc)
        q = rng.uniform(-1.0, 1.0, (4096, sc.q_dim)).astype(np.float32)
        s.is_collision_free_batch(q)
        s.is_edge_collision_free_batch(q[:2048], q[2048:], 0.05)
        s.is_collision_free_host(q[:8])
    v = ctypes.c_uint32(7)
    lib.check(lib.load().mrmg_table_stage_timeouts(ctypes.byref(v)))
    assert v.value == 0


def test_stream_handle_is_the_current_stream(gpu):
    """The library's current-stream lookup (torch's raw accessor) names the
    same cudaStream_t as torch.cuda.current_stream(), on the default stream
    and inside a stream context; an explicit stream passes through."""
    import torch

    lib = pkg("_lib")
    assert lib.stream_handle(None) == torch.cuda.current_stream().cuda_stream
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        assert lib.stream_handle(None) == side.cuda_stream == torch.cuda.current_stream().cuda_stream
    assert lib.stream_handle(side) == side.cuda_stream
    assert lib.stream_handle(None) == torch.cuda.current_stream().cuda_stream
