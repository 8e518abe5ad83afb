"""CPU property test of the abstract kernels' FP32 band: a numpy float32
restatement of the device's configuration classification (coordinates
rounded once to FP32, fused multiply-add sums of squares, the band
delta = 8 * dim * 2^-24 * (qmax + omax) around every threshold), run on
configurations placed within 1e-9 .. 1e-4 of a contact (agent against box
faces and corners, agent pairs, sphere obstacles; 2-D and 3-D agents).
Every definite FP32 verdict (free, or collides) must be the FP64 oracle's;
the undecided ones are what the device's exact FP64 pass decides.  The
fused multiply-add is emulated through FP64 (the product of two FP32 values
is exact there)."""
import numpy as np
import pytest

from conftest import pkg

F32 = np.float32


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def _up32(x: float) -> np.float32:
    f = F32(x)
    return f if float(f) >= x else np.nextafter(f, F32(np.inf))


def classify32(scene, q: np.ndarray) -> np.ndarray:
    """0 free, 1 collides, 2 undecided, per configuration (rows of q)."""
    t = scene.tables()
    A, dim = len(scene.agent_radii), scene.dim
    off = [int(o) for o in t["agent_offsets"]]
    omax = max([abs(r) for r in t["agent_radius"]] + list(np.abs(t["pair_threshold"]).ravel()) +
               list(np.abs(t["box_lo"]).ravel()) + list(np.abs(t["box_hi"]).ravel()) +
               list(np.abs(t["sphere_pos"]).ravel()) + list(np.abs(t["sphere_threshold"]).ravel()))
    omax32 = _up32(omax * (1.0 + 1e-6) + 1e-30)
    dk = F32(8.0 * dim * 2.0 ** -24)
    qf = q.astype(F32)
    qmax = np.max(np.abs(qf), axis=1)
    delta = (dk * (qmax + omax32)).astype(F32)
    n = len(q)
    coll = np.zeros(n, bool)
    unc = np.zeros(n, bool)

    def test(ss, thr_lo_hi):
        lo, hi = thr_lo_hi
        free = ss > (hi * hi).astype(F32)
        c = (lo > 0) & (ss < (lo * lo).astype(F32))
        return c, ~free & ~c

    for i in range(A):
        for j in range(i + 1, A):
            ss = np.zeros(n, F32)
            for k in range(dim):
                d = (qf[:, off[i] + k] - qf[:, off[j] + k]).astype(F32)
                ss = _fma(d, d, ss)
            thr = F32(t["pair_threshold"][i, j])
            c, u = test(ss, ((thr - F32(2) * delta).astype(F32), (thr + F32(2) * delta).astype(F32)))
            coll |= c
            unc |= u
    lo32, hi32 = t["box_lo"].astype(F32), t["box_hi"].astype(F32)
    sp32, sthr32 = t["sphere_pos"].astype(F32), t["sphere_threshold"].astype(F32)
    for i in range(A):
        c_ = qf[:, off[i]:off[i] + dim]
        r = F32(t["agent_radius"][i])
        rlo, rhi = (r - delta).astype(F32), (r + delta).astype(F32)
        for b in range(len(lo32)):
            ss = np.zeros(n, F32)
            for k in range(dim):
                v = (np.minimum(np.maximum(c_[:, k], lo32[b, k]), hi32[b, k]) - c_[:, k]).astype(F32)
                ss = _fma(v, v, ss)
            c, u = test(ss, (rlo, rhi))
            coll |= c
            unc |= u
        for o in range(len(sp32)):
            ss = np.zeros(n, F32)
            for k in range(dim):
                d = (sp32[o, k] - c_[:, k]).astype(F32)
                ss = _fma(d, d, ss)
            thr = sthr32[o, i]
            c, u = test(ss, ((thr - F32(2) * delta).astype(F32), (thr + F32(2) * delta).astype(F32)))
            coll |= c
            unc |= u
    return np.where(coll, 1, np.where(unc, 2, 0))


def _near_contacts(scene, rng, n: int) -> np.ndarray:
    """Configurations with one agent within 1e-9 .. 1e-4 of a contact (inside
    or outside), the other agents at random positions."""
    t = scene.tables()
    A, dim = len(scene.agent_radii), scene.dim
    off = t["agent_offsets"]
    q = rng.uniform(-1, 1, (n, scene.q_dim))
    gap = 10.0 ** rng.uniform(-9, -4, n) * rng.choice([-1.0, 1.0], n)
    nb, ns = len(t["box_lo"]), len(t["sphere_pos"])
    for s in range(n):
        i = int(rng.integers(A))
        r = float(t["agent_radius"][i])
        kind = int(rng.integers(3))
        if kind == 0 and nb:       # a box face or corner
            b = int(rng.integers(nb))
            lo, hi = t["box_lo"][b], t["box_hi"][b]
            p = rng.uniform(lo, hi)
            u = rng.normal(size=dim)
            for k in range(dim):   # snap to the faces the direction points at
                if rng.random() < 0.6:
                    p[k] = hi[k] if u[k] > 0 else lo[k]
                else:
                    u[k] = 0.0
            if not np.any(u):
                k = int(rng.integers(dim))
                u[k] = 1.0
                p[k] = hi[k]
            u /= np.linalg.norm(u)
            q[s, off[i]:off[i] + dim] = p + u * (r + gap[s])
        elif kind == 1 and A > 1:  # another agent
            j = int((i + 1 + rng.integers(A - 1)) % A)
            u = rng.normal(size=dim)
            u /= np.linalg.norm(u)
            q[s, off[j]:off[j] + dim] = q[s, off[i]:off[i] + dim] + u * (t["pair_threshold"][i, j] + gap[s])
        elif ns:                   # a sphere obstacle
            o = int(rng.integers(ns))
            u = rng.normal(size=dim)
            u /= np.linalg.norm(u)
            q[s, off[i]:off[i] + dim] = t["sphere_pos"][o] + u * (t["sphere_threshold"][o, i] + gap[s])
    return q


def _scene_3d(seed):
    scenes = pkg("scenes")
    rng = np.random.default_rng(seed)
    return scenes.AbstractScene(
        agent_slices=np.array([[0, 3], [3, 6], [6, 9]], dtype=np.int64), agent_radii=[0.1, 0.07, 0.13],
        box_center=rng.uniform(-0.8, 0.8, (8, 3)), box_bounds=rng.uniform(0.1, 0.4, (8, 3)),
        sphere_pos=rng.uniform(-0.8, 0.8, (4, 3)), sphere_radius=[0.05, 0.1, 0.2, 0.15], q_dim=9)


@pytest.mark.parametrize("which", ["discs", "discs_far", "spheres_3d"])
def test_definite_fp32_verdicts_are_the_oracles(oracle, which):
    scenes = pkg("scenes")
    rng = np.random.default_rng({"discs": 1, "discs_far": 2, "spheres_3d": 3}[which])
    if which == "spheres_3d":
        sc = _scene_3d(7)
    else:
        sc = scenes.make_disc_scene(0)
        if which == "discs_far":   # the scene moved far from the origin: a wider band
            sc.box_center = sc.box_center + 250.0
    q = _near_contacts(sc, rng, 60_000)   # contacts with the scene as placed (boxes near 250 when moved)
    got = classify32(sc, q)
    ref = oracle.OracleScene(sc).configs_free(q)
    assert not np.any((got == 0) & (ref == 0)), "FP32 says free where the oracle collides"
    assert not np.any((got == 1) & (ref == 1)), "FP32 says collides where the oracle is free"
    # not vacuous: many near-contact cases are still decided in FP32 (gaps
    # wider than the band), and some are left to the exact pass
    assert np.mean(got != 2) > 0.3 and np.any(got == 2)
    assert np.any(got == 0) and np.any(got == 1)
