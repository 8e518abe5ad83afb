"""CPU property test of the edge kernels' FP32 step count: a numpy float32
restatement of the device's estimate (the largest FP32 coordinate
difference over the FP32 resolution, correctly rounded, accepted only when
its fractional part lies more than 4.8e-7 * max(t, 1) from an integer) must
give the reference's N = max(2, int(max|q1 - q2| / resolution) + 1)
(abstract_env.py:321-323) whenever it is accepted; the rest go to the FP64
computation.  Edge lengths are drawn at, just above and just below integer
multiples of the resolution."""
import numpy as np
import pytest

F32 = np.float32


def steps_fp32(m32: np.ndarray, res32: np.float32):
    """(accepted, N) per edge, as the device computes them."""
    ok = (res32 >= F32(2.0 ** -60)) & (m32 >= F32(2.0 ** -60))
    t32 = (m32 / res32).astype(F32)
    ok &= t32 < F32(4194304.0)
    fl = np.floor(t32).astype(F32)
    fr = (t32 - fl).astype(F32)
    tol = (F32(4.8e-7) * np.maximum(t32, F32(1.0))).astype(F32)
    ok &= (fr > tol) & (fr < (F32(1.0) - tol))
    N = np.maximum(2, fl.astype(np.int64) + 1)
    return ok, N


@pytest.mark.parametrize("res", [0.01, 0.05, 0.001, 0.1, 0.0123456789, 1e-5])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_accepted_fp32_step_counts_are_the_references(res, dtype):
    rng = np.random.default_rng(int(res * 1e6) + (dtype == np.float32))
    n, D = 300_000, 6
    a = rng.uniform(-3, 3, (n, D)).astype(dtype)
    k = np.floor(10.0 ** rng.uniform(0, 3.7, n))             # edge lengths of 1 .. 5,000 steps
    near = rng.random(n) < 0.5                                  # half at an integer multiple (+- up to 1e-4)
    frac = np.where(near, rng.choice([0.0, 1.0, -1.0], n) * 10.0 ** rng.uniform(-12, -4, n), rng.random(n))
    m_target = (k + frac) * res
    direction = rng.integers(0, D, n)
    b = a.astype(np.float64) + rng.uniform(-1, 1, (n, D)) * m_target[:, None] * 0.5
    b[np.arange(n), direction] = a[np.arange(n), direction] + m_target * rng.choice([-1.0, 1.0], n)
    b = b.astype(dtype)
    # the reference: FP64 differences (float32 inputs widened first), max, / res, int() + 1
    diff64 = np.abs(b.astype(np.float64) - a.astype(np.float64))
    N_ref = np.maximum(2, (np.max(diff64, axis=1) / res).astype(np.int64) + 1)
    # the device: the FP32 rounding of each FP64 difference (exact for float32 inputs' FP64 difference)
    m32 = np.max(np.abs(diff64.astype(F32)), axis=1)
    ok, N = steps_fp32(m32, F32(res))
    assert np.array_equal(N[ok], N_ref[ok])
    assert ok[~near].mean() > 0.99  # edges with a generic length take the FP32 path
    if dtype == np.float64 or res >= 1e-3:   # (float32 endpoints move an edge by ~2e-7 / res steps)
        assert (~ok[near]).mean() > 0.5  # most near-integer ones are handed to FP64
