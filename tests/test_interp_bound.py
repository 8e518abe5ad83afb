"""CPU property test of the edge kernels' FP32 interpolation: a numpy
restatement of the double-float position q1 + (q2 - q1) * i / (N - 1)
(endpoints split into FP32 hi/lo pairs from their FP64 values, the step
fraction from a correctly rounded FP32 reciprocal, error-free products and
sums, one final rounding), compared with the reference's FP64 position
q1 + ((q2 - q1) / (N - 1)) * i.  Per coordinate the difference must stay
within the final rounding, 2^-24 |x|, plus 2^-30 * max_k(|q1_k| + |q2_k|),
the interpolation term the classification band adds (times the agent
dimension) for edge positions.  FP32 fused multiply-adds are emulated
through FP64, where the product of two FP32 values is exact."""
import numpy as np
import pytest

F32 = np.float32
F64 = np.float64


def _fma32(a, b, c):
    return (a.astype(F64) * b.astype(F64) + c.astype(F64)).astype(F32)


def _two_sum(a, b):
    s = (a + b).astype(F32)
    bb = (s - a).astype(F32)
    e = ((a - (s - bb).astype(F32)).astype(F32) + (b - bb).astype(F32)).astype(F32)
    return s, e


def interp_df(a, b, N, i):
    """The device's FP32 position for FP64 endpoints a, b (arrays [n, D]),
    step counts N [n] and indices i [n]."""
    a_h = a.astype(F32)
    a_l = (a - a_h.astype(F64)).astype(F32)
    d = b - a
    d_h = d.astype(F32)
    d_l = (d - d_h.astype(F64)).astype(F32)
    nm1 = (N - 1).astype(F32)[:, None]
    rn = (1.0 / (N - 1).astype(F64)).astype(F32)[:, None]   # correctly rounded in all but double-rounding ties
    fi = i.astype(F32)[:, None]
    th = (fi * rn).astype(F32)
    tl = (_fma32(-th, nm1, fi) * rn).astype(F32)
    ph = (d_h * th).astype(F32)
    pl = _fma32(d_h, th, -ph)
    pl = _fma32(d_h, tl, _fma32(d_l, th, pl))
    sh, sl = _two_sum(a_h, ph)
    h = sh
    l_ = ((sl + pl).astype(F32) + a_l).astype(F32)
    return (h + l_).astype(F32), a_h, d_h


@pytest.mark.parametrize("scale,nmax", [(1.0, 600), (np.pi, 10_000), (50.0, 1 << 20), (1e3, 1 << 24)])
def test_interpolation_error_within_the_band_term(scale, nmax):
    rng = np.random.default_rng(int(scale * 7) + nmax)
    n, D = 200_000, 4
    a = rng.uniform(-scale, scale, (n, D))
    b = a + rng.uniform(-scale, scale, (n, D)) * 10.0 ** rng.uniform(-6, 0, (n, 1))
    N = rng.integers(2, nmax + 1, n)
    i = (rng.random(n) * N).astype(np.int64)
    i = np.minimum(i, N - 1)
    ref = a + ((b - a) / (N - 1).astype(F64)[:, None]) * i.astype(F64)[:, None]
    x, a_h, d_h = interp_df(a, b, N, i)
    M = np.max(np.abs(a_h.astype(F64)) + np.abs(a_h.astype(F64) + d_h.astype(F64)), axis=1)
    err = np.abs(x.astype(F64) - ref)
    allowed = 2.0 ** -24 * np.abs(x.astype(F64)) + 2.0 ** -30 * M[:, None]
    worst = np.max(err / allowed)
    assert worst <= 1.0, worst
