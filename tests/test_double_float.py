"""The double-FP32 arithmetic of the mixed path's gradient and objective-check
products (df_split / df_fma / df_renorm in pqdts_gb300/csrc/kernels.cuh),
restated with numpy float32 operations and checked against exact rational
sums on the CPU: each output within 2 * sqrt(K) * 2^-48 of the sum of its
K terms' magnitudes (the low word's own roundings dominate and add up like
a random walk: measured 2^-45 at 100 terms, 2^-43 at 4400).

The restatement rounds an fma twice (the exact product plus the addend in
float64, then to float32); that differs from one rounding only on rare
ties, which does not affect the bound tested here.  The GPU kernels
themselves are held to the FP64 oracle in tests/test_gpu_ops.py.
"""
from fractions import Fraction

import numpy as np

F32 = np.float32


def _split(v):
    h = v.astype(F32)
    return h, (v - h.astype(np.float64)).astype(F32)


def _fma(a, b, c):
    # float32 operands: a*b is exact in float64
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def _df_dot(a, x, renorm_every=8):
    """sum_k a[:, k] * x[:, k] per row, as the kernels accumulate it."""
    ah, al = _split(a)
    xh, xl = _split(x)
    sh = np.zeros(a.shape[0], F32)
    sl = np.zeros(a.shape[0], F32)
    for k in range(a.shape[1]):
        p = ah[:, k] * xh[:, k]
        q = _fma(ah[:, k], xh[:, k], -p)
        q = _fma(ah[:, k], xl[:, k], q)
        q = _fma(al[:, k], xh[:, k], q)
        s = sh + p
        bb = s - sh
        t = (sh - (s - bb)) + (p - bb)
        sh = s
        sl = sl + (t + q)
        if k % renorm_every == renorm_every - 1:
            s = sh + sl
            sl = sl - (s - sh)
            sh = s
    return sh.astype(np.float64) + sl.astype(np.float64)


def _exact(a, x):
    out, mag = [], []
    for i in range(a.shape[0]):
        terms = [Fraction(float(u)) * Fraction(float(v)) for u, v in zip(a[i], x[i])]
        out.append(sum(terms))
        mag.append(sum(abs(t) for t in terms))
    return out, mag


def _check(a, x):
    got = _df_dot(a, x)
    ex, mag = _exact(a, x)
    worst = 0.0
    for g, e, m in zip(got, ex, mag):
        if m == 0:
            assert g == 0.0
            continue
        worst = max(worst, float(abs(Fraction(float(g)) - e) / m))
    bound = 2.0 * np.sqrt(a.shape[1]) * 2.0**-48
    assert worst <= bound, (worst, bound)
    return worst


def test_forward_terms_poisson_band():
    """F.X terms: band values spanning 1e-16..0.3 (Poisson-like), X in [0, 1]
    with some entries tiny or zero."""
    rng = np.random.default_rng(0)
    rows, k = 64, 400
    a = 10.0 ** rng.uniform(-16, -0.5, (rows, k))
    x = rng.random((rows, k))
    x[rng.random(x.shape) < 0.2] = 0.0
    x[rng.random(x.shape) < 0.1] *= 1e-12
    _check(a, x)


def test_long_bands():
    """4400 terms (the widest transposed rows of M=5e4, N=5e3, D=1e5)."""
    rng = np.random.default_rng(3)
    a = 10.0 ** rng.uniform(-16, -0.5, (16, 4400))
    x = rng.random((16, 4400))
    _check(a, x)


def test_transposed_terms_signed_residual():
    """F^T.R terms: residuals of both signs (heavy cancellation)."""
    rng = np.random.default_rng(1)
    rows, k = 64, 600
    a = 10.0 ** rng.uniform(-12, -0.5, (rows, k))
    r = rng.standard_normal((rows, k)) * 1e-4
    _check(a, r)


def test_double_float_beats_float32_and_matches_float64_scale():
    """Against plain FP32 accumulation the error drops by many orders; it is
    of the order of a float64 chain's."""
    rng = np.random.default_rng(2)
    a = rng.random((32, 500))
    x = rng.standard_normal((32, 500))
    ex, mag = _exact(a, x)
    err_df = max(float(abs(Fraction(float(g)) - e) / m) for g, e, m in zip(_df_dot(a, x), ex, mag))
    f32 = np.zeros(32, F32)
    for k in range(500):
        f32 = _fma(a[:, k].astype(F32), x[:, k].astype(F32), f32)
    err_32 = max(float(abs(Fraction(float(g)) - e) / m) for g, e, m in zip(f32.astype(np.float64), ex, mag))
    assert err_df < 1e-6 * err_32
    assert err_df <= 2.0 * np.sqrt(500) * 2.0**-48
