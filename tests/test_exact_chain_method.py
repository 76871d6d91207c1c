"""The method of warp_chain (pqdts_gb300/csrc/kernels.cuh), restated on the
CPU, against the sequential chain it replaces, in exact arithmetic.

The FP64 path's dot products and sums are sequential chains in the
reference's order (acc = fma(a, b, acc), pqdts.f90:589-614).  On the GPU a
warp takes 32 steps at a time: while acc stays in one binade every step
rounds to the same grid, so each step adds an integer number of grid units
computed from the exact product, and a prefix sum gives every partial sum.
Steps that may leave the binade, ties, inexact product errors, zero / tiny /
non-finite accumulators run as one fma.  This test restates exactly that
integer method (the bit tests and comparisons of the kernel, per lane) and
checks it bit for bit against the sequential fma chain evaluated with
rationals (Fraction -> float rounds to nearest, ties to even), on data made
to hit every branch.  The kernel itself is checked on the GPU by
tests/test_gpu_ops.py::test_pdot_exact_chains.
"""
import random
import struct
from fractions import Fraction

M52 = (1 << 52) - 1
NEGZERO = -(1 << 63)


def _bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def _from_bits(b):
    return struct.unpack("<d", struct.pack("<q", b))[0]


def _fma(x, y, z):
    return float(Fraction(x) * Fraction(y) + Fraction(z))


def _acc_from(S, ea):
    m = -S if S < 0 else S
    v = _from_bits((ea << 52) | (m & M52))
    return -v if S < 0 else v


def warp_chain(acc, xs, ys, tpl=1):
    """acc <- fma(x_g, y_g, acc) for g = 0 .. 32*tpl-1, the kernel's way."""
    n = len(xs)
    assert n == 32 * tpl
    ph = [x * y for x, y in zip(xs, ys)]
    pl = [_fma(x, y, -p) for x, y, p in zip(xs, ys, ph)]
    hb = [_bits(p) for p in ph]
    pb = [_bits(p) for p in pl]
    eh = [(b >> 52) & 0x7FF for b in hb]
    zero = [((b << 1) & 0xFFFFFFFFFFFFFFFF) == 0 and (((_bits(x) << 1) & 0xFFFFFFFFFFFFFFFF) == 0 or
                                                     ((_bits(y) << 1) & 0xFFFFFFFFFFFFFFFF) == 0)
            for b, x, y in zip(hb, xs, ys)]
    mh = [(b & M52) | (1 << 52) for b in hb]
    neg = [b < 0 for b in hb]
    rel = [0 if ((q << 1) & 0xFFFFFFFFFFFFFFFF) == 0 else (1 if (q < 0) == ng else -1) for q, ng in zip(pb, neg)]
    usable = [z or (1023 - 969 <= e < 0x7FF) for z, e in zip(zero, eh)]
    plb = [q & 0x7FFFFFFFFFFFFFFF for q in pb]
    if all(zero) and _bits(acc) != NEGZERO:
        return acc  # a round of exactly zero products
    start = 0
    while start < n:
        ab = _bits(acc)
        ea = (ab >> 52) & 0x7FF
        acc_ok = 1023 - 960 <= ea < 0x7FF
        aneg = ab < 0
        k = [0] * n
        ok = [True] * n
        for g in range(start, n):
            if not acc_ok:
                ok[g] = zero[g] and ab != NEGZERO
            elif not zero[g]:
                if not usable[g] or eh[g] > ea:
                    ok[g] = False
                    continue
                sh = ea - eh[g]
                q = 0
                if sh == 0:
                    q = mh[g]
                    ok[g] = plb[g] != ((ea - 53) << 52)
                elif sh <= 53:
                    r, half = mh[g] & ((1 << sh) - 1), 1 << (sh - 1)
                    q = mh[g] >> sh
                    if r > half or (r == half and rel[g] > 0):
                        q += 1
                    ok[g] = not (r == half and rel[g] == 0)
                k[g] = -q if neg[g] else q
        A = ((ab & M52) | (1 << 52)) * (-1 if aneg else 1) if acc_ok else 0
        S, run = [0] * n, A
        for g in range(n):
            run += k[g]
            S[g] = run
        fail = None
        for g in range(start, n):
            T = -S[g] if aneg else S[g]
            if not ok[g] or (acc_ok and not ((1 << 52) + 1 <= T <= (1 << 53) - 1)):
                fail = g
                break
        if fail is None:
            if acc_ok:
                acc = _acc_from(S[n - 1], ea)
            break
        if acc_ok and fail > start:
            acc = _acc_from(S[fail - 1], ea)
        acc = _fma(xs[fail], ys[fail], acc)
        start = fail + 1
    return acc


def _sequential(acc, xs, ys):
    for x, y in zip(xs, ys):
        acc = _fma(x, y, acc)
    return acc


def _value(rng, kind):
    if kind == 0:
        return rng.uniform(-1, 1) * 2.0 ** rng.randint(-30, 30)
    if kind == 1:
        return rng.uniform(0, 1)
    if kind == 2:
        return float(rng.randint(-8, 8)) * 2.0 ** rng.randint(-3, 3)  # ties
    if kind == 3:
        return rng.choice([0.0, -0.0, 1.0, 0.5, 2.0 ** -60, 3.0, -1.5])
    if kind == 4:
        return rng.uniform(-1, 1) * 2.0 ** rng.randint(-1000, -940)  # underflowing products
    return rng.uniform(0.9, 1.1)


def test_random_chains_bitwise():
    rng = random.Random(11)
    for tpl in (1, 4):
        for _ in range(150):
            kind = rng.randint(0, 5)
            xs = [_value(rng, kind) for _ in range(32 * tpl)]
            ys = [_value(rng, rng.choice([kind, 1, 5])) for _ in range(32 * tpl)]
            acc = rng.choice([0.0, -0.0, _value(rng, kind), _value(rng, 1), 1e-300, 2.0 ** 10])
            assert _bits(warp_chain(acc, xs, ys, tpl)) == _bits(_sequential(acc, xs, ys))


def test_targeted_chains_bitwise():
    """Ties at the accumulator's exponent (3 * (2^52 + 1)), accumulators at
    binade edges and at +-0, cancellation, huge and zero terms."""
    rng = random.Random(12)
    for _ in range(200):
        e = rng.randint(-20, 20)
        xs, ys = [], []
        for _ in range(32):
            t = rng.randint(0, 5)
            if t == 0:
                xs.append(3.0 * 2.0 ** e)
                ys.append(float((1 << 52) + rng.choice([1, 3, 5])))
            elif t == 1:
                xs.append(rng.choice([1.0, -1.0]) * 2.0 ** (e + 50))
                ys.append(rng.choice([0.5, 1.5, -0.5]))
            elif t == 2:
                xs.append(rng.uniform(-1, 1) * 2.0 ** (e + 52))
                ys.append(1.0)
            elif t == 3:
                xs.append(2.0 ** (e + rng.randint(-60, 60)))
                ys.append(rng.choice([1.0, -1.0]))
            elif t == 4:
                xs.append(0.0)
                ys.append(rng.uniform(-1, 1))
            else:
                xs.append(rng.uniform(-1, 1))
                ys.append(rng.uniform(-1, 1) * 2.0 ** (e + 54))
        E = e + 53 + rng.randint(-2, 2)
        acc = rng.choice([2.0 ** E, 2.0 ** E - 2.0 ** (E - 53), -(2.0 ** E), 2.0 ** E * 1.5, 0.0, -0.0,
                          2.0 ** E + 2.0 ** (E - 52)])
        assert _bits(warp_chain(acc, xs, ys)) == _bits(_sequential(acc, xs, ys))


def test_long_dot_product_chain():
    """A 2048-step dot product in rounds of 32 equals the sequential chain."""
    rng = random.Random(13)
    xs = [rng.uniform(0, 1) if rng.random() < 0.3 else 0.0 for _ in range(2048)]
    ys = [rng.uniform(-0.2, 1) for _ in range(2048)]
    acc = 0.0
    for j in range(0, 2048, 32):
        acc = warp_chain(acc, xs[j:j + 32], ys[j:j + 32])
    assert _bits(acc) == _bits(_sequential(0.0, xs, ys))


def test_binade_edge_steps():
    """Steps whose exact sum falls just below a power of two: there the
    correctly rounded sum lies on the finer grid of the binade below, so the
    method must not take them on the accumulator's grid (a rounded sum one
    grid unit above the binade's start is the closest it accepts)."""
    ulp = 2.0 ** -52
    cases = [
        (1.0 + ulp, -1.3 * ulp),  # exact 1 - 0.3 ulp: the nearest double is 1 - ulp/2
        (1.0 + ulp, -1.2 * ulp),
        (1.0 + 2 * ulp, -2.3 * ulp),
        (-(1.0 + ulp), 1.3 * ulp),
        (2.0 - ulp, 0.6 * ulp),  # rounds up to the next binade's start
        (4.0 + 4 * ulp, -4.6 * ulp),
    ]
    for acc, t in cases:
        xs = [t] + [0.0] * 31
        ys = [1.0] * 32
        want = _sequential(acc, xs, ys)
        assert _bits(warp_chain(acc, xs, ys)) == _bits(want), (acc, t, want)
    # the same steps inside a round of other terms
    rng = random.Random(14)
    for _ in range(50):
        acc = 1.0 + ulp
        xs = [rng.uniform(0, 1) * 2.0 ** -80 for _ in range(32)]
        xs[rng.randrange(32)] = -1.3 * ulp
        ys = [1.0] * 32
        assert _bits(warp_chain(acc, xs, ys)) == _bits(_sequential(acc, xs, ys))
