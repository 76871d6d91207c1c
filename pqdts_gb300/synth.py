"""Seeded synthetic detector-tomography instances (numpy only).

The reference ships no datasets; its inputs are a probe matrix F (D x M) and
measured outcome frequencies P (D x N).  These generators produce instances of
the shapes and value distributions of the benchmark configurations:

* probe d is a coherent state with mean photon number x_d, x linearly spaced
  0.01 .. x_max, so F[d, i] = Poisson pmf(i; x_d) for i < M; entries below
  1e-16 are dropped (each row keeps one contiguous window, since the pmf is
  unimodal);
* the true POVM is an ideal detector of efficiency eta:
  Pi[i, n] = Binomial(n; i, eta) for n < N-1, with the tail mass P(k >= N-1)
  in the last column, so every row lies on the probability simplex;
* P[d, :] is a multinomial sample of (F Pi)[d, :] / sum with `shots` counts,
  divided by `shots`.

Files are written exactly as pqdts.py's npz_to_fortran does (pqdts.py:15-28):
data/{F,P}_{row,col,data}.bin with int32 0-based COO indices and float64 data.
The dense data/F.bin and data/P.bin side files of the wrapper are not written
(the solver never reads them).
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np
from scipy import stats

CUTOFF = 1e-16

# Benchmark configurations, keyed by their position in the benchmark list.
CONFIGS = {
    1: dict(M=200, N=20, D=400, xmax=150.0, eta=0.9, shots=10**6, gamma=1e-4, eps=1e-6),
    2: dict(M=2000, N=200, D=4000, xmax=1800.0, eta=0.9, shots=10**7, gamma=1e-5, eps=1e-6),
    3: dict(M=10000, N=1000, D=20000, xmax=9000.0, eta=0.75, shots=10**8, gamma=1e-6, eps=1e-6),
    5: dict(M=50000, N=5000, D=100000, xmax=45000.0, eta=0.85, shots=10**8, gamma=1e-6, eps=1e-6),
    # configuration 5's dense-F variant: every entry of F kept (N, x_max, eta
    # are this generator's choice)
    6: dict(M=8192, N=256, D=8192, xmax=7373.0, eta=0.85, shots=10**8, gamma=1e-6, eps=1e-6, dense=True),
}


@dataclasses.dataclass
class Instance:
    M: int
    N: int
    D: int
    gamma: float
    eps: float
    band_lo: np.ndarray  # int64 (D,), first column of row d's window, -1 if empty
    band_hi: np.ndarray  # int64 (D,), last column (inclusive)
    band_val: np.ndarray  # float64, concatenated windows
    P: np.ndarray  # float64 (D, N) row-major == the reference's P(N, D)
    pi_true: np.ndarray | None = None

    @property
    def nnz(self) -> int:
        return int(self.band_val.size)

    def band_offsets(self) -> np.ndarray:
        w = np.where(self.band_lo >= 0, self.band_hi - self.band_lo + 1, 0)
        off = np.zeros(self.D, dtype=np.int64)
        off[1:] = np.cumsum(w)[:-1]
        return off

    def coo_F(self):
        """F as COO (row-major order) with int32 indices, like coo_array(csr)."""
        w = np.where(self.band_lo >= 0, self.band_hi - self.band_lo + 1, 0)
        rows = np.repeat(np.arange(self.D, dtype=np.int32), w)
        starts = np.repeat(self.band_lo, w)
        within = np.arange(w.sum(), dtype=np.int64) - np.repeat(self.band_offsets(), w)
        cols = (starts + within).astype(np.int32)
        return rows, cols, self.band_val.copy()

    def coo_P(self):
        r, c = np.nonzero(self.P)
        return r.astype(np.int32), c.astype(np.int32), self.P[r, c].astype(np.float64)

    def dense_F(self) -> np.ndarray:
        F = np.zeros((self.D, self.M))
        r, c, v = self.coo_F()
        F[r, c] = v
        return F


# Elementary functions from IEEE basic operations only (+, -, *, /, rint,
# ldexp, frexp), so the generated F is bit-identical on every platform
# (numpy's vectorised exp/log differ between x86 and aarch64 builds).
_LN2_HI = 6.93147180369123816490e-01
_LN2_LO = 1.90821492927058770002e-10
_INV_LN2 = 1.44269504088896338700e+00


def det_exp(t):
    t = np.asarray(t, dtype=np.float64)
    k = np.rint(t * _INV_LN2)
    r = (t - k * _LN2_HI) - k * _LN2_LO
    # Taylor series of e^r, |r| <= 0.35: 18 terms reach 1e-17
    p = np.ones_like(r)
    term = np.ones_like(r)
    for n in range(1, 19):
        term = term * r / n
        p = p + term
    return np.ldexp(p, k.astype(np.int64))


def det_log(x):
    x = np.asarray(x, dtype=np.float64)
    m, e = np.frexp(x)  # x = m * 2^e, m in [0.5, 1)
    small = m < 0.7071067811865476
    m = np.where(small, m * 2.0, m)
    e = np.where(small, e - 1, e).astype(np.float64)
    s = (m - 1.0) / (m + 1.0)  # |s| < 0.172
    s2 = s * s
    acc = np.zeros_like(s)
    for n in range(27, 0, -2):
        acc = acc * s2 + 1.0 / n
    return (e * _LN2_HI + 2.0 * s * acc) + e * _LN2_LO


def det_log_factorial(i):
    """log(i!) for integer arrays i >= 0 (Stirling series above 16)."""
    i = np.asarray(i, dtype=np.int64)
    out = np.zeros(i.shape, dtype=np.float64)
    fact = np.cumprod(np.concatenate([[1.0], np.arange(1, 17, dtype=np.float64)]))  # exact up to 16!
    lo = i <= 16
    out[lo] = det_log(fact[i[lo]])
    z = (i[~lo] + 1).astype(np.float64)
    zi = 1.0 / z
    zi2 = zi * zi
    series = zi * (1.0 / 12 - zi2 * (1.0 / 360 - zi2 * (1.0 / 1260 - zi2 * (1.0 / 1680 - zi2 / 1188))))
    half_log_2pi = 0.91893853320467274178
    out[~lo] = (z - 0.5) * det_log(z) - z + half_log_2pi + series
    return out


def poisson_bands(M: int, D: int, xmax: float, cutoff: float = CUTOFF, dense: bool = False):
    """Row windows of F[d, i] = Poisson pmf(i; x_d), x_d = linspace(0.01, xmax, D).
    dense=True keeps every entry (each row spans all M columns)."""
    x = np.linspace(0.01, xmax, D)
    lo = np.full(D, -1, dtype=np.int64)
    hi = np.full(D, -1, dtype=np.int64)
    vals = []
    logx = det_log(x)
    if dense:
        ii = np.arange(M, dtype=np.int64)
        lf = det_log_factorial(ii)
        for d0 in range(0, D, 256):
            d1 = min(D, d0 + 256)
            t = ii[None, :] * logx[d0:d1, None] - x[d0:d1, None] - lf[None, :]
            vals.append(det_exp(np.maximum(t, -745.0)).ravel())
        lo[:] = 0
        hi[:] = M - 1
        return lo, hi, np.concatenate(vals)
    lf_all = det_log_factorial(np.arange(M, dtype=np.int64))  # elementwise: the same values per row
    for d in range(D):
        xd = float(x[d])
        half = 12.0 * math.sqrt(xd) + 40.0
        a = max(0, int(math.floor(xd - half)))
        b = min(M - 1, int(math.ceil(xd + half)))
        if a > b:
            continue
        ii = np.arange(a, b + 1, dtype=np.int64)
        p = det_exp(ii * logx[d] - xd - lf_all[a : b + 1])
        keep = np.nonzero(p >= cutoff)[0]
        if keep.size == 0:
            continue
        k0, k1 = keep[0], keep[-1]
        # the window must contain the whole super-cutoff region
        assert (a == 0 or k0 > 0) and (b == M - 1 or k1 < p.size - 1), "window too narrow"
        lo[d] = a + k0
        hi[d] = a + k1
        vals.append(p[k0 : k1 + 1])
    val = np.concatenate(vals) if vals else np.zeros(0)
    return lo, hi, val


def binomial_povm(M: int, N: int, eta: float) -> np.ndarray:
    i = np.arange(M)[:, None]
    n = np.arange(N - 1)[None, :]
    pi = np.empty((M, N))
    pi[:, : N - 1] = stats.binom.pmf(n, i, eta)
    pi[:, N - 1] = stats.binom.sf(N - 2, np.arange(M), eta)
    return pi


def band_matvec(lo, hi, val, X, block=None):
    """(F @ X) for banded F and dense X (M, K).  block=None: one row at a
    time (the generator's reference order); block=b: b rows at a time as a
    dense product over their union band (large instances)."""
    D = lo.size
    out = np.zeros((D, X.shape[1]))
    w = np.where(lo >= 0, hi - lo + 1, 0)
    offs = np.concatenate([[0], np.cumsum(w)[:-1]])
    if block is None:
        for d in range(D):
            if lo[d] < 0:
                continue
            out[d] = val[offs[d] : offs[d] + w[d]] @ X[lo[d] : hi[d] + 1]
        return out
    for d0 in range(0, D, block):
        rows = [d for d in range(d0, min(D, d0 + block)) if lo[d] >= 0]
        if not rows:
            continue
        a = min(lo[d] for d in rows)
        b = max(hi[d] for d in rows)
        Fb = np.zeros((len(rows), b - a + 1))
        for j, d in enumerate(rows):
            Fb[j, lo[d] - a : hi[d] - a + 1] = val[offs[d] : offs[d] + w[d]]
        out[rows] = Fb @ X[a : b + 1]
    return out


def sample_P(FPi: np.ndarray, shots: int, rng: np.random.Generator) -> np.ndarray:
    probs = np.clip(FPi, 0.0, None)
    s = probs.sum(axis=1, keepdims=True)
    s[s == 0] = 1.0
    probs = probs / s
    counts = rng.multinomial(shots, probs)
    return counts.astype(np.float64) / float(shots)


def make_instance(M, N, D, xmax, eta, shots, gamma, eps, seed=0, keep_truth=False, dense=False) -> Instance:
    rng = np.random.default_rng(seed)
    lo, hi, val = poisson_bands(M, D, xmax, dense=dense)
    pi = binomial_povm(M, N, eta)
    # instances above 1e8 entries of P use the blocked product (its own
    # summation order); the benchmark configurations 1-3 and the batch keep
    # the row-by-row one
    FPi = band_matvec(lo, hi, val, pi, block=256 if D * N > 10**8 else None)
    P = sample_P(FPi, shots, rng)
    return Instance(M, N, D, gamma, eps, lo, hi, val, P, pi if keep_truth else None)


def make_config(cfg: int, seed: int = 0, keep_truth=False) -> Instance:
    return make_instance(**CONFIGS[cfg], seed=seed, keep_truth=keep_truth)


def make_batch(n_base=8, n_resample=8, shots=10**7, seed=0, m_range=(500, 5000), n_range=(50, 500)):
    """Uneven batch: M log-uniform, N uniform, D = 2M, eta uniform 0.6..0.95,
    x_max = 0.9 M; each base instance gets n_resample multinomial draws of P,
    paired with gamma log-spaced 1e-7 .. 1e-2 (a regularisation sweep)."""
    rng = np.random.default_rng(seed)
    gammas = np.logspace(-7, -2, n_resample)
    out = []
    for b in range(n_base):
        M = int(round(math.exp(rng.uniform(math.log(m_range[0]), math.log(m_range[1])))))
        N = int(rng.integers(n_range[0], n_range[1] + 1))
        D = 2 * M
        eta = float(rng.uniform(0.6, 0.95))
        lo, hi, val = poisson_bands(M, D, 0.9 * M)
        FPi = band_matvec(lo, hi, val, binomial_povm(M, N, eta))
        for r in range(n_resample):
            P = sample_P(FPi, shots, rng)
            out.append(Instance(M, N, D, float(gammas[r]), 1e-6, lo, hi, val, P))
    return out


def write_data_dir(inst: Instance, workdir: str, with_F: bool = True):
    """Write data/{F,P}_{row,col,data}.bin under workdir; returns (nnzF, nnzP)."""
    ddir = os.path.join(workdir, "data")
    os.makedirs(ddir, exist_ok=True)
    nF = -1
    if with_F:
        r, c, v = inst.coo_F()
        r.tofile(os.path.join(ddir, "F_row.bin"))
        c.tofile(os.path.join(ddir, "F_col.bin"))
        v.tofile(os.path.join(ddir, "F_data.bin"))
        nF = int(v.size)
    r, c, v = inst.coo_P()
    r.tofile(os.path.join(ddir, "P_row.bin"))
    c.tofile(os.path.join(ddir, "P_col.bin"))
    v.tofile(os.path.join(ddir, "P_data.bin"))
    return nF, int(v.size)
