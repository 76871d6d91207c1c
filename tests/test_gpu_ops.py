"""Per-operation parity of the CUDA path (through the C ABI) against the oracle.

FP64 path: every product accumulates in the reference's order with one fma
per term, every reduction follows the oracle's order, and the projection is
Condat's algorithm in the reference's visiting order -- so every operation
must be bit-identical to the oracle (np.array_equal, ==).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu



def _pair(inst, precision=0, tensor_cores=-1):
    import pqdts_gb300 as pq
    from oracle.oracle import Oracle

    s = pq.Solver(0)
    s.set_option("tensor_cores", tensor_cores)
    s.set_instance(inst, precision)
    return s, Oracle.from_instance(inst)


def _random_x(inst, seed, feasible=True):
    rng = np.random.default_rng(seed)
    X = rng.random((inst.M, inst.N))
    if feasible:
        X /= X.sum(axis=1, keepdims=True)
        X[rng.random(X.shape) < 0.2] = 0.0
        X /= np.maximum(X.sum(axis=1, keepdims=True), 1e-300)
    return np.asfortranarray(X)


def _maxr(X):
    return np.argmax(X, axis=1).astype(np.int32)


@pytest.mark.parametrize("which", ["cfg1", "small"])
def test_bands_and_bdiag(built, request, which):
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    lo, hi, nnz = s.bands()
    olo, ohi, _, oval = o.bands()
    assert np.array_equal(lo, olo) and np.array_equal(hi, ohi) and nnz == oval.size
    for full in (True, False):
        m = None if full else _maxr(_random_x(inst, 1))
        s.set_space(full, m)
        o.set_space(full, m)
        assert np.array_equal(s.Bdiag(), o.Bdiag())


@pytest.mark.parametrize("which", ["cfg1", "small"])
def test_redO_bitwise(built, request, which):
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    X = _random_x(inst, 2)
    s.set_x(X)
    assert np.array_equal(s.redO(), o.redO(X))


@pytest.mark.parametrize("which", ["cfg1", "small"])
@pytest.mark.parametrize("full", [True, False])
def test_L_dL(built, request, which, full):
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    X = _random_x(inst, 3)
    m = None if full else _maxr(X)
    s.set_space(full, m)
    o.set_space(full, m)
    s.set_x(X)
    Lg = s.L()
    Lo, Xo = o.L(X)
    assert Lg == Lo
    assert np.array_equal(s.get_x(), Xo)  # reduced space: identical max-column rebuild
    s.set_x(X)
    G = s.dL()
    Go, Xo2 = o.dL(X)
    assert np.array_equal(G, Go)
    assert np.array_equal(s.get_x(), Xo2)


@pytest.mark.parametrize("which", ["cfg1", "small"])
@pytest.mark.parametrize("full", [True, False])
def test_BF_bitwise(built, request, which, full):
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    X = _random_x(inst, 4)
    m = None if full else _maxr(X)
    s.set_space(full, m)
    o.set_space(full, m)
    V = np.asfortranarray(np.random.default_rng(5).standard_normal((inst.M, inst.N)))
    assert np.array_equal(s.BF(V), o.BF(V))


@pytest.mark.parametrize("which", ["cfg1", "small"])
def test_doproj(built, request, which):
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    Y = np.asfortranarray(np.random.default_rng(6).standard_normal((inst.M, inst.N)) * 0.7 + 0.05)
    s.set_x(Y)
    s.doproj()
    Xg = s.get_x()
    Xo = o.doproj(Y)
    assert np.array_equal(Xg, Xo)
    assert Xg.min() >= 0.0
    assert np.max(np.abs(Xg.sum(axis=1) - 1.0)) < 1e-13


@pytest.mark.parametrize("which", ["cfg1", "small"])
def test_doproj2_bitwise(built, request, which):
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    X = _random_x(inst, 7)
    Y = np.asfortranarray(X + 0.01 * np.random.default_rng(8).standard_normal(X.shape))
    m = _maxr(X)
    s.set_space(False, m)
    o.set_space(False, m)
    s.set_x(Y)
    xmin = s.doproj2()
    Xo, xmino = o.doproj2(Y)
    assert np.array_equal(s.get_x(), Xo)
    assert xmin == xmino


@pytest.mark.parametrize("which", ["cfg1", "small"])
@pytest.mark.parametrize("full", [True, False])
def test_conv_test(built, request, which, full):
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    X = _random_x(inst, 9)
    m = None if full else _maxr(X)
    s.set_space(full, m)
    o.set_space(full, m)
    s.set_x(X)
    cg = s.conv_test()
    co, Xo, _ = o.conv_test(X)
    assert cg == co
    assert np.array_equal(s.get_x(), Xo)


def test_simplexproj_dropin(built):
    """pqdts_cuda_simplexproj is the drop-in for simplexproj_condat_."""
    import pqdts_gb300 as pq
    from oracle.oracle import condat

    rng = np.random.default_rng(10)
    with pq.Solver(0) as s:
        for n in (1, 2, 3, 31, 32, 33, 200, 1000):
            Y = rng.standard_normal((5, n)) * rng.choice([1e-3, 1.0, 50.0])
            Xg = s.simplexproj(Y)
            Xo = np.stack([condat(y) for y in Y])
            assert np.array_equal(Xg, Xo)
            assert Xg.min() >= 0 and np.max(np.abs(Xg.sum(1) - 1)) < 1e-12


def test_internal_F(built):
    """F computed internally (nnzF < 0, M == (D-1)^2), random P from the seeded stream."""
    import pqdts_gb300 as pq
    from oracle.oracle import Oracle

    M, N, D = 400, 20, 21
    with pq.Solver(0) as s:
        s.set_problem_coo(M, N, D, None, None, 1e-4)
        o = Oracle(M, N, D, 1e-4, None, None)
        lo, hi, nnz = s.bands()
        olo, ohi, _, oval = o.bands()
        assert np.array_equal(lo, olo) and np.array_equal(hi, ohi) and nnz == oval.size
        X = _random_x(type("I", (), {"M": M, "N": N})(), 11)
        s.set_x(X)
        assert np.array_equal(s.dL(), o.dL(X)[0])
        assert np.array_equal(s.maxr(), o.maxr())


@pytest.mark.parametrize("D", [21, 61])
def test_internal_F_on_device(built, D):
    """Internal F computed on the device (option internal_f = 1; the default
    for mixed problems): the same windows as the host's (the oracle's), and
    values within 1e-12 relative (CUDA's lgamma / exp / log against the
    host's libm), seen through F.X at a positive X."""
    import pqdts_gb300 as pq
    from oracle.oracle import Oracle

    M, N = (D - 1) ** 2, 8
    o = Oracle(M, N, D, 1e-4, None, None)
    olo, ohi, _, oval = o.bands()
    X = _random_x(type("I", (), {"M": M, "N": N})(), 12)
    Oo = o.redO(X)
    for prec, opt in ((pq.FP64, 1), (pq.MIXED, -1)):
        with pq.Solver(0) as s:
            s.set_option("internal_f", opt)
            s.set_problem_coo(M, N, D, None, None, 1e-4, prec)
            lo, hi, nnz = s.bands()
            assert np.array_equal(lo, olo) and np.array_equal(hi, ohi) and nnz == oval.size
            s.set_x(X)
            Og = s.redO()
            assert np.max(np.abs(Og - Oo) / np.maximum(np.abs(Oo), 1e-300)) <= 1e-12
            if prec == pq.MIXED:
                st = s.solve(mode=2, maxiter=30, eps=1e-6)
                Xs = s.get_x()
                assert np.isfinite(st["L"]) and Xs.min() >= 0.0
                assert np.max(np.abs(Xs.sum(axis=1) - 1.0)) <= 1e-12


def test_errors_are_codes(built):
    import pqdts_gb300 as pq

    with pq.Solver(0) as s:
        with pytest.raises(pq.PqdtsError, match="no problem set"):
            s.L()
        with pytest.raises(pq.PqdtsError, match="out of range"):
            s.set_problem_coo(10, 3, 5, (np.array([0]), np.array([99]), np.array([1.0])), None, 0.0)
        with pytest.raises(pq.PqdtsError, match=r"\(D-1\)"):
            s.set_problem_coo(10, 3, 5, None, None, 0.0)


@pytest.mark.parametrize("full", [True, False])
def test_BF32_mixed_precision(built, cfg1, full):
    """The mixed solver's FP32 Hessian product against the FP64 oracle:
    FP32 values and accumulation, so relative to the product's scale the
    error is bounded by a few FP32 ulps times sqrt(band width).  (CUDA-core
    tiles; the tensor-core variant is tests/test_gpu_tc.py.)"""
    s, o = _pair(cfg1, precision=1, tensor_cores=0)
    X = _random_x(cfg1, 4)
    m = None if full else _maxr(X)
    s.set_space(full, m)
    o.set_space(full, m)
    V = np.asfortranarray(np.random.default_rng(5).standard_normal((cfg1.M, cfg1.N)))
    H32 = s.BF32(V)
    H64 = o.BF(V)
    err = np.max(np.abs(H32 - H64)) / np.max(np.abs(H64))
    assert err < 2e-5, err


def _df_instances():
    from pqdts_gb300 import synth

    return {
        # N > 1024: two column chunks per row block
        "wide": synth.make_instance(M=40, N=1100, D=90, xmax=60.0, eta=0.8, shots=10**6, gamma=1e-3, eps=1e-6,
                                    seed=7),
    }


@pytest.mark.parametrize("which", ["cfg1", "small", "mid", "empty_rows", "wide"])
@pytest.mark.parametrize("full", [True, False])
def test_L_dL_double_float(built, request, which, full):
    """The mixed path's objective and gradient products in double-FP32
    (pairs of FP32 numbers): ~sqrt(K) * 2^-48 relative to the terms' magnitudes, so L
    within 1e-12 relative and dL within 1e-11 of max|dL| of the FP64 oracle."""
    import pqdts_gb300 as pq
    from oracle.oracle import Oracle

    inst = _df_instances()[which] if which == "wide" else request.getfixturevalue(which)
    s = pq.Solver(0)
    s.set_option("df_products", 1)
    s.set_instance(inst, pq.MIXED)
    assert s.get_option("sched.df_fwd") == 1 and s.get_option("sched.df_trans") == 1
    o = Oracle.from_instance(inst)
    X = _random_x(inst, 3)
    m = None if full else _maxr(X)
    s.set_space(full, m)
    o.set_space(full, m)
    s.set_x(X)
    Lg = s.L()
    Lo, _ = o.L(X)
    assert abs(Lg - Lo) <= 1e-12 * abs(Lo), (Lg, Lo)
    s.set_x(X)
    G = s.dL()
    Go, _ = o.dL(X)
    err = np.max(np.abs(G - Go)) / np.max(np.abs(Go))
    assert err < 1e-11, err
    s.close()


def _sparse_x(inst, seed):
    """A feasible X that is zero except near n = 0.6 i N / M and in the last
    column: the shape of a tomography iterate (an outcome reached from photon
    numbers near n / eta, the tail mass in the last column)."""
    rng = np.random.default_rng(seed)
    M, N = inst.M, inst.N
    X = np.zeros((M, N))
    for i in range(M):
        c = min(N - 1, int(0.6 * i * N / M))
        lo, hi = max(0, c - 2), min(N, c + 3)
        X[i, lo:hi] = rng.random(hi - lo)
        X[i, N - 1] = rng.random()
    return np.asfortranarray(X / X.sum(1, keepdims=True))


@pytest.mark.parametrize("which", ["cfg1", "wide", "banded"])
@pytest.mark.parametrize("precision", [0, 1])
def test_row_masks_forward_product(built, request, which, precision):
    """The forward product F.X visiting only the rows of X where a warp's 32
    columns hold a non-zero (row-occupancy masks): FP64 -- the same bits as
    the full chains, in L and in dL (whose residual it forms), and the
    oracle's; double-FP32 (mixed) -- the same objective to 1e-14 and
    gradient to 1e-13 of its scale, and the oracle's to 1e-12 / 1e-11."""
    import pqdts_gb300 as pq
    from oracle.oracle import Oracle
    from pqdts_gb300 import synth

    if which == "banded":
        inst = synth.make_instance(M=300, N=200, D=600, xmax=250.0, eta=0.8, shots=10**6, gamma=1e-4, eps=1e-6, seed=8)
    else:
        inst = _df_instances()[which] if which == "wide" else request.getfixturevalue(which)
    X = _sparse_x(inst, 5)
    assert np.mean(X == 0.0) > 0.5
    out = {}
    for masks in (1, 0):
        with pq.Solver(0) as s:
            s.set_option("row_masks", masks)
            s.set_instance(inst, precision)
            s.set_x(X)
            L = s.L()
            s.set_x(X)
            out[masks] = (L, s.dL())
    o = Oracle.from_instance(inst)
    Lo, _ = o.L(X)
    Go, _ = o.dL(X)
    (L1, G1), (L0, G0) = out[1], out[0]
    if precision == 0:
        assert L1 == L0 == Lo
        assert np.array_equal(G1, G0) and np.array_equal(G1, Go)
    else:
        assert abs(L1 - L0) <= 1e-14 * abs(L0)
        assert abs(L1 - Lo) <= 1e-12 * abs(Lo)
        assert np.max(np.abs(G1 - G0)) <= 1e-13 * np.max(np.abs(G0))
        assert np.max(np.abs(G1 - Go)) <= 1e-11 * np.max(np.abs(Go))


def test_row_masks_fma_counts(built):
    """The masked FP64 products count the FMAs they execute (option
    count_fmas): with a direction of no zeros they run every term of F's
    32-row tiles (forward; each tile spans the union of its 32 rows' bands,
    zero-filled) and of F^T's (transposed): a little over nnz * N each; with
    Pi-like zeros (7 groups of 32 columns, two of them empty) fewer, and the
    Hessian product is the same bits."""
    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    inst = synth.make_instance(M=300, N=200, D=600, xmax=250.0, eta=0.8, shots=10**6, gamma=1e-4, eps=1e-6, seed=8)
    nnz_n = int(inst.nnz) * inst.N
    # F^T's tiles: rows i of 32 b .. 32 b + 31, d over the union of their columns' ranges
    rows = np.flatnonzero(inst.band_lo >= 0)
    clo = np.full(inst.M, inst.D)
    chi = np.zeros(inst.M, dtype=np.int64)
    for d in rows:
        a, b = inst.band_lo[d], inst.band_hi[d] + 1
        clo[a:b] = np.minimum(clo[a:b], d)
        chi[a:b] = np.maximum(chi[a:b], d + 1)
    tile_terms = 0
    for b0 in range(0, inst.M, 32):
        lo, hi = clo[b0 : b0 + 32], chi[b0 : b0 + 32]
        if (hi > lo).any():
            tile_terms += (hi[hi > lo].max() - lo[hi > lo].min()) * min(32, inst.M - b0)
    tile_n = int(tile_terms) * inst.N
    # F's tiles: rows d of 32 b .. 32 b + 31 (every row a lane), i over the union of their bands
    ftile_terms = 0
    for b0 in range(0, inst.D, 32):
        lo, hi = inst.band_lo[b0 : b0 + 32], inst.band_hi[b0 : b0 + 32] + 1
        ok = lo >= 0
        if ok.any():
            ftile_terms += (hi[ok].max() - lo[ok].min()) * min(32, inst.D - b0)
    ftile_n = int(ftile_terms) * inst.N
    assert tile_n >= nnz_n and ftile_n >= nnz_n
    rng = np.random.default_rng(4)
    dense = np.asfortranarray(rng.standard_normal((inst.M, inst.N)) + 3.0)  # no zeros
    sparse = _sparse_x(inst, 6)
    with pq.Solver(0) as s:
        s.set_instance(inst, pq.FP64)
        s.set_option("count_fmas", 1)
        counts = []
        for V in (dense, sparse):
            f0, t0 = s.get_option("fmas.forward"), s.get_option("fmas.transposed")
            H = s.BF(V)
            counts.append((s.get_option("fmas.forward") - f0, s.get_option("fmas.transposed") - t0))
        s.set_option("row_masks", 0)
        H0 = s.BF(sparse)
    assert counts[0] == (ftile_n, tile_n), (counts, nnz_n, ftile_n, tile_n)
    assert 0 < counts[1][0] < ftile_n and 0 < counts[1][1] < tile_n, counts
    assert np.array_equal(H, H0)


def _chain_cases(M, N, seed):
    """Arrays whose pdot chains meet every branch of the warp-parallel exact
    chain: products that tie at the accumulator's grid (3 * (2^52 + 1)
    scaled), partial sums crossing binades up and down and cancelling to
    exactly zero, signed zeros, underflowing products and huge terms."""
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((M, N)) * 2.0 ** rng.integers(-40, 40, (M, N))
    B = rng.standard_normal((M, N))
    k = rng.random((M, N))
    t = k < 0.08  # ties
    A[t] = 3.0 * 2.0 ** rng.integers(-20, 20, t.sum())
    B[t] = float((1 << 52) + 1)
    z = (k >= 0.08) & (k < 0.16)  # signed zeros
    A[z] = rng.choice([0.0, -0.0], z.sum())
    u = (k >= 0.16) & (k < 0.2)  # products that underflow
    A[u] = 1e-200
    B[u] = -1e-200
    c = (k >= 0.2) & (k < 0.26)  # cancel the column so far
    A[c] = 1.0
    B[c] = 0.0
    h = (k >= 0.26) & (k < 0.27)  # huge terms (no overflow: a few per column)
    A[h] = 1e300
    B[h] = rng.choice([1.0, -1.0], h.sum())
    for n in range(N):
        for i in np.flatnonzero(c[:, n]):
            B[i, n] = -float(np.sum(A[:i, n] * B[:i, n]))  # roughly cancels: the chain passes near 0
    return np.asfortranarray(A), np.asfortranarray(B)


@pytest.mark.parametrize("which", ["cfg1", "small"])
def test_pdot_exact_chains(built, request, which):
    """pdot through the warp-parallel exact chains (k_colchain) equals the
    oracle's sequential pdot bit for bit, on ordinary arrays, on arrays made
    to hit every fallback branch, and on a = b."""
    inst = request.getfixturevalue(which)
    s, o = _pair(inst)
    rng = np.random.default_rng(21)
    cases = [(_random_x(inst, 22), _random_x(inst, 23)),
             (np.asfortranarray(rng.standard_normal((inst.M, inst.N))),) * 2]
    for seed in range(4):
        cases.append(_chain_cases(inst.M, inst.N, 30 + seed))
    # steps whose exact sum falls just below a power of two (the correctly
    # rounded sum is on the finer grid below it), one column each
    ulp = 2.0 ** -52
    A = np.zeros((inst.M, inst.N))
    for n in range(inst.N):
        k = 1 + n % 4
        A[0, n] = (1.0 + k * ulp) * 2.0 ** (n % 7 - 3)
        A[1, n] = -(k + 0.2 + 0.1 * (n % 3)) * ulp * 2.0 ** (n % 7 - 3)
        A[2:, n] = np.random.default_rng(n).uniform(0, 1e-30, inst.M - 2)
    cases.append((np.asfortranarray(A), np.asfortranarray(np.ones((inst.M, inst.N)))))
    for A, B in cases:
        g, r = s.pdot(A, B), o.pdot(A, B)
        assert np.float64(g).tobytes() == np.float64(r).tobytes(), (g, r)
