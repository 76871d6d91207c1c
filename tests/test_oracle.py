"""CPU checks of the oracle itself (no GPU).

* The Condat restatement is bit-identical to the reference's own
  condat_simplexproj.c (compiled from the reference tree into oracle/_ref
  where that tree exists; the test skips elsewhere).
* The derivative identities of the reference's self test (pqdts.f90:1737-1831)
  hold for L/dL/BF/Bdiag in the full and the reduced space.
* The oracle is deterministic across OpenMP thread counts.
"""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libcondat_ref.so")


def _ref_condat():
    if not os.path.exists(REF_SO):
        pytest.skip("reference condat_simplexproj.c not built here (reference tree absent)")
    L = C.CDLL(REF_SO)
    L.simplexproj_condat_.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
    L.simplexproj_condat_.restype = None

    def f(y):
        y = np.ascontiguousarray(y, np.float64)
        x = np.empty_like(y)
        n = C.c_int(y.size)
        L.simplexproj_condat_(y.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p), C.byref(n))
        return x

    return f


def test_condat_bitexact_vs_reference(built):
    from oracle.oracle import condat

    ref = _ref_condat()
    rng = np.random.default_rng(0)
    cases = [np.array([0.5]), np.array([1.0, 1.0]), np.zeros(7), np.full(9, 1 / 9), np.array([5.0, -3.0, 2.0])]
    for n in (2, 3, 5, 20, 64, 200, 1000, 5000):
        for scale in (1e-3, 0.1, 1.0, 30.0):
            cases.append(rng.standard_normal(n) * scale)
            cases.append(rng.random(n) * scale)
            y = rng.random(n)
            cases.append(y / y.sum())  # already feasible
    # rows like the solver's line-search points: a feasible row plus a step
    for _ in range(50):
        n = int(rng.integers(2, 300))
        y = rng.random(n)
        y /= y.sum()
        cases.append(y + 0.3 * rng.standard_normal(n) * y)
    for y in cases:
        a, b = condat(y), ref(y)
        assert np.array_equal(a, b), (y.size, np.max(np.abs(a - b)))


def _fd_setup(full, seed=0):
    from oracle.oracle import Oracle
    from pqdts_gb300 import synth

    inst = synth.make_instance(M=30, N=6, D=60, xmax=25.0, eta=0.8, shots=10**5, gamma=3e-3, eps=1e-6, seed=seed)
    o = Oracle.from_instance(inst)
    rng = np.random.default_rng(seed)
    X = rng.random((inst.M, inst.N))
    X = np.asfortranarray(X / X.sum(1, keepdims=True))
    maxr = np.argmax(X, axis=1).astype(np.int32)
    o.set_space(full, None if full else maxr)
    if not full:
        # the reference rebuilds the max column before testing (1747-1753)
        X = o.L(X)[1]
    return inst, o, X, maxr


@pytest.mark.parametrize("full", [True, False])
def test_derivative_identities(built, full):
    """pqdts.f90:1759-1828: dL vs central differences of L, BF vs the
    gradient difference, Bdiag vs BF(e_ij) at the corner indices."""
    inst, o, X, maxr = _fd_setup(full)
    M, N = inst.M, inst.N
    G, Xr = o.dL(X)
    dxp = 1e-7
    idx = [(i % M, j % N) for i in (-3, -2, -1, 0, 1, 2) for j in (-3, -2, -1, 0, 1, 2)]
    for i, j in idx:
        if not full and j == maxr[i]:
            continue  # the max column is implicit in the reduced space
        Xp = Xr.copy(order="F")
        Xp[i, j] += dxp
        Xm = Xr.copy(order="F")
        Xm[i, j] -= dxp
        fd = (o.L(Xp)[0] - o.L(Xm)[0]) / (2 * dxp)
        assert abs(fd - G[i, j]) <= 1e-6 * max(1.0, abs(G[i, j])), (i, j, fd, G[i, j])
    rng = np.random.default_rng(3)
    S = np.asfortranarray(rng.random((M, N)))
    if not full:
        S[np.arange(M), maxr] = 0.0
    B = o.BF(S)
    G0, _ = o.dL(Xr)
    G1, _ = o.dL(np.asfortranarray(Xr + dxp * S))
    fdh = (G1 - G0) / dxp
    for i, j in idx:
        assert abs(fdh[i, j] - B[i, j]) <= 1e-5 * max(1.0, abs(B[i, j])), (i, j)
    BD = o.Bdiag()
    for i, j in idx:
        if not full and j == maxr[i]:
            continue
        E = np.zeros((M, N), order="F")
        E[i, j] = 1.0
        h = o.BF(E)
        # exact in the full space; in the reduced space Bdiag is the
        # reference's approximation 2x the full-space diagonal
        if full:
            assert abs(h[i, j] - BD[i, j]) <= 1e-12 * abs(BD[i, j])
        else:
            assert h[i, j] <= BD[i, j] + 1e-12 * abs(BD[i, j])


def test_thread_count_determinism(built):
    from oracle import oracle as om
    from pqdts_gb300 import synth

    inst = synth.make_instance(M=50, N=7, D=100, xmax=40.0, eta=0.9, shots=10**5, gamma=1e-4, eps=1e-6, seed=2)
    out = []
    for t in (1, 3):
        om.set_threads(t)
        X, st = om.Oracle.from_instance(inst).solve(mode=2, maxiter=50, eps=1e-6)
        out.append((X, st["L"]))
    om.set_threads(os.cpu_count() or 1)
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


def test_oracle_solution_feasible_and_converged(built, cfg1):
    from oracle.oracle import Oracle

    X, st = Oracle.from_instance(cfg1).solve(mode=2, maxiter=200, eps=cfg1.eps)
    assert st["conv"] < cfg1.eps
    assert X.min() >= -1e-12 and np.max(np.abs(X.sum(1) - 1)) <= 1e-12
