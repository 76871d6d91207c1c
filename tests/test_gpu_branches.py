"""Branches of the product path that the full-solve tests do not reach on
their own, each checked through the C ABI:

* simplexproj_condat_ -- the reference's own projection symbol with its
  exact signature (condat_simplexproj.c:60), bitwise against the oracle's
  Condat (itself bitwise against the reference's compiled file);
* the mixed path's warp-per-row projection (k_simplex, used by its stage-1
  doproj) against Condat's threshold;
* the FP64 refinement of a mixed solve (the FP64 CG in stage 2);
* the error path of the tensor-core kernels' bounded barrier waits: a wait
  that runs out before any copy or MMA is issued (a barrier that nothing
  arrives on) fails the call with PQDTS_E_CUDA and leaves the context usable;
* the benchmark workload's FP64 solve against the oracle's full solve.
"""
import ctypes as C
import os
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# warp-per-row projection vs Condat: both thresholds are (sum of the kept
# values - 1) / count, summed in different orders -> entries agree to a few
# ulps of the row's scale
SIMPLEX_ABS = 1e-13


def _condat_symbol():
    import pqdts_gb300 as pq

    f = pq.lib().simplexproj_condat_
    f.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int)]
    f.restype = None
    return f


def _call(f, y, x):
    n = C.c_int(y.size)
    f(y.ctypes.data_as(C.POINTER(C.c_double)), x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n))


def test_reference_condat_symbol(built):
    from oracle.oracle import condat

    f = _condat_symbol()
    rng = np.random.default_rng(21)
    for n in (1, 2, 3, 31, 32, 33, 200, 1000, 5000):
        y = rng.standard_normal(n) * rng.choice([1e-3, 1.0, 50.0])
        y0 = y.copy()
        x = np.full(n, 7.0)
        _call(f, y, x)
        assert np.array_equal(y, y0)  # input untouched
        assert np.array_equal(x, condat(y0)), n
        z = y0.copy()
        _call(f, z, z)  # x == y: still the projection
        assert np.array_equal(z, condat(y0))


def test_reference_condat_symbol_threads(built):
    """Concurrent host threads on private buffers, as the reference's OpenMP
    loop calls it (pqdts.f90:1130-1135): each thread's own stream/buffers."""
    from oracle.oracle import condat

    f = _condat_symbol()
    rng = np.random.default_rng(22)
    rows = [rng.standard_normal(int(n)) for n in rng.integers(5, 700, size=64)]
    out = [np.empty_like(r) for r in rows]

    def work(k0):
        for k in range(k0, len(rows), 4):
            _call(f, rows[k], out[k])

    th = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for r, x in zip(rows, out):
        assert np.array_equal(x, condat(r))


@pytest.mark.parametrize("which", ["cfg1", "small", "mid", "wide"])
def test_mixed_projection_matches_condat(built, request, which):
    """doproj on a mixed problem runs the warp-per-row projection (rows
    staged in shared memory, Michelot's iteration on a shrinking active
    list); wide: N = 1500 rows (47 entries per lane, 4 rows per block)."""
    import pqdts_gb300 as pq
    from oracle.oracle import condat
    from pqdts_gb300 import synth

    if which == "wide":
        inst = synth.make_instance(M=70, N=1500, D=140, xmax=60.0, eta=0.85, shots=10**5, gamma=1e-4, eps=1e-6,
                                   seed=1)
    else:
        inst = request.getfixturevalue(which)
    rng = np.random.default_rng(23)
    Y = np.asfortranarray(rng.standard_normal((inst.M, inst.N)) * 0.7 + 0.05)
    with pq.Solver(0) as s:
        s.set_instance(inst, pq.MIXED)
        s.set_x(Y)
        s.doproj()
        X = s.get_x()
    Xo = np.stack([condat(np.ascontiguousarray(y)) for y in Y])
    scale = np.maximum(1.0, np.max(np.abs(Y), axis=1))
    assert np.all(np.max(np.abs(X - Xo), axis=1) <= SIMPLEX_ABS * scale)
    assert X.min() >= 0.0
    assert np.max(np.abs(X.sum(axis=1) - 1.0)) <= 1e-12


def test_fp64_refinement_of_mixed_solve(built, small):
    """fp64_refine = 1: every stage-2 CG of the mixed solve in FP64; the
    solve still ends within 1e-8 of the FP64 objective (conv < 1e-9 pins it)
    with Pi >= 0 exactly."""
    import pqdts_gb300 as pq

    with pq.Solver(0) as s64:
        s64.set_instance(small, pq.FP64)
        st64 = s64.solve(mode=2, maxiter=2000, eps=1e-9)
    with pq.Solver(0) as s:
        s.set_option("fp64_refine", 1)
        assert s.get_option("fp64_refine") == 1
        s.set_instance(small, pq.MIXED)
        st = s.solve(mode=2, maxiter=2000, eps=1e-9)
        X = s.get_x()
    assert st["refine"] > 0
    assert abs(st["L"] - st64["L"]) <= 1e-8 * abs(st64["L"]), (st, st64)
    assert X.min() >= 0.0 and np.max(np.abs(X.sum(axis=1) - 1.0)) <= 1e-12


@pytest.mark.parametrize("persistent", [0, 1])
def test_tc_barrier_timeout_is_an_error(built, small, persistent):
    """A bounded barrier wait that runs out (5 ms, on a barrier nothing
    arrives on, before any copy or MMA) fails BF32 with PQDTS_E_CUDA; with the
    probe off the same context computes the product and solves."""
    import pqdts_gb300 as pq
    from oracle.oracle import Oracle

    V = np.asfortranarray(np.random.default_rng(24).standard_normal((small.M, small.N)))
    with pq.Solver(0) as s:
        s.set_option("tensor_cores", 1)
        s.set_option("tc_persistent", persistent)
        s.set_instance(small, pq.MIXED)
        assert s.get_option("sched.tc") == 1
        s.set_space(True, None)
        s.set_option("tc_wait_ms", 5)
        s.set_option("tc_wait_probe", 1)
        with pytest.raises(pq.PqdtsError, match=r"\(-2\).*barrier wait timed out"):
            s.BF32(V)
        s.set_option("tc_wait_probe", 0)
        s.set_option("tc_wait_ms", 2000)
        H = s.BF32(V)
        st = s.solve(mode=2, maxiter=200, eps=small.eps)
        X = s.get_x()
    o = Oracle.from_instance(small)
    o.set_space(True, None)
    H64 = o.BF(V)
    assert np.max(np.abs(H - H64)) <= 1e-4 * np.max(np.abs(H64))
    assert np.isfinite(st["L"]) and X.min() >= 0.0 and np.max(np.abs(X.sum(axis=1) - 1.0)) <= 1e-12


def test_fp64_config2_matches_oracle(built):
    """The benchmark workload (M=2000, N=200, D=4000, seed 0) at the
    reference's stopping rule conv < 1e-6: the GPU's FP64 solve is the
    oracle's full solve bit for bit (objective, iteration counts, Pi)."""
    from oracle.oracle import Oracle, set_threads
    from pqdts_gb300 import synth

    import pqdts_gb300 as pq

    inst = synth.make_config(2, seed=0)
    with pq.Solver(0) as s:
        s.set_instance(inst, pq.FP64)
        st = s.solve(mode=2, maxiter=2000, eps=inst.eps)
        X = s.get_x()
    set_threads(len(os.sched_getaffinity(0)))
    Xo, so = Oracle.from_instance(inst).solve(mode=2, maxiter=2000, eps=inst.eps)
    assert st["L"] == so["L"], (st, so)
    assert st["outer"] == so["outer"] and st["cg"] == so["cg"]
    assert np.array_equal(X, Xo)
    assert X.min() >= -1e-12 and np.max(np.abs(X.sum(axis=1) - 1.0)) <= 1e-12
