"""Full-solve parity: the FP64 GPU solve against the oracle's solve on the same
seeded inputs.  Tolerances are the drop-in requirement: final objective within
1e-10 relative, Pi within 1e-8 max-abs, rows on the simplex (sums 1 within
1e-12, entries >= 0).  The mixed-precision solve must reach an objective
within 1e-8 relative of the FP64 solve with the same feasibility.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OBJ_REL = 1e-10
PI_ABS = 1e-8
MIXED_OBJ_REL = 1e-8


def _feasible(X):
    assert X.min() >= -1e-12, X.min()
    assert np.max(np.abs(X.sum(axis=1) - 1.0)) <= 1e-12


def _solve_gpu(inst, precision=0, mode=2, maxiter=200, eps=None):
    import pqdts_gb300 as pq

    with pq.Solver(0) as s:
        s.set_instance(inst, precision)
        st = s.solve(mode=mode, maxiter=maxiter, eps=inst.eps if eps is None else eps)
        return s.get_x(), st, s.kernel_launches()


@pytest.mark.parametrize("which", ["cfg1", "small"])
def test_fp64_solve_matches_oracle(built, request, which):
    from oracle.oracle import Oracle

    inst = request.getfixturevalue(which)
    X, st, launches = _solve_gpu(inst)
    Xo, so = Oracle.from_instance(inst).solve(mode=2, maxiter=200, eps=inst.eps)
    assert launches > 0
    assert abs(st["L"] - so["L"]) <= OBJ_REL * abs(so["L"]), (st, so)
    assert np.max(np.abs(X - Xo)) <= PI_ABS
    _feasible(X)
    assert st["conv"] < inst.eps


def test_mode1_matches_oracle(built, small):
    from oracle.oracle import Oracle

    X, st, _ = _solve_gpu(small, mode=1, maxiter=40)
    Xo, so = Oracle.from_instance(small).solve(mode=1, maxiter=40, eps=small.eps)
    assert abs(st["L"] - so["L"]) <= OBJ_REL * abs(so["L"])
    assert np.max(np.abs(X - Xo)) <= PI_ABS
    _feasible(X)


@pytest.mark.parametrize("which", ["cfg1", "small"])
def test_mixed_precision_solve(built, request, which):
    inst = request.getfixturevalue(which)
    X64, s64, _ = _solve_gpu(inst, 0)
    X32, s32, _ = _solve_gpu(inst, 1)
    assert abs(s32["L"] - s64["L"]) <= MIXED_OBJ_REL * abs(s64["L"]), (s32, s64)
    _feasible(X32)
    assert s32["conv"] < inst.eps


def test_start_stage2_and_restart(built, small):
    """start_stage = 2 from a given point (the restart path) matches the oracle."""
    import pqdts_gb300 as pq
    from oracle.oracle import Oracle

    rng = np.random.default_rng(1)
    X0 = rng.random((small.M, small.N))
    X0 = np.asfortranarray(X0 / X0.sum(1, keepdims=True))
    with pq.Solver(0) as s:
        s.set_instance(small)
        s.set_x(X0)
        st = s.solve(mode=2, maxiter=100, eps=small.eps, start_stage=2)
        X = s.get_x()
    Xo, so = Oracle.from_instance(small).solve(X0, mode=2, maxiter=100, eps=small.eps, start_stage=2)
    assert abs(st["L"] - so["L"]) <= OBJ_REL * abs(so["L"])
    assert np.max(np.abs(X - Xo)) <= PI_ABS


def test_batch_matches_single(built):
    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    insts = synth.make_batch(n_base=2, n_resample=3, shots=10**6, seed=4, m_range=(40, 90), n_range=(5, 12))
    Xs, stats = pq.solve_batch(insts, maxiter=100)
    for inst, X, st in zip(insts, Xs, stats):
        Xs1, s1, _ = _solve_gpu(inst, maxiter=100)
        assert abs(st["L"] - s1["L"]) <= 1e-13 * abs(s1["L"])
        assert np.array_equal(X, Xs1)
