"""Tensor-core (tcgen05 + TMA, split-BF16x3) Hessian products of the mixed
solver against the FP64 oracle's BF (pqdts.f90:246-342).

Split-BF16x3 keeps ~16 significant bits per operand (hi + lo) and drops the
lo.lo term, with FP32 accumulation: relative to the product's scale the
error stays below 1e-4 (measured well below it); the FP32 CUDA-core path is
held to 2e-5 in test_gpu_ops.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TC_REL = 1e-4


def _tc_solver(inst, persistent=-1, splits1=-1):
    import pqdts_gb300 as pq

    s = pq.Solver(0)
    s.set_option("tensor_cores", 1)
    s.set_option("tc_persistent", persistent)
    s.set_option("tc_splits1", splits1)
    s.set_instance(inst, pq.MIXED)
    assert s.get_option("sched.tc") == 1
    if persistent >= 0:
        assert s.get_option("sched.tc_persistent") == persistent
    if splits1 > 0:
        assert s.get_option("sched.tc_splits1") == splits1
    return s


def _instances():
    from pqdts_gb300 import synth

    return {
        # one 128-row block, N below one MMA tile of 16
        "tiny": synth.make_instance(M=60, N=12, D=100, xmax=40.0, eta=0.85, shots=10**5, gamma=1e-3, eps=1e-6, seed=3),
        "cfg1": synth.make_config(1, seed=0),
        # several row blocks and N tiles (N = 300 -> 2 tiles of 160), ragged edges
        "medium": synth.make_instance(M=700, N=300, D=1300, xmax=620.0, eta=0.8, shots=10**6, gamma=1e-5, eps=1e-6,
                                      seed=5),
        # every entry kept: the dense-F variant
        "dense": synth.make_instance(M=300, N=40, D=300, xmax=250.0, eta=0.85, shots=10**6, gamma=1e-4, eps=1e-6,
                                     seed=6, dense=True),
        # probe rows whose window lies beyond M (rows 117.. empty: whole
        # 128-row blocks without a band), gamma = 0, N = 10
        "empty_rows": synth.make_instance(M=60, N=10, D=400, xmax=500.0, eta=0.85, shots=10**5, gamma=0.0, eps=1e-6,
                                          seed=9),
    }


@pytest.fixture(scope="module")
def tc_insts():
    return _instances()


@pytest.mark.parametrize("which", ["tiny", "cfg1", "medium", "dense", "empty_rows"])
@pytest.mark.parametrize("full", [True, False])
@pytest.mark.parametrize("persistent", [0, 1])
def test_tc_hessian_product_matches_fp64(built, tc_insts, which, full, persistent):
    """Both kernels: one CTA per output tile, and the persistent
    warp-specialized one with double-buffered accumulators."""
    from oracle.oracle import Oracle

    inst = tc_insts[which]
    s = _tc_solver(inst, persistent)
    o = Oracle.from_instance(inst)
    rng = np.random.default_rng(11)
    X = rng.random((inst.M, inst.N))
    X = np.asfortranarray(X / X.sum(1, keepdims=True))
    m = None if full else np.argmax(X, axis=1).astype(np.int32)
    s.set_space(full, m)
    o.set_space(full, m)
    V = np.asfortranarray(rng.standard_normal((inst.M, inst.N)))
    H = s.BF32(V)
    H64 = o.BF(V)
    err = np.max(np.abs(H - H64)) / np.max(np.abs(H64))
    assert err < TC_REL, err
    s.close()


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("screen", [0, 1])
def test_tc_mixed_solve_reaches_fp64_objective(built, tc_insts, persistent, screen):
    """The mixed solve with tensor-core CG products ends within 1e-8 of the
    FP64 solve's objective (conv < 1e-9 pins it), feasible -- with the line
    search's probe products F.dX on the tensor cores (screen = 1: one
    split-BF16x3 product over all probes' columns) or on the CUDA cores."""
    import pqdts_gb300 as pq

    inst = tc_insts["cfg1"]
    with pq.Solver(0) as s64:
        s64.set_instance(inst, pq.FP64)
        st64 = s64.solve(mode=2, maxiter=2000, eps=1e-9)
    s = _tc_solver(inst, persistent)
    s.set_option("tc_screen", screen)
    assert s.get_option("sched.tc_screen") == screen
    st = s.solve(mode=2, maxiter=2000, eps=1e-9)
    X = s.get_x()
    s.close()
    assert abs(st["L"] - st64["L"]) <= 1e-8 * abs(st64["L"]), (st, st64)
    assert X.min() >= 0.0 and np.max(np.abs(X.sum(1) - 1.0)) <= 1e-12


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("which", ["tiny", "dense"])
def test_tc_split_forward_product(built, tc_insts, which, persistent):
    """F.V with its K range split (FP32 partials summed and split again by
    k_finish_t) gives the same Hessian product to the split-BF16x3 bound."""
    from oracle.oracle import Oracle

    inst = tc_insts[which]
    s = _tc_solver(inst, persistent, splits1=3)
    o = Oracle.from_instance(inst)
    rng = np.random.default_rng(12)
    V = np.asfortranarray(rng.standard_normal((inst.M, inst.N)))
    H = s.BF32(V)
    H64 = o.BF(V)
    s.close()
    err = np.max(np.abs(H - H64)) / np.max(np.abs(H64))
    assert err < TC_REL, err
