"""Host-side entry points that need no GPU: the restart state's smoothing
(pqdts_cuda_smooth, pqdts.f90:1877-1902) against a loop restatement of the
reference, and the in-process run_pqdts's interface against the reference
wrapper's (pqdts.py:30)."""
import ast
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _smooth_restated(X, smo_fact):
    """pqdts.f90:1877-1902, loop for loop (1-based j, k as there)."""
    M, N = X.shape
    Y = X.copy()
    for j in range(1, M + 1):
        dist = math.floor(j / smo_fact + 0.5)  # anint of a positive value
        if j <= 100:
            continue
        for i in range(N):
            s, c = 0.0, 0
            for k in range(max(1, j - dist), min(j + dist, M) + 1):
                s = s + X[k - 1, i]
                c += 1
            Y[j - 1, i] = s / c
        rs = 0.0
        for i in range(N):
            rs += Y[j - 1, i]
        for i in range(N):
            Y[j - 1, i] = Y[j - 1, i] / rs
    return Y


@pytest.mark.parametrize("smo_fact", [7.0, 2.5, 1000.0])
def test_smooth_matches_restatement(built, smo_fact):
    import pqdts_gb300 as pq

    rng = np.random.default_rng(5)
    X = rng.random((260, 5))
    X /= X.sum(axis=1, keepdims=True)
    assert np.array_equal(pq.smooth(X, smo_fact), _smooth_restated(X, smo_fact))


def test_smooth_rejects_bad_arguments(built):
    import pqdts_gb300 as pq

    with pytest.raises(pq.PqdtsError):
        pq.smooth(np.ones((120, 3)), 0.0)


def test_run_pqdts_interface_matches_wrapper():
    """Same parameter names, order and defaults as the wrapper's run_pqdts
    (read from the reference tree where present), then precision / device."""
    import inspect

    sys.path.insert(0, ROOT)
    import pqdts_gb300 as pq
    from oracle import build as obuild

    path = os.path.join(obuild.REFERENCE_TREE, "pqdts.py")
    if not os.path.exists(path):
        pytest.skip("reference wrapper not present")
    fn = next(n for n in ast.walk(ast.parse(open(path).read()))
              if isinstance(n, ast.FunctionDef) and n.name == "run_pqdts")
    names = [a.arg for a in fn.args.args]
    defaults = [ast.literal_eval(d) for d in fn.args.defaults]
    ref = dict(zip(names[len(names) - len(defaults):], defaults))
    ours = inspect.signature(pq.run_pqdts).parameters
    assert list(ours)[: len(names)] == names
    for k, v in ref.items():
        assert ours[k].default == v, k
    assert list(ours)[len(names):] == ["precision", "device"]


def test_run_pqdts_dry_run_needs_no_gpu():
    import scipy.sparse as sps

    import pqdts_gb300 as pq

    P = sps.csr_matrix(np.full((6, 3), 1.0 / 3))
    assert pq.run_pqdts(3, 4, 6, P, F=sps.csr_matrix(np.ones((6, 4))), dry=True) is None
    with pytest.raises(ValueError):
        pq.run_pqdts(3, 4, 6, P, F=sps.csr_matrix(np.ones((5, 4))), dry=True)


def test_batch_groups_host_only(built):
    """The batch's lockstep grouping is a host computation: instances with
    identical F (and N <= 4096) share a group, others are alone."""
    import dataclasses

    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    insts = synth.make_batch(n_base=2, n_resample=3, shots=10**6, seed=4, m_range=(60, 150), n_range=(33, 60))
    assert list(pq.batch_groups(insts)) == [0, 0, 0, 1, 1, 1]
    # one changed F value splits that instance off
    v = insts[1].band_val.copy()
    v[5] *= 1.0 + 1e-15
    changed = insts[:3] + [dataclasses.replace(insts[1], band_val=v)]
    assert list(pq.batch_groups(changed)) == [0, 0, 0, -1]
    # small N groups too; N above 4096 is solved alone
    small = synth.make_batch(n_base=1, n_resample=3, shots=10**6, seed=4, m_range=(40, 90), n_range=(5, 12))
    assert list(pq.batch_groups(small)) == [0, 0, 0]
    wide = [dataclasses.replace(i, N=5000, P=np.zeros((i.D, 5000))) for i in small]
    assert list(pq.batch_groups(wide)) == [-1, -1, -1]
