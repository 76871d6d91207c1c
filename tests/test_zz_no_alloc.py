"""pqdts_cuda_simplexproj_noalloc: the simplex projection for callers that
cannot allocate device memory (they pass their own device buffers; the
scratch is a static device array inside the library).  Checked through the
C ABI against the allocating entry point pqdts_cuda_simplexproj, with the
same bitwise tolerance as the other projection tests, on two calls in a row
(the shared scratch keeps the previous call's contents).  Collected last so
that a run stopping at the first failure has already run everything else."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reference_projection(Y):
    import pqdts_gb300 as pq

    with pq.Solver(0) as s:
        return s.simplexproj(Y)


def _noalloc(Y, out_alias=False):
    import torch

    import pqdts_gb300 as pq

    rows, length = Y.shape
    d_y = torch.from_numpy(np.ascontiguousarray(Y)).to("cuda:0")
    d_x = d_y if out_alias else torch.empty_like(d_y)
    stream = torch.cuda.current_stream(0).cuda_stream
    rc = pq.lib().pqdts_cuda_simplexproj_noalloc(C.c_void_p(d_y.data_ptr()), C.c_void_p(d_x.data_ptr()), length, rows,
                                                 C.c_void_p(stream))
    torch.cuda.synchronize(0)
    assert rc == 0
    return d_x.cpu().numpy()


def test_noalloc_matches_allocating_entry_point(built):
    rng = np.random.default_rng(123)
    # two calls in a row with different shapes: the second must not see the
    # first call's scratch contents
    Y1 = rng.standard_normal((300, 200)) * 0.6 + 0.01
    Y2 = rng.standard_normal((1000, 37)) * 3.0
    for Y in (Y1, Y2):
        X = _noalloc(Y)
        assert np.array_equal(X, _reference_projection(Y))
        assert X.min() >= 0.0 and np.max(np.abs(X.sum(axis=1) - 1.0)) < 1e-12
    # in place (d_y == d_x), as the allocating entry point allows
    assert np.array_equal(_noalloc(Y1, out_alias=True), _reference_projection(Y1))


def test_noalloc_rejects_sizes_beyond_the_scratch(built):
    import torch

    import pqdts_gb300 as pq

    cap = 1 << 20
    d = torch.empty(16, dtype=torch.float64, device="cuda:0")
    p = C.c_void_p(d.data_ptr())
    # checked on the host before any launch: nothing touches the buffers
    assert pq.lib().pqdts_cuda_simplexproj_noalloc(p, p, cap + 1, 1, None) == -1
    assert pq.lib().pqdts_cuda_simplexproj_noalloc(p, p, 1024, cap // 1024 + 1, None) == -1
    assert pq.lib().pqdts_cuda_simplexproj_noalloc(p, p, 0, 1, None) == -1
