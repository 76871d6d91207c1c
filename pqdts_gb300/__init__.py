"""pqdts_gb300: GB300 (sm_103a) drop-in for pqdts's two-metric projected
truncated Newton solve.

The compute path is libpqdts_cuda.so (hand-written CUDA, built in place by
pqdts_gb300/build.py) behind the C ABI in include/pqdts_cuda.h.  This module
is a thin ctypes binding of that ABI with the reference's operation names
(L, dL, BF, Bdiag, doproj, doproj2, conv_test; pqdts.f90:208-1164) and its
solve (program pqdts, 1908-2167).  There is no CPU fallback: every entry
raises if the library cannot be loaded or a CUDA call fails.

Array conventions are the reference's: X-shaped arrays are (M, N) (held in
Fortran order on the way in and out), P is (D, N) row-major, i.e. the
reference's P(N, D).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpqdts_cuda.so")
CLI_PATH = os.path.join(HERE, "pqdts_cuda.x")

FP64, MIXED = 0, 1
STAT_KEYS = ["L", "conv", "norm_der", "outer", "cg", "ls_evals", "refine", "seconds"]

_lib = None


class PqdtsError(RuntimeError):
    pass


def lib():
    """Load libpqdts_cuda.so (building it first if absent); raise if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build

        _build.build()
    L = C.CDLL(LIB_PATH)
    p, i64, i32, d = C.c_void_p, C.c_int64, C.c_int32, C.c_double
    sig = {
        "pqdts_cuda_create": [i32, C.POINTER(C.c_void_p)],
        "pqdts_cuda_destroy": [p],
        "pqdts_cuda_last_error": [p, C.c_char_p, i64],
        "pqdts_cuda_kernel_launches": [p, C.POINTER(i64)],
        "pqdts_cuda_set_verbose": [p, i32],
        "pqdts_cuda_set_problem": [p, i64, i64, i64, p, p, p, p, d, i32],
        "pqdts_cuda_set_problem_coo": [p, i64, i64, i64, i64, p, p, p, i64, p, p, p, d, i32],
        "pqdts_cuda_get_bands": [p, p, p, C.POINTER(i64)],
        "pqdts_cuda_set_x": [p, p],
        "pqdts_cuda_init_x": [p],
        "pqdts_cuda_get_stream": [p, C.POINTER(C.c_void_p)],
        "pqdts_cuda_transfer_bytes": [p, C.POINTER(i64), C.POINTER(i64)],
        "pqdts_cuda_get_x": [p, p],
        "pqdts_cuda_set_space": [p, i32, p],
        "pqdts_cuda_get_maxr": [p, p],
        "pqdts_cuda_L": [p, C.POINTER(d)],
        "pqdts_cuda_dL": [p, p],
        "pqdts_cuda_redO": [p, p],
        "pqdts_cuda_BF": [p, p, p],
        "pqdts_cuda_BF32": [p, p, p],
        "pqdts_cuda_Bdiag": [p, p],
        "pqdts_cuda_pdot": [p, p, p, C.POINTER(d)],
        "pqdts_cuda_doproj": [p],
        "pqdts_cuda_doproj2": [p, C.POINTER(d)],
        "pqdts_cuda_conv_test": [p, C.POINTER(d)],
        "pqdts_cuda_simplexproj": [p, p, p, i64, i64],
        "pqdts_cuda_simplexproj_noalloc": [p, p, i64, i64, p],
        "pqdts_cuda_run_stage": [p, i32, i32, i32, d, i32, p],
        "pqdts_cuda_solve": [p, i32, i32, d, i32, i32, p, p, p],
        "pqdts_cuda_timer": [p, C.c_char_p, C.POINTER(d), C.POINTER(i64)],
        "pqdts_cuda_set_objective_target": [p, d],
        "pqdts_cuda_set_option": [p, C.c_char_p, i64],
        "pqdts_cuda_get_option": [p, C.c_char_p, C.POINTER(i64)],
        "pqdts_cuda_solve_batch": [i32, i32, p, p, p, p, p, p, p, p, p, p, p, i32, i32, i32, d, p, p, p],
        "pqdts_cuda_smooth": [i64, i64, d, p],
        "pqdts_cuda_batch_groups": [i32, p, p, p, p, p, p, p, p, p],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Solver:
    """One problem on one GPU (a pqdts_ctx)."""

    def __init__(self, device: int = 0, verbose: bool = False):
        self._L = lib()
        h = C.c_void_p()
        rc = self._L.pqdts_cuda_create(int(device), C.byref(h))
        if rc != 0:
            raise PqdtsError(f"pqdts_cuda_create failed ({rc}): no usable CUDA device {device}")
        self.h = h
        self.M = self.N = self.D = 0
        if verbose:
            self._L.pqdts_cuda_set_verbose(self.h, 1)

    def close(self):
        if getattr(self, "h", None):
            self._L.pqdts_cuda_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            buf = C.create_string_buffer(2048)
            self._L.pqdts_cuda_last_error(self.h, buf, 2048)
            raise PqdtsError(f"{what} failed ({rc}): {buf.value.decode(errors='replace')}")

    # -- problem ------------------------------------------------------------
    def set_problem(self, M, N, D, band_lo, band_hi, band_vals, P, gamma, precision=FP64):
        lo = np.ascontiguousarray(band_lo, np.int64)
        hi = np.ascontiguousarray(band_hi, np.int64)
        v = np.ascontiguousarray(band_vals, np.float64)
        Pd = np.ascontiguousarray(P, np.float64)
        assert lo.size == D and hi.size == D and Pd.size == D * N
        self._check(self._L.pqdts_cuda_set_problem(self.h, M, N, D, _ptr(lo), _ptr(hi), _ptr(v), _ptr(Pd),
                                                   float(gamma), int(precision)), "set_problem")
        self.M, self.N, self.D = int(M), int(N), int(D)

    def set_problem_coo(self, M, N, D, F_coo, P_coo, gamma, precision=FP64):
        """F_coo / P_coo = (row, col, val) triplets as in data/*_{row,col,data}.bin;
        F_coo None = internal F (needs M == (D-1)^2); P_coo None = random P."""
        if F_coo is None:
            fr = fc = fv = None
            nf = -1
        else:
            fr, fc, fv = (np.ascontiguousarray(F_coo[0], np.int32), np.ascontiguousarray(F_coo[1], np.int32),
                          np.ascontiguousarray(F_coo[2], np.float64))
            nf = fv.size
        if P_coo is None:
            pr = pc = pv = None
            npp = -1
        else:
            pr, pc, pv = (np.ascontiguousarray(P_coo[0], np.int32), np.ascontiguousarray(P_coo[1], np.int32),
                          np.ascontiguousarray(P_coo[2], np.float64))
            npp = pv.size
        self._check(self._L.pqdts_cuda_set_problem_coo(self.h, M, N, D, nf, _ptr(fr), _ptr(fc), _ptr(fv), npp,
                                                       _ptr(pr), _ptr(pc), _ptr(pv), float(gamma), int(precision)),
                    "set_problem_coo")
        self.M, self.N, self.D = int(M), int(N), int(D)

    def set_instance(self, inst, precision=FP64):
        self.set_problem(inst.M, inst.N, inst.D, inst.band_lo, inst.band_hi, inst.band_val, inst.P, inst.gamma,
                         precision)

    def bands(self):
        lo = np.empty(self.D, np.int64)
        hi = np.empty(self.D, np.int64)
        nnz = C.c_int64()
        self._check(self._L.pqdts_cuda_get_bands(self.h, _ptr(lo), _ptr(hi), C.byref(nnz)), "get_bands")
        return lo, hi, nnz.value

    # -- iterate --------------------------------------------------------------
    def set_x(self, X):
        X = np.asfortranarray(X, np.float64)
        assert X.shape == (self.M, self.N)
        self._check(self._L.pqdts_cuda_set_x(self.h, _ptr(X)), "set_x")

    def init_x(self):
        """X = 1/N on the device (the reference's starting point)."""
        self._check(self._L.pqdts_cuda_init_x(self.h), "init_x")

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        v = C.c_void_p()
        self._check(self._L.pqdts_cuda_get_stream(self.h, C.byref(v)), "get_stream")
        return v.value or 0

    def transfer_bytes(self):
        a, b = C.c_int64(), C.c_int64()
        self._check(self._L.pqdts_cuda_transfer_bytes(self.h, C.byref(a), C.byref(b)), "transfer_bytes")
        return a.value, b.value

    def get_x(self):
        X = np.empty((self.M, self.N), order="F")
        self._check(self._L.pqdts_cuda_get_x(self.h, _ptr(X)), "get_x")
        return X

    def set_space(self, fullspace, maxr=None):
        m = None if maxr is None else np.ascontiguousarray(maxr, np.int32)
        self._check(self._L.pqdts_cuda_set_space(self.h, 1 if fullspace else 0, _ptr(m)), "set_space")

    def maxr(self):
        m = np.empty(self.M, np.int32)
        self._check(self._L.pqdts_cuda_get_maxr(self.h, _ptr(m)), "get_maxr")
        return m

    # -- the reference's operations ------------------------------------------
    def L(self):
        v = C.c_double()
        self._check(self._L.pqdts_cuda_L(self.h, C.byref(v)), "L")
        return v.value

    def dL(self):
        G = np.empty((self.M, self.N), order="F")
        self._check(self._L.pqdts_cuda_dL(self.h, _ptr(G)), "dL")
        return G

    def redO(self):
        O = np.empty((self.D, self.N))
        self._check(self._L.pqdts_cuda_redO(self.h, _ptr(O)), "redO")
        return O

    def BF(self, V):
        V = np.asfortranarray(V, np.float64)
        H = np.empty((self.M, self.N), order="F")
        self._check(self._L.pqdts_cuda_BF(self.h, _ptr(V), _ptr(H)), "BF")
        return H

    def BF32(self, V):
        """The mixed-precision solver's FP32 Hessian product (mixed problems)."""
        V = np.asfortranarray(V, np.float64)
        H = np.empty((self.M, self.N), order="F")
        self._check(self._L.pqdts_cuda_BF32(self.h, _ptr(V), _ptr(H)), "BF32")
        return H

    def Bdiag(self):
        B = np.empty((self.M, self.N), order="F")
        self._check(self._L.pqdts_cuda_Bdiag(self.h, _ptr(B)), "Bdiag")
        return B

    def pdot(self, A, B):
        """sum(A*B) over the problem's M x N arrays (pdot, pqdts.f90:589-614)."""
        A = np.asfortranarray(A, np.float64)
        B = np.asfortranarray(B, np.float64)
        out = C.c_double()
        self._check(self._L.pqdts_cuda_pdot(self.h, _ptr(A), _ptr(B), C.byref(out)), "pdot")
        return out.value

    def doproj(self):
        self._check(self._L.pqdts_cuda_doproj(self.h), "doproj")

    def doproj2(self):
        v = C.c_double()
        self._check(self._L.pqdts_cuda_doproj2(self.h, C.byref(v)), "doproj2")
        return v.value

    def conv_test(self):
        v = C.c_double()
        self._check(self._L.pqdts_cuda_conv_test(self.h, C.byref(v)), "conv_test")
        return v.value

    def simplexproj(self, Y):
        Y = np.ascontiguousarray(Y, np.float64)
        rows = 1 if Y.ndim == 1 else Y.shape[0]
        X = np.empty_like(Y)
        self._check(self._L.pqdts_cuda_simplexproj(self.h, _ptr(Y), _ptr(X), Y.shape[-1], rows), "simplexproj")
        return X

    # -- solve ------------------------------------------------------------------
    def solve(self, mode=2, maxiter=100, eps=1e-6, start_stage=1, output=0):
        stats = np.zeros(8)
        self._check(self._L.pqdts_cuda_solve(self.h, int(mode), int(maxiter), float(eps), int(start_stage),
                                             int(output), None, None, _ptr(stats)), "solve")
        return dict(zip(STAT_KEYS, stats.tolist()))

    def run_stage(self, mode, oiter, maxiter=100, eps=1e-6, output=0):
        stats = np.zeros(8)
        self._check(self._L.pqdts_cuda_run_stage(self.h, int(mode), int(oiter), int(maxiter), float(eps),
                                                 int(output), _ptr(stats)), "run_stage")
        return dict(zip(STAT_KEYS, stats.tolist()))

    def set_objective_target(self, target):
        """Extra stopping rule (off by default): stop once L <= target."""
        self._check(self._L.pqdts_cuda_set_objective_target(self.h, float(target)), "set_objective_target")

    def set_option(self, name, value):
        """"graphs" (CG chunks as CUDA graphs) or "autotune" (timed launch
        schedules at set-up), 1 = on (default) / 0 = off."""
        self._check(self._L.pqdts_cuda_set_option(self.h, name.encode(), int(value)), "set_option")

    def get_option(self, name):
        v = C.c_int64()
        self._check(self._L.pqdts_cuda_get_option(self.h, name.encode(), C.byref(v)), "get_option")
        return v.value

    def schedule(self):
        """Launch schedule of the banded products in use (autotuned or heuristic)."""
        keys = ("fwd_tile", "trn_tile", "trn_splits", "trans_threads", "trans_cols", "tuned", "tc", "tc_bn",
                "tc_splits", "tc_splits1", "tc_persistent", "df_fwd", "df_trans", "tc_screen")
        return {k: self.get_option("sched." + k) for k in keys}

    def kernel_launches(self):
        v = C.c_int64()
        self._check(self._L.pqdts_cuda_kernel_launches(self.h, C.byref(v)), "kernel_launches")
        return v.value

    def timer(self, name):
        s = C.c_double()
        n = C.c_int64()
        self._check(self._L.pqdts_cuda_timer(self.h, name.encode(), C.byref(s), C.byref(n)), "timer")
        return s.value, n.value


def _batch_arrays(instances):
    M = np.array([i.M for i in instances], np.int64)
    N = np.array([i.N for i in instances], np.int64)
    D = np.array([i.D for i in instances], np.int64)
    lo = np.concatenate([i.band_lo for i in instances]).astype(np.int64)
    hi = np.concatenate([i.band_hi for i in instances]).astype(np.int64)
    vals = np.concatenate([i.band_val for i in instances]).astype(np.float64)
    row_off = np.concatenate([[0], np.cumsum(D)[:-1]]).astype(np.int64)
    val_off = np.concatenate([[0], np.cumsum([i.band_val.size for i in instances])[:-1]]).astype(np.int64)
    return M, N, D, lo, hi, vals, row_off, val_off


def batch_groups(instances):
    """The lockstep groups solve_batch forms for a mixed-precision batch:
    group index per instance (-1: solved alone).  Host only."""
    M, N, D, lo, hi, vals, row_off, val_off = _batch_arrays(instances)
    out = np.empty(len(instances), np.int32)
    rc = lib().pqdts_cuda_batch_groups(len(instances), _ptr(M), _ptr(N), _ptr(D), _ptr(lo), _ptr(hi), _ptr(vals),
                                       _ptr(row_off), _ptr(val_off), _ptr(out))
    if rc != 0:
        raise PqdtsError(f"pqdts_cuda_batch_groups failed ({rc})")
    return out


def solve_batch(instances, X0=None, precision=FP64, mode=2, maxiter=100, eps=1e-6, device=0, targets=None):
    """Solve independent instances (uneven M, N, D, gamma) on one GPU;
    `targets`: optional per-instance objective targets (stop once L <= it).
    With the environment variable PQDTS_BATCH_GROUPS=1, mixed-precision
    instances that share F are solved in lockstep groups with a joint CG
    (batch_groups shows the grouping); off by default."""
    L = lib()
    k = len(instances)
    M, N, D, lo, hi, vals, row_off, val_off = _batch_arrays(instances)
    P = np.concatenate([i.P.ravel() for i in instances]).astype(np.float64)
    P_off = np.concatenate([[0], np.cumsum(D * N)[:-1]]).astype(np.int64)
    gam = np.array([i.gamma for i in instances], np.float64)
    if X0 is None:
        X = np.concatenate([np.full(m * n, 1.0 / n) for m, n in zip(M, N)])
    else:
        X = np.concatenate([np.asfortranarray(x).ravel(order="F") for x in X0])
    stats = np.zeros(8 * k)
    tg = None if targets is None else np.ascontiguousarray(targets, np.float64)
    if tg is not None and tg.size != k:
        raise ValueError("one target per instance")
    rc = L.pqdts_cuda_solve_batch(int(device), k, _ptr(M), _ptr(N), _ptr(D), _ptr(lo), _ptr(hi), _ptr(vals),
                                  _ptr(row_off), _ptr(val_off), _ptr(P), _ptr(P_off), _ptr(gam), int(precision),
                                  int(mode), int(maxiter), float(eps), None if tg is None else _ptr(tg), _ptr(X),
                                  _ptr(stats))
    if rc != 0:
        raise PqdtsError(f"pqdts_cuda_solve_batch failed ({rc})")
    out, off = [], 0
    for m, n in zip(M, N):
        out.append(X[off : off + m * n].reshape((m, n), order="F"))
        off += m * n
    return out, [dict(zip(STAT_KEYS, stats[8 * j : 8 * j + 8].tolist())) for j in range(k)]


def smooth(X, smo_fact):
    """Smoothing of a restart state (pqdts.f90:1877-1902, pqdts_cuda_smooth,
    host only): a copy of X (M x N) whose rows j > 100 are the mean of the
    rows within nint(j / smo_fact) of j, renormalised to sum 1."""
    Xs = np.array(X, dtype=np.float64, order="F", copy=True)
    if Xs.ndim != 2:
        raise ValueError("X must be M x N")
    rc = lib().pqdts_cuda_smooth(Xs.shape[0], Xs.shape[1], float(smo_fact), _ptr(Xs))
    if rc != 0:
        raise PqdtsError(f"pqdts_cuda_smooth failed ({rc})")
    return Xs


def run_pqdts(N, M, D, P, threads=1, pqdtspath=None, maxiter=100, tol=1e-6, gamma=0, smo_int=0, smo_dist=0,
              start_stage=1, smo_fact=0, output=1, verbose=False, F=None, initial=None, dry=False, benchops=0,
              precision=FP64, device=0):
    """In-process counterpart of the reference wrapper's run_pqdts
    (pqdts.py:30-109): the same arguments with the same meaning and the same
    result, the POVM X (M x N) of the mode-2 solve, without the wrapper's
    data files (COO triplets and a dense copy of F, pqdts.py:15-28, 36-57)
    and without a subprocess.

    P (D x N) and F (D x M; None: the internal F, needs M == (D-1)^2) are
    scipy sparse matrices or arrays, passed on as the COO triplets the
    wrapper would write; `initial` (M x N) is the starting point, smoothed
    first when smo_fact > 0 (the wrapper's read_input = 1 path).  threads,
    pqdtspath (OpenMP threads, the executable) and smo_int, smo_dist
    (unused by the reference too) are accepted and ignored; dry returns None
    without solving, as the wrapper's dry run returns before executing;
    output >= 1 makes no files here (the result is returned); benchops is
    the executable's operation benchmark (pqdts_cuda.x ... bench = 1) and
    raises here.  precision / device choose the GPU path."""
    import scipy.sparse as sps

    if benchops:
        raise ValueError("benchops: run the executable (pqdts_cuda.x, last argument 1)")
    Pc = sps.coo_array(P)
    Fc = None if F is None else sps.coo_array(F)
    if Pc.shape != (D, N) or (Fc is not None and Fc.shape != (D, M)):
        raise ValueError("P must be D x N and F D x M")
    X0 = None
    if initial is not None:
        # Fortran order as the wrapper writes it (pqdts.py:57): a flat
        # length-M*N input is X column by column, a 2-D one is X itself
        X0 = np.asarray(initial, dtype=np.float64).reshape((M, N), order="F")
        if smo_fact > 0:
            X0 = smooth(X0, smo_fact)
    if dry:
        return None
    with Solver(device, verbose) as s:
        s.set_problem_coo(M, N, D, None if Fc is None else (Fc.row, Fc.col, Fc.data), (Pc.row, Pc.col, Pc.data),
                          gamma, precision)
        if X0 is not None:
            s.set_x(X0)
        s.solve(mode=2, maxiter=maxiter, eps=tol, start_stage=start_stage, output=output)
        return s.get_x()
