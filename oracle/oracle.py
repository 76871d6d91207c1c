"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker.  Arrays follow the reference's layout: X and G are
(M, N) column-major (Fortran order), O and P are (N, D) column-major, i.e.
(D, N) row-major numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def lib():
    global _lib
    if _lib is None:
        from . import build as _build

        _build.build()
        L = C.CDLL(os.path.join(HERE, "liboracle.so"))
        p, i64, d, i32 = C.c_void_p, C.c_int64, C.c_double, C.c_int
        L.orc_create.restype = p
        L.orc_create.argtypes = [i64, i64, i64, d, i64, p, p, p, i64, p, p, p]
        L.orc_destroy.argtypes = [p]
        L.orc_set_threads.argtypes = [i32]
        L.orc_band.restype = i64
        L.orc_band.argtypes = [p, p, p, p]
        L.orc_band_values.argtypes = [p, p]
        L.orc_get_P.argtypes = [p, p]
        L.orc_set_space.argtypes = [p, i32, p]
        L.orc_get_maxr.argtypes = [p, p]
        L.orc_L.restype = d
        L.orc_L.argtypes = [p, p]
        L.orc_redO.argtypes = [p, p, p]
        L.orc_dL.argtypes = [p, p, p]
        L.orc_BF.argtypes = [p, p, p]
        L.orc_Bdiag.argtypes = [p, p]
        L.orc_doproj.argtypes = [p, p]
        L.orc_doproj2.restype = d
        L.orc_doproj2.argtypes = [p, p]
        L.orc_conv_test.restype = d
        L.orc_conv_test.argtypes = [p, p, p]
        L.orc_pdot.restype = d
        L.orc_pdot.argtypes = [p, p, p]
        L.orc_timer.restype = d
        L.orc_timer.argtypes = [p, C.c_char_p]
        L.orc_condat.argtypes = [p, p, i64]
        L.orc_solve.restype = i32
        L.orc_solve.argtypes = [p, p, i32, i32, d, i32, i32, i32, p, p, p]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def condat(y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    x = np.empty_like(y)
    lib().orc_condat(_ptr(y), _ptr(x), y.size)
    return x


def set_threads(n):
    lib().orc_set_threads(int(n))


class Oracle:
    """One problem instance of the restated reference solver."""

    def __init__(self, M, N, D, gamma, F_coo=None, P_coo=None):
        self.M, self.N, self.D = int(M), int(N), int(D)
        L = lib()
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
        self._keep = (fr, fc, fv, pr, pc, pv)
        self.h = L.orc_create(self.M, self.N, self.D, float(gamma), nf, _ptr(fr), _ptr(fc), _ptr(fv), npp, _ptr(pr),
                              _ptr(pc), _ptr(pv))
        if not self.h:
            raise ValueError("oracle rejected the problem (index out of range or M != (D-1)^2 for internal F)")

    @classmethod
    def from_instance(cls, inst):
        return cls(inst.M, inst.N, inst.D, inst.gamma, inst.coo_F(), inst.coo_P())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def _X(self, X):
        X = np.asfortranarray(X, dtype=np.float64)
        assert X.shape == (self.M, self.N)
        return X

    def bands(self):
        lo = np.empty(self.D, np.int64)
        hi = np.empty(self.D, np.int64)
        off = np.empty(self.D, np.int64)
        nnz = lib().orc_band(self.h, _ptr(lo), _ptr(hi), _ptr(off))
        val = np.empty(nnz, np.float64)
        lib().orc_band_values(self.h, _ptr(val))
        return lo, hi, off, val

    def P(self):
        P = np.empty((self.D, self.N))
        lib().orc_get_P(self.h, _ptr(P))
        return P

    def set_space(self, fullspace, maxr=None):
        m = None if maxr is None else np.ascontiguousarray(maxr, np.int32)
        lib().orc_set_space(self.h, 1 if fullspace else 0, _ptr(m))

    def maxr(self):
        m = np.empty(self.M, np.int32)
        lib().orc_get_maxr(self.h, _ptr(m))
        return m

    def L(self, X):
        X = self._X(X).copy(order="F")
        v = lib().orc_L(self.h, _ptr(X))
        return v, X

    def redO(self, X):
        X = self._X(X)
        O = np.empty((self.D, self.N))
        lib().orc_redO(self.h, _ptr(X), _ptr(O))
        return O

    def dL(self, X):
        X = self._X(X).copy(order="F")
        G = np.empty((self.M, self.N), order="F")
        lib().orc_dL(self.h, _ptr(X), _ptr(G))
        return G, X

    def BF(self, V):
        V = self._X(V)
        B = np.empty((self.M, self.N), order="F")
        lib().orc_BF(self.h, _ptr(V), _ptr(B))
        return B

    def Bdiag(self):
        B = np.empty((self.M, self.N), order="F")
        lib().orc_Bdiag(self.h, _ptr(B))
        return B

    def doproj(self, X):
        X = self._X(X).copy(order="F")
        lib().orc_doproj(self.h, _ptr(X))
        return X

    def doproj2(self, X):
        X = self._X(X).copy(order="F")
        xmin = lib().orc_doproj2(self.h, _ptr(X))
        return X, xmin

    def conv_test(self, X):
        X = self._X(X).copy(order="F")
        G = np.empty((self.M, self.N), order="F")
        c = lib().orc_conv_test(self.h, _ptr(X), _ptr(G))
        return c, X, G

    def pdot(self, A, B):
        return lib().orc_pdot(self.h, _ptr(self._X(A)), _ptr(self._X(B)))

    def solve(self, X0=None, mode=2, maxiter=100, eps=1e-6, start_stage=1, verbose=False):
        X = np.full((self.M, self.N), 1.0 / self.N, order="F") if X0 is None else self._X(X0).copy(order="F")
        stats = np.zeros(8)
        lib().orc_solve(self.h, _ptr(X), int(mode), int(maxiter), float(eps), int(start_stage), 0, 1 if verbose else 0,
                        _ptr(stats), None, None)
        keys = ["L", "conv", "norm_der", "outer", "cg", "ls", "dl", "seconds"]
        return X, dict(zip(keys, stats.tolist()))
