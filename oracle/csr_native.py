"""ctypes wrapper of oracle/_build/libcsr_bicgstab.so (built by
oracle/build_oracle.py): the multi-threaded CPU baseline of the assembled
A.  Test infrastructure only; the product never imports it."""
import ctypes as C
import os

import numpy as np

from .build_oracle import OUT, build

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(OUT):
            build()
        lib = C.CDLL(OUT)
        dp = C.POINTER(C.c_double)
        lp = C.POINTER(C.c_int64)
        ip = C.POINTER(C.c_int32)
        lib.csr_threads.restype = C.c_int
        lib.csr_threads.argtypes = [C.c_int]
        lib.csr_spmv.restype = None
        lib.csr_spmv.argtypes = [C.c_int64, lp, ip, dp, dp, dp]
        lib.csr_bicgstab.restype = C.c_int64
        lib.csr_bicgstab.argtypes = [C.c_int64, lp, ip, dp, dp, dp, C.c_double, C.c_int64, dp]
        lib.csr_bicgstabl.restype = C.c_int64
        lib.csr_bicgstabl.argtypes = [C.c_int64, lp, ip, dp, dp, dp, C.c_int, C.c_double, C.c_int64, dp]
        _lib = lib
    return _lib


class NativeCSR:
    """A scipy CSR matrix held in the layout the C code reads."""

    def __init__(self, A, threads=0):
        A = A.tocsr()
        self.n = A.shape[0]
        self.indptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
        self.indices = np.ascontiguousarray(A.indices, dtype=np.int32)
        self.data = np.ascontiguousarray(A.data, dtype=np.complex128)
        self.nnz = int(A.nnz)
        self.threads = load().csr_threads(int(threads))

    def _p(self, a, t):
        return a.ctypes.data_as(C.POINTER(t))

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        load().csr_spmv(self.n, self._p(self.indptr, C.c_int64), self._p(self.indices, C.c_int32),
                        self._p(self.data, C.c_double), self._p(x, C.c_double), self._p(y, C.c_double))
        return y

    def bicgstab(self, b, tol=1e-6, maxit=100000, x0=None):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(x0, dtype=np.complex128).copy()
        rel = C.c_double()
        it = load().csr_bicgstab(self.n, self._p(self.indptr, C.c_int64), self._p(self.indices, C.c_int32),
                                 self._p(self.data, C.c_double), self._p(b, C.c_double), self._p(x, C.c_double),
                                 float(tol), int(maxit), C.byref(rel))
        if it < 0:
            raise MemoryError("csr_bicgstab: allocation failed")
        return x, int(it), rel.value

    def bicgstabl(self, b, ell=4, tol=1e-6, maxmv=200000, x0=None):
        """BiCGStab(ℓ); returns (x, operator applications, recursive relres)."""
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(x0, dtype=np.complex128).copy()
        rel = C.c_double()
        mv = load().csr_bicgstabl(self.n, self._p(self.indptr, C.c_int64), self._p(self.indices, C.c_int32),
                                  self._p(self.data, C.c_double), self._p(b, C.c_double), self._p(x, C.c_double),
                                  int(ell), float(tol), int(maxmv), C.byref(rel))
        if mv < 0:
            raise MemoryError("csr_bicgstabl: allocation failed or bad l")
        return x, int(mv), rel.value
