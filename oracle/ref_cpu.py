"""nbots' own CPU SpMV and Jacobi-PCG, called through ctypes on the library
that oracle/Makefile.ref builds from the unmodified nbots sources
(oracle/_ref/libnbots_ref.so).

Test and benchmark infrastructure only: the CPU baseline times nbots' own
code with it where that library exists (it is built where the nbots sources
are; a machine without them, or of another architecture, has none and the
baseline falls back to the C restatement in nbots_oracle.c).

The matrix is handed to nbots as its own struct (sparse_struct.h:6-11: row
pointers into the caller's CSR arrays, which must stay alive); nbots' solver
and SpMV only read it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libnbots_ref.so")

_lib = None


class _Sparse(C.Structure):
    _fields_ = [("rows_values", C.POINTER(C.POINTER(C.c_double))),
                ("rows_index", C.POINTER(C.POINTER(C.c_uint32))),
                ("rows_size", C.POINTER(C.c_uint32)), ("N", C.c_uint32)]


def available() -> bool:
    """True when the reference library loads on this machine."""
    try:
        lib()
        return True
    except OSError:
        return False


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(REF_SO)
        sp = C.POINTER(_Sparse)
        L.nb_sparse_multiply_vector.argtypes = [sp, C.c_void_p, C.c_void_p, C.c_uint32]
        L.nb_sparse_multiply_vector.restype = None
        L.nb_sparse_solve_CG_precond_Jacobi.argtypes = [
            sp, C.c_void_p, C.c_void_p, C.c_uint32, C.c_double, C.POINTER(C.c_uint32),
            C.POINTER(C.c_double), C.c_uint32]
        L.nb_sparse_solve_CG_precond_Jacobi.restype = C.c_int
        _lib = L
    return _lib


class Matrix:
    """An nb_sparse_t view of a CSR (row_ptr, col_idx, values)."""

    def __init__(self, rp, ci, K):
        self.rp = np.ascontiguousarray(rp, np.uint32)
        self.ci = np.ascontiguousarray(ci, np.uint32)
        self.K = np.ascontiguousarray(K, np.float64)
        N = self.rp.shape[0] - 1
        self.sizes = np.diff(self.rp).astype(np.uint32)
        vb = self.K.ctypes.data + 8 * self.rp[:-1].astype(np.uint64)
        ib = self.ci.ctypes.data + 4 * self.rp[:-1].astype(np.uint64)
        self.vptr = np.ascontiguousarray(vb, np.uint64)
        self.iptr = np.ascontiguousarray(ib, np.uint64)
        self.s = _Sparse(C.cast(self.vptr.ctypes.data, C.POINTER(C.POINTER(C.c_double))),
                         C.cast(self.iptr.ctypes.data, C.POINTER(C.POINTER(C.c_uint32))),
                         self.sizes.ctypes.data_as(C.POINTER(C.c_uint32)), N)
        self.N = N


def spmv(m: Matrix, x, threads):
    """nb_sparse_multiply_vector (sparse.c:405-414)."""
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros(m.N)
    lib().nb_sparse_multiply_vector(C.byref(m.s), x.ctypes.data, y.ctypes.data, threads)
    return y


def cg_jacobi(m: Matrix, b, tol, threads, max_iter=None, x0=None):
    """nb_sparse_solve_CG_precond_Jacobi (cg_precond_jacobi.c:13-90), absolute
    tolerance as nbots takes it: (x, iterations, tol_reached, status)."""
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(m.N) if x0 is None else np.array(x0, np.float64)
    it, tr = C.c_uint32(0), C.c_double(0.0)
    st = lib().nb_sparse_solve_CG_precond_Jacobi(
        C.byref(m.s), b.ctypes.data, x.ctypes.data, m.N if max_iter is None else max_iter, tol,
        C.byref(it), C.byref(tr), threads)
    return x, it.value, tr.value, st
