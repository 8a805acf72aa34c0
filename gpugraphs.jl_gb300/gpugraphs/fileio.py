"""Graph files: Rutherford-Boeing and Matrix Market matrices and edge lists, read by the
library on the host (gg_read_rb / gg_read_mtx / gg_read_edgelist), as the reference's
benchmark loads its inputs (benchmark/benchmarks.jl:12-14, 262-266)."""
import ctypes
import os

import numpy as np

from . import core
from .errors import check

PATTERN, INTEGER, SYMMETRIC, SKEW, HERMITIAN = 1, 2, 4, 8, 16


def _take(L, colptr, rowval, values, ncol, nnz):
    try:
        cp = np.ctypeslib.as_array(ctypes.cast(colptr, ctypes.POINTER(ctypes.c_int32)),
                                   shape=(ncol + 1,)).copy()
        if nnz:
            rv = np.ctypeslib.as_array(ctypes.cast(rowval, ctypes.POINTER(ctypes.c_int32)),
                                       shape=(nnz,)).copy()
            vv = np.ctypeslib.as_array(ctypes.cast(values, ctypes.POINTER(ctypes.c_double)),
                                       shape=(nnz,)).copy()
        else:
            rv, vv = np.zeros(0, np.int32), np.zeros(0, np.float64)
    finally:
        for p in (colptr, rowval, values):
            L.gg_host_free(p)
    return cp, rv, vv


class RBData:
    """RutherfordBoeingData(path) (HarwellRutherfordBoeing.jl): ``data`` is the matrix
    as a scipy CSC matrix (Float64 values; ones for pattern files), ``kind`` the flags
    of gg_read_rb (PATTERN, INTEGER, SYMMETRIC, SKEW, HERMITIAN)."""

    def __init__(self, path, expand_symmetric=True):
        import scipy.sparse as sp

        L = core.lib()
        m, n, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        cp, rv, vv = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        kind = ctypes.c_int()
        check(L.gg_read_rb(os.fsencode(path), 1 if expand_symmetric else 0, ctypes.byref(m),
                           ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(cp), ctypes.byref(rv),
                           ctypes.byref(vv), ctypes.byref(kind)), L)
        colptr, rowval, values = _take(L, cp, rv, vv, n.value, nnz.value)
        self.kind = kind.value
        self.colptr, self.rowval, self.nzval = colptr, rowval, values
        self.data = sp.csc_matrix((values, rowval - 1, colptr - 1), shape=(m.value, n.value))


def read_rb(path, expand_symmetric=True):
    """The matrix of a Rutherford-Boeing / Harwell-Boeing file as a scipy CSC matrix."""
    return RBData(path, expand_symmetric).data


def read_mtx(path, expand_symmetric=True):
    """The matrix of a Matrix Market coordinate file as a scipy CSC matrix (Float64
    values, ones for pattern files); symmetric storage expanded unless told not to."""
    import scipy.sparse as sp

    L = core.lib()
    m, n, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    cp, rv, vv = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    kind = ctypes.c_int()
    check(L.gg_read_mtx(os.fsencode(path), 1 if expand_symmetric else 0, ctypes.byref(m),
                        ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(cp), ctypes.byref(rv),
                        ctypes.byref(vv), ctypes.byref(kind)), L)
    colptr, rowval, values = _take(L, cp, rv, vv, n.value, nnz.value)
    return sp.csc_matrix((values, rowval - 1, colptr - 1), shape=(m.value, n.value))


def read_edgelist(path, base=1):
    """(A_T, weighted): the transposed adjacency of an edge-list file as a scipy CSR
    matrix (row v lists the in-neighbours of v; Float64 weights, ones without a third
    column), ready for SparseGPUMatrixCSR.from_scipy."""
    import scipy.sparse as sp

    L = core.lib()
    nv, nnz = ctypes.c_int64(), ctypes.c_int64()
    cp, rv, vv = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    w = ctypes.c_int()
    check(L.gg_read_edgelist(os.fsencode(path), int(base), ctypes.byref(nv), ctypes.byref(nnz),
                             ctypes.byref(cp), ctypes.byref(rv), ctypes.byref(vv), ctypes.byref(w)), L)
    colptr, rowval, values = _take(L, cp, rv, vv, nv.value, nnz.value)
    AT = sp.csr_matrix((values, rowval - 1, colptr - 1), shape=(nv.value, nv.value))
    return AT, bool(w.value)
