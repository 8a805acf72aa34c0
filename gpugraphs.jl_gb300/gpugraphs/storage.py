"""Device storage types: SparseGPUMatrixCSR (src/storage/CSR.jl) and
SparseGPUMatrixSELL (src/storage/SELL.jl) of GPUGraphs.jl.

Fields keep the reference's 1-based layout and are zero-copy torch views of the
library-owned device arrays, so ``A.rowptr``, ``A.colval``, ``A.nzval``,
``A.slice_ptr`` compare equal to the reference's field values
(test/structs.jl:54-56,204-206)."""
import ctypes

import numpy as np
import torch

from . import core
from .errors import ArgumentError, BoundsError, check

_FMT_CSR, _FMT_SELL = 1, 2


def _host_array(a, dtype=None):
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    if dtype is not None:
        a = a.astype(dtype, copy=False)
    return np.ascontiguousarray(a)


class AbstractSparseGPUMatrix:
    """Common interface of the device sparse matrices (src/storage/GPUGraphsMatrix.jl)."""

    def __init__(self):
        self._h = None

    @property
    def handle(self):
        return self._h

    def size(self, i=None):
        """size(A) / size(A, i)."""
        if i is None:
            return (self.m, self.n)
        return self.m if i == 1 else self.n

    @property
    def shape(self):
        return (self.m, self.n)

    def length(self):
        """length(A) = m * n (src/storage/CSR.jl:144)."""
        return self.m * self.n

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and core._lib._lib is not None:
            try:
                core.lib().gg_mat_destroy(h)
            except Exception:
                pass
            self._h = None

    def _info(self):
        L = core.lib()
        fmt, dt = ctypes.c_int(), ctypes.c_int()
        m, n, nnz, nst, C, ns = (ctypes.c_int64() for _ in range(6))
        check(L.gg_mat_info(self._h, ctypes.byref(fmt), ctypes.byref(m), ctypes.byref(n),
                            ctypes.byref(nnz), ctypes.byref(dt), ctypes.byref(nst),
                            ctypes.byref(C), ctypes.byref(ns)), L)
        self.m, self.n, self._nnz = m.value, n.value, nnz.value
        self.dtype_code = dt.value
        self.n_stored, self.slice_size, self.nslices = nst.value, C.value, ns.value
        p, cv, nz, pm = (ctypes.c_void_p() for _ in range(4))
        check(L.gg_mat_arrays(self._h, ctypes.byref(p), ctypes.byref(cv), ctypes.byref(nz),
                              ctypes.byref(pm)), L)
        return p.value, cv.value, nz.value, pm.value

    @property
    def dtype(self):
        return core.CODE2TORCH[self.dtype_code]

    def nnz(self):
        return self._nnz


class SparseGPUMatrixCSR(AbstractSparseGPUMatrix):
    """Compressed Sparse Row matrix on the device (src/storage/CSR.jl:14-92).

    ``SparseGPUMatrixCSR(m, n, rowptr, colval, nzval)`` takes 1-based arrays (numpy
    or torch, host or device) and validates them like CSR.jl:48-63, raising
    ArgumentError.  Use the class methods for the other reference constructors."""

    def __init__(self, m, n, rowptr, colval, nzval, device=None):
        super().__init__()
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else
                           torch.device(device).index or 0)
        if len(rowptr) != m + 1:
            raise ArgumentError("length(rowptr) must be equal to m + 1")
        if len(colval) != len(nzval):
            raise ArgumentError("length(colval) must be equal to length(nzval)")
        on_dev = all(isinstance(a, torch.Tensor) and a.is_cuda for a in (rowptr, colval, nzval))
        if on_dev:
            rp = rowptr.to(torch.int32).contiguous()
            cv = colval.to(torch.int32).contiguous()
            nz = nzval.contiguous()
            code = core.dtype_code(nz)
            args = (ctypes.c_void_p(rp.data_ptr()), ctypes.c_void_p(cv.data_ptr()),
                    ctypes.c_void_p(nz.data_ptr()))
        else:
            rp = _host_array(rowptr)
            cv = _host_array(colval)
            if rp.size and (rp.min() < np.iinfo(np.int32).min or rp.max() > np.iinfo(np.int32).max):
                raise ArgumentError("rowptr does not fit in Int32")
            rp = rp.astype(np.int32)
            if cv.size and (cv.min() < 1 or cv.max() > n):
                raise ArgumentError("colval contains an index out of bounds")
            cv = cv.astype(np.int32)
            nz = _host_array(nzval)
            if nz.dtype not in core.NP2CODE:
                nz = nz.astype(np.float64 if np.issubdtype(nz.dtype, np.floating) else np.int64)
            code = core.NP2CODE[nz.dtype]
            args = (rp.ctypes.data_as(ctypes.c_void_p), cv.ctypes.data_as(ctypes.c_void_p),
                    nz.ctypes.data_as(ctypes.c_void_p))
        with torch.cuda.device(dev):
            c = core.ctx(dev)
            L = core.lib()
            h = ctypes.c_void_p()
            check(L.gg_csr_create(c, int(m), int(n), int(len(colval)), *args, code,
                                  1 if on_dev else 0, ctypes.byref(h)), L)
        self._h = h
        self.device = dev
        p, cv_, nz_, _ = self._info()
        self.rowptr = core.wrap_device(self, p, self.m + 1, core.INT32, dev)
        self.colval = core.wrap_device(self, cv_, self._nnz, core.INT32, dev)
        self.nzval = core.wrap_device(self, nz_, self._nnz, self.dtype_code, dev)

    # ---- reference constructors ----
    @classmethod
    def from_scipy(cls, A, dtype=None, device=None):
        """SparseGPUMatrixCSR(transpose(A_csc)) / SparseGPUMatrixCSR(A_csc)
        (CSR.jl:95-117): the CSR of A with column indices sorted in each row."""
        import scipy.sparse as sp

        A = sp.csr_matrix(A)
        A.sort_indices()
        data = A.data if dtype is None else A.data.astype(dtype)
        return cls(A.shape[0], A.shape[1], A.indptr + 1, A.indices + 1, data, device=device)

    @classmethod
    def from_dense(cls, M, device=None):
        """SparseGPUMatrixCSR(m::Matrix) (CSR.jl:106-113): stores the nonzeros of M."""
        import scipy.sparse as sp

        M = np.asarray(M)
        return cls.from_scipy(sp.csr_matrix(M), dtype=M.dtype, device=device)

    @classmethod
    def empty(cls, m=0, n=0, dtype=np.float32, device=None):
        """SparseGPUMatrixCSR(Tv, Ti, backend) / (m, n, Tv, Ti, backend) (CSR.jl:120-136)."""
        return cls(m, n, np.ones(m + 1, np.int32), np.zeros(0, np.int32),
                   np.zeros(0, dtype), device=device)

    def to_scipy(self):
        import scipy.sparse as sp

        return sp.csr_matrix((self.nzval.cpu().numpy(), self.colval.cpu().numpy() - 1,
                              self.rowptr.cpu().numpy() - 1), shape=(self.m, self.n))

    def __getitem__(self, ij):
        """A[i, j] with 1-based indices (CSR.jl:153-164); BoundsError outside."""
        i, j = ij
        if i < 1 or i > self.m or j < 1 or j > self.n:
            raise BoundsError("attempt to access %dx%d matrix at index [%d, %d]" % (self.m, self.n, i, j))
        lo, hi = int(self.rowptr[i - 1]), int(self.rowptr[i])
        cols = self.colval[lo - 1:hi - 1].cpu()
        hit = (cols == j).nonzero()
        if len(hit) == 0:
            return core.CODE2NP[self.dtype_code].type(0)
        return self.nzval[lo - 1 + int(hit[0])].item()

    def __setitem__(self, ij, v):
        """A[i, j] = v for a stored entry (CSR.jl:166-180)."""
        i, j = ij
        if i < 1 or i > self.m or j < 1 or j > self.n:
            raise BoundsError("attempt to access %dx%d matrix at index [%d, %d]" % (self.m, self.n, i, j))
        lo, hi = int(self.rowptr[i - 1]), int(self.rowptr[i])
        hit = (self.colval[lo - 1:hi - 1].cpu() == j).nonzero()
        if len(hit) == 0:
            raise ArgumentError("Index (%d, %d) is not in the matrix. Adding new values is not supported yet." % (i, j))
        self.nzval[lo - 1 + int(hit[0])] = v
        self.values_changed()

    def values_changed(self):
        """Drop the copies and analyses the library derived from the old values (call
        after writing to ``nzval`` directly)."""
        L = core.lib()
        with torch.cuda.device(self.device):
            check(L.gg_mat_values_changed(core.ctx(self.device), self._h), L)

    def __repr__(self):
        return "SparseGPUMatrixCSR{%s}(%d, %d) - %d explicit elements" % (
            core.CODE2NP[self.dtype_code], self.m, self.n, self._nnz)


class SparseGPUMatrixCSC(AbstractSparseGPUMatrix):
    """Compressed Sparse Column matrix on the device (src/storage/CSC.jl, marked "not
    properly supported yet" in the reference).  ``SparseGPUMatrixCSC(m, n, colptr,
    rowval, nzval)`` follows Julia's SparseMatrixCSC convention (colptr of length
    n + 1, 1-based rows in 1:m; the reference's constructor compares colptr with m + 1,
    the same thing for square matrices).  The arrays are held as the CSR storage of the
    transpose (same colptr / rowval / nzval), and gpu_spmv_ on this type runs the
    transposed SpMV of that handle, so ``C = A * B`` in the semiring."""

    def __init__(self, m, n, colptr, rowval, nzval, device=None):
        super().__init__()
        if len(colptr) != n + 1:
            raise ArgumentError("length(colptr) must be equal to n + 1")
        if len(rowval) != len(nzval):
            raise ArgumentError("length(rowval) must be equal to length(nzval)")
        try:
            self._t = SparseGPUMatrixCSR(n, m, colptr, rowval, nzval, device=device)
        except ArgumentError as e:
            msg = str(e).replace("rowptr", "colptr").replace("colval", "rowval")
            raise ArgumentError(msg.replace("m + 1", "n + 1")) from None
        self.m, self.n, self._nnz = int(m), int(n), self._t.nnz()
        self.dtype_code = self._t.dtype_code
        self.device = self._t.device
        self.colptr, self.rowval, self.nzval = self._t.rowptr, self._t.colval, self._t.nzval

    @property
    def handle(self):
        """The CSR handle of the transpose (the library's view of this matrix)."""
        return self._t.handle

    @classmethod
    def from_scipy(cls, A, dtype=None, device=None):
        """SparseGPUMatrixCSC(A::SparseMatrixCSC, backend): the CSC of A, rows sorted."""
        import scipy.sparse as sp

        A = sp.csc_matrix(A)
        A.sort_indices()
        data = A.data if dtype is None else A.data.astype(dtype)
        return cls(A.shape[0], A.shape[1], A.indptr + 1, A.indices + 1, data, device=device)

    def values_changed(self):
        self._t.values_changed()

    def __repr__(self):
        return "SparseGPUMatrixCSC{%s}(%d, %d) - %d explicit elements" % (
            core.CODE2NP[self.dtype_code], self.m, self.n, self._nnz)


class SparseGPUMatrixSELL(AbstractSparseGPUMatrix):
    """Sliced ELLPACK matrix on the device (src/storage/SELL.jl:3-87).

    ``SparseGPUMatrixSELL(A, slice_size=32, sigma=1)`` builds from a
    SparseGPUMatrixCSR, a scipy sparse matrix or a dense array.  sigma == 1 gives
    the reference layout (identity perm); sigma > 1 sorts rows by decreasing length
    within windows of sigma rows (SELL-C-sigma) to cut padding."""

    def __init__(self, A, slice_size=32, sigma=1, device=None):
        super().__init__()
        if not isinstance(A, SparseGPUMatrixCSR):
            import scipy.sparse as sp

            if sp.issparse(A):
                A = SparseGPUMatrixCSR.from_scipy(A, device=device)
            else:
                A = SparseGPUMatrixCSR.from_dense(A, device=device)
        dev = A.device
        with torch.cuda.device(dev):
            c = core.ctx(dev)
            L = core.lib()
            h = ctypes.c_void_p()
            check(L.gg_sell_create(c, A.handle, int(slice_size), int(sigma), ctypes.byref(h)), L)
        self._h = h
        self.device = dev
        self.sigma = int(sigma)
        p, cv, nz, pm = self._info()
        self.slice_ptr = core.wrap_device(self, p, self.nslices + 1, core.INT32, dev)
        self.colval = core.wrap_device(self, cv, self.n_stored, core.INT32, dev)
        self.nzval = core.wrap_device(self, nz, self.n_stored, self.dtype_code, dev)
        self.perm = core.wrap_device(self, pm, self.m, core.INT32, dev)

    def __getitem__(self, ij):
        """A[i, j] (1-based).  Walks the slice holding row i (the reference's
        getindex strides by A.n, SELL.jl:204-219, which is only right for one slice)."""
        i, j = ij
        if i < 1 or i > self.m or j < 1 or j > self.n:
            raise BoundsError("attempt to access %dx%d matrix at index [%d, %d]" % (self.m, self.n, i, j))
        perm = self.perm.cpu().numpy()
        t = int(np.nonzero(perm == i)[0][0])
        C = self.slice_size
        s, o = divmod(t, C)
        lo, hi = int(self.slice_ptr[s]), int(self.slice_ptr[s + 1])
        cols = self.colval[lo - 1 + o:hi - 1:C].cpu().numpy()
        hit = np.nonzero(cols == j)[0]
        if len(hit) == 0:
            return core.CODE2NP[self.dtype_code].type(0)
        return self.nzval[lo - 1 + o + C * int(hit[0])].item()

    def __repr__(self):
        return "SparseGPUMatrixSELL{%s - int32}(%d, %d) - %d explicit elements" % (
            core.CODE2NP[self.dtype_code], self.m, self.n, self._nnz)


def sprand_gpu(T, m, n, p, seed=None, device=None):
    """sprand_gpu(T, m, n, p, backend) (src/storage/CSR.jl:185-186)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    A = sp.random(m, n, density=p, format="csr", random_state=rng, dtype=np.float64)
    return SparseGPUMatrixCSR.from_scipy(A, dtype=np.dtype(T), device=device)
