"""gpu_spmv! / gpu_spmm! (src/spmv/*.jl, src/spmm/*.jl of GPUGraphs.jl).

``gpu_spmv_(C, A, B; mul, add, accum, range, mask)`` computes, for every row r
selected by `mask` (mask[r] != 0) and `range` (1-based rows, a Python range or a
(lo, hi) inclusive pair),

    C[r] = accum(C[r], add_k mul(A[r, k], B[k], r, k, k, 1))

on the GPU, asynchronously on the caller's current torch stream.  Unselected rows
are left untouched.  Argument checks follow _validate_args (src/spmv/CSR.jl:358-408):
DimensionMismatch for shapes, ArgumentError when the result type is not
promote_type(eltype(A), eltype(B)) or when an input is not on the GPU."""
import ctypes

import torch

from . import core
from .algebra import GPUGraphs_add, GPUGraphs_mul, GPUGraphs_second, op_code
from .errors import ArgumentError, DimensionMismatch, SpmmAssertionError, check
from .storage import AbstractSparseGPUMatrix, SparseGPUMatrixCSC, SparseGPUMatrixCSR
from .vectors import SparseGPUVector


def _range_bounds(rng):
    if rng is None:
        return 0, 0
    if isinstance(rng, range):
        if rng.step != 1:
            raise ArgumentError("range must be a unit range")
        lo, hi = rng.start, rng.stop - 1
    else:
        lo, hi = int(rng[0]), int(rng[1])
    if hi < lo:
        return 1, 0  # empty UnitRange
    return lo, hi


def gpu_spmv_(C, A, B, mul=GPUGraphs_mul, add=GPUGraphs_add, accum=GPUGraphs_second,
              range=None, mask=None):
    """In-place semiring SpMV, the drop-in of gpu_spmv! (src/spmv/CSR.jl:2-29)."""
    if not isinstance(A, AbstractSparseGPUMatrix):
        raise ArgumentError("A must be a SparseGPUMatrixCSR, SparseGPUMatrixCSC or SparseGPUMatrixSELL")
    if not isinstance(B, torch.Tensor) or not isinstance(C, torch.Tensor):
        raise ArgumentError("All inputs must be on the same backend")
    if A.size(2) != B.numel():
        raise DimensionMismatch("Matrix dimensions must agree")
    if C.shape[0] != A.size(1):
        raise DimensionMismatch("Matrix dimensions must agree")
    tv, tx, ty = A.dtype_code, core.dtype_code(B), core.dtype_code(C)
    if core.promote_code(tv, tx) != ty:
        raise ArgumentError("Result type must be able to hold the result of the multiplication")
    for t, name in ((B, "B"), (C, "C")):
        core.device_vector(t, name)
        if t.device != A.device:
            raise ArgumentError("All inputs must be on the same backend")
    mcode, mlen, mp = 0, 0, None
    if mask is not None:
        if not isinstance(mask, torch.Tensor) or mask.dim() != 1:
            raise DimensionMismatch("Mask must be a vector")
        if mask.numel() != A.size(1):
            raise DimensionMismatch("Mask length must be equal to the number of rows in A")
        if not mask.is_cuda or mask.device != A.device:
            raise ArgumentError("Mask must be on the same backend as A")
        mask = mask.contiguous()
        mcode, mlen, mp = core.dtype_code(mask), mask.numel(), core.ptr(mask)
    lo, hi = _range_bounds(range)
    L = core.lib()
    # a CSC matrix is the CSR storage of its transpose: its product is the transposed SpMV
    fn = L.gg_spmv_t if isinstance(A, SparseGPUMatrixCSC) else L.gg_spmv
    with torch.cuda.device(A.device):
        c = core.ctx(A.device)
        check(fn(c, A.handle, op_code(mul), op_code(add), op_code(accum), core.ptr(C), ty,
                 C.numel(), core.ptr(B), tx, B.numel(), mp, mcode, mlen, lo, hi), L)
    return None


def _dense_layout(M):
    """(layout code, leading dimension) of a 2-D CUDA tensor: column-major (Julia)
    when its transpose is contiguous, row-major when it is contiguous."""
    if M.dim() != 2:
        raise ArgumentError("expected a matrix")
    r, c = M.shape
    s0, s1 = M.stride()
    if s0 == 1 and (s1 >= max(r, 1) or c <= 1):
        return 0, max(s1, r) if c > 1 else max(r, 1)
    if s1 == 1 and (s0 >= max(c, 1) or r <= 1):
        return 1, max(s0, c) if r > 1 else max(c, 1)
    raise ArgumentError("matrix must be row-major or column-major contiguous")


def gpu_spmm_(C, A, B, mul=GPUGraphs_mul, add=GPUGraphs_add, accum=GPUGraphs_second,
              mask=None, range=None):
    """In-place semiring SpMM, the drop-in of gpu_spmm! (src/spmm/CSR.jl:111-204):
    C[r, j] = accum(C[r, j], add_k mul(A[r, k], B[k, j], r, k, k, j)).
    B and C may be column-major (Julia's layout, e.g. ``t.T.contiguous().T``) or
    row-major; both must use the same layout.  Shape violations raise
    SpmmAssertionError like the reference's @assert."""
    if not isinstance(A, AbstractSparseGPUMatrix) or isinstance(A, SparseGPUMatrixCSC):
        raise ArgumentError("A must be a SparseGPUMatrixCSR or SparseGPUMatrixSELL")
    if B.dim() != 2 or C.dim() != 2:
        raise SpmmAssertionError("B and C must be matrices")
    if A.size(2) != B.shape[0]:
        raise SpmmAssertionError("size(A, 2) == size(B, 1)")
    if C.shape[0] != A.size(1):
        raise SpmmAssertionError("size(C, 1) == size(A, 1)")
    if C.shape[1] != B.shape[1]:
        raise SpmmAssertionError("size(C, 2) == size(B, 2)")
    lb, ldb = _dense_layout(B)
    lc, ldc = _dense_layout(C)
    if B.shape[1] <= 1 and C.shape[1] > 1:
        lb = lc
    if C.shape[1] <= 1:
        lc = lb
        ldc = C.shape[0] if lc == 0 else 1
        ldb = B.shape[0] if lb == 0 else 1
    if lb != lc:
        raise ArgumentError("B and C must have the same layout")
    if not B.is_cuda or not C.is_cuda or B.device != A.device or C.device != A.device:
        raise ArgumentError("All inputs must be on the same backend")
    mcode, mlen, mp = 0, 0, None
    if mask is not None:
        mask = mask.contiguous()
        mcode, mlen, mp = core.dtype_code(mask), mask.numel(), core.ptr(mask)
    lo, hi = _range_bounds(range)
    L = core.lib()
    with torch.cuda.device(A.device):
        c = core.ctx(A.device)
        check(L.gg_spmm(c, A.handle, op_code(mul), op_code(add), op_code(accum), core.ptr(C),
                        core.dtype_code(C), C.shape[0], ldc, core.ptr(B), core.dtype_code(B),
                        B.shape[0], ldb, B.shape[1], lb, mp, mcode, mlen, lo, hi), L)
    return None


def gpu_spmspv_(C, A, B, mul=GPUGraphs_mul, add=GPUGraphs_add, accum=GPUGraphs_second):
    """Semiring SpMV over a sparse input vector, the drop-in of gpu_spmspv!
    (src/spmspv.jl:23-54) over A's CSR storage.  B is a SparseGPUVector; C a dense
    device vector of length size(A, 1).  Every row i holding an entry whose column
    carries an entry of B gets C[i] = accum(C[i], add over those entries, in storage
    order, of mul(A[i, j], B[j], i, j, j, 1)) (absorb early exit as gpu_spmv!); other
    rows are untouched.  Returns the 1-based rows written, ascending (Int32 device
    tensor).  Synchronous.  DimensionMismatch as gpu_spmspv!; ArgumentError when B's
    indices are not strictly increasing inside 1:n."""
    if not isinstance(A, SparseGPUMatrixCSR):
        raise ArgumentError("gpu_spmspv! takes a SparseGPUMatrixCSR")
    if not isinstance(B, SparseGPUVector):
        raise ArgumentError("B must be a SparseGPUVector")
    if A.size(2) != B.n:
        raise DimensionMismatch("Matrix dimensions must agree")
    if not isinstance(C, torch.Tensor) or C.shape[0] != A.size(1):
        raise DimensionMismatch("Matrix dimensions must agree")
    core.device_vector(C, "C")
    tv, tx, ty = A.dtype_code, core.dtype_code(B.nzval), core.dtype_code(C)
    if core.promote_code(tv, tx) != ty:
        raise ArgumentError("Result type must be able to hold the result of the multiplication")
    out = torch.empty(max(A.size(1), 1), dtype=torch.int32, device=A.device)
    cnt = ctypes.c_int64(0)
    L = core.lib()
    with torch.cuda.device(A.device):
        c = core.ctx(A.device)
        check(L.gg_spmspv(c, A.handle, op_code(mul), op_code(add), op_code(accum), core.ptr(C), ty,
                          C.numel(), core.ptr(B.nzind), core.ptr(B.nzval), tx, B.nnz(), B.n,
                          core.ptr(out), ctypes.byref(cnt)), L)
    return out[:cnt.value]


def gpu_spmspv(A, B, mul=GPUGraphs_mul, add=GPUGraphs_add):
    """Allocating form: the SparseGPUVector of length size(A, 1) holding, for the rows
    that have a contributing entry, add over mul(A[i, j], B[j]) (no accum)."""
    tc = core.CODE2TORCH[core.promote_code(A.dtype_code, core.dtype_code(B.nzval))]
    C = torch.zeros(A.size(1), dtype=tc, device=A.device)
    rows = gpu_spmspv_(C, A, B, mul=mul, add=add, accum=GPUGraphs_second)
    return SparseGPUVector(A.size(1), rows, C[rows.long() - 1], device=A.device)


def gpu_spmv_rows_(C, A, B, rows, mul=GPUGraphs_mul, add=GPUGraphs_add, accum=GPUGraphs_second):
    """SpMV of the listed rows only: sparse_masked_csr_spmv_kernel! (src/spmv/CSR.jl:90-115),
    whose mask is a list of 1-based row ids.  C[r] = accum(C[r], add over row r of
    mul(A[r, j], B[j], r, j, j, 1)) for r in rows; other rows untouched.  Synchronous;
    BoundsError for a row outside 1:size(A, 1)."""
    if not isinstance(A, SparseGPUMatrixCSR):
        raise ArgumentError("the row-list SpMV takes a SparseGPUMatrixCSR")
    if A.size(2) != B.numel() or C.shape[0] != A.size(1):
        raise DimensionMismatch("Matrix dimensions must agree")
    for t, name in ((B, "B"), (C, "C")):
        core.device_vector(t, name)
    tv, tx, ty = A.dtype_code, core.dtype_code(B), core.dtype_code(C)
    if core.promote_code(tv, tx) != ty:
        raise ArgumentError("Result type must be able to hold the result of the multiplication")
    if not isinstance(rows, torch.Tensor):
        rows = torch.as_tensor(rows, dtype=torch.int32)
    rows = rows.to(device=A.device, dtype=torch.int32).contiguous()
    L = core.lib()
    with torch.cuda.device(A.device):
        c = core.ctx(A.device)
        check(L.gg_spmv_rows(c, A.handle, op_code(mul), op_code(add), op_code(accum), core.ptr(C),
                             ty, C.numel(), core.ptr(B), tx, B.numel(), core.ptr(rows),
                             rows.numel()), L)
    return None


def synchronize(device=None):
    """KernelAbstractions.synchronize(backend) (test/spmv.jl:25)."""
    L = core.lib()
    check(L.gg_stream_sync(core.ctx(device)), L)


def set_wait_limit(polls, device=None):
    """Poll limit of the device-side waits of later calls on this device's context
    (grid barriers of the persistent searches, bulk-copy waits of the staged SpMV
    kernels); 0 restores the built-in limits.  A wait that runs out makes the call
    raise TimeoutError_ and leaves the context usable."""
    L = core.lib()
    check(L.gg_set_wait_limit(core.ctx(device), int(polls)), L)
