"""Per-matrix autotuning of the plus-times kernels (gg_tune).

The reference's storage layouts are fixed when a matrix is built (SELL slice height
chosen by the caller, no row sorting: src/storage/SELL.jl:99-181).  autotune() times
the library's own kernels on the matrix -- the built-in choice (column-window tiles
for a large power-law CSR), CSR row blocks of 32..256 rows, SELL-C-sigma layouts with
C in {8, 16, 32} and sigma in {1, 64, 1024, m}, and the SpMM column tile -- and keeps
the fastest on the handle, so later gpu_spmv_ / gpu_spmm_ calls use it."""
import ctypes

from . import core
from .errors import check


class TuneResult(ctypes.Structure):
    _fields_ = [("spmv_kernel", ctypes.c_int), ("block_rows", ctypes.c_int),
                ("slice_size", ctypes.c_int64), ("sigma", ctypes.c_int64),
                ("spmv_ms", ctypes.c_double), ("spmv_default_ms", ctypes.c_double),
                ("mm_cols_per_lane", ctypes.c_int), ("spmm_ms", ctypes.c_double),
                ("candidates", ctypes.c_int), ("sell_variant", ctypes.c_int),
                ("hot_cols", ctypes.c_int)]

# SELL-32 plus-times kernels: register loads (the built-in choice), the matrix stream
# staged by bulk copies, register loads with the hub rows folded from shared-memory
# column windows where dense enough
SELL_VARIANTS = ("registers", "bulk_copy", "hub_windows")
KERNELS = {1: "csr_row_blocks", 2: "sell", 3: "window_tiles"}


def autotune(A, spmm_k=0):
    """Tune A (a Float32 SparseGPUMatrixCSR / SELL) for plus-times SpMV and, when
    spmm_k > 0, SpMM with a row-major n x spmm_k operand.  Returns the choice as a
    dict: spmv_kernel ("csr_row_blocks", "sell" or "window_tiles"), block_rows or (slice_size,
    sigma), the chosen and built-in median times in ms, the SpMM column tile, and
    the number of configurations timed."""
    L = core.lib()
    r = TuneResult()
    check(L.gg_tune(core.ctx(A.device), A.handle, int(spmm_k), ctypes.byref(r)), L)
    out = {"spmv_kernel": KERNELS.get(r.spmv_kernel, "none"),
           "spmv_ms": r.spmv_ms, "spmv_default_ms": r.spmv_default_ms,
           "candidates": r.candidates}
    if r.spmv_kernel == 1:
        out["block_rows"] = r.block_rows
    elif r.spmv_kernel == 2:
        out["slice_size"], out["sigma"] = r.slice_size, r.sigma
        out["sell_variant"] = SELL_VARIANTS[r.sell_variant]
        out["hot_cols"] = r.hot_cols
    if spmm_k > 0:
        out["spmm_column_tile"] = 32 * r.mm_cols_per_lane
        out["spmm_ms"] = r.spmm_ms
    return out


_CACHE = {}


def signature(A):
    """Key of the tuning cache: shape, entries, format and a fingerprint of rowptr
    (the row lengths decide every layout's cost)."""
    import torch
    rp = A.rowptr if hasattr(A, "rowptr") else None
    fp = 0
    if rp is not None and A.m > 0:
        idx = torch.linspace(0, A.m, steps=min(A.m + 1, 257), device=rp.device).long()
        fp = hash(tuple(rp[idx].tolist()))
    return (type(A).__name__, A.m, A.n, A.nnz(), fp)


def apply(A, choice):
    """Apply a dict returned by autotune() (for example for another handle of the
    same matrix) without timing anything."""
    L = core.lib()
    r = TuneResult()
    kind = choice.get("spmv_kernel")
    r.spmv_kernel = {v: k for k, v in KERNELS.items()}.get(kind, 0)
    r.block_rows = int(choice.get("block_rows", 0))
    r.slice_size = int(choice.get("slice_size", 0))
    r.sigma = int(choice.get("sigma", 0))
    r.mm_cols_per_lane = int(choice.get("spmm_column_tile", 0)) // 32
    r.sell_variant = SELL_VARIANTS.index(choice["sell_variant"]) if "sell_variant" in choice else -1
    r.hot_cols = int(choice.get("hot_cols", 0))
    check(L.gg_tune_apply(core.ctx(A.device), A.handle, ctypes.byref(r)), L)


def autotune_cached(A, spmm_k=0):
    """autotune() once per matrix signature in this process; later handles of the same
    matrix get the cached choice through apply()."""
    key = signature(A) + (int(spmm_k),)
    if key in _CACHE:
        apply(A, _CACHE[key])
        return dict(_CACHE[key], cached=True)
    res = autotune(A, spmm_k)
    _CACHE[key] = res
    return dict(res, cached=False)


def spmv_layout(A):
    """Layout the last plus-times Float32 gpu_spmv_ of A ran on: None (no such call
    yet), "csr_row_blocks", "sell" or "window_tiles"."""
    return KERNELS.get(core.lib().gg_spmv_layout(A.handle))


def spmv_hub_rows(A):
    """Rows of A whose plus-times Float32 gpu_spmv_ is folded from shared-memory column
    windows (the hub rows of the sorted SELL-32 layout; 0 when none qualified or no
    such call ran yet)."""
    return int(core.lib().gg_spmv_hub_rows(A.handle))
