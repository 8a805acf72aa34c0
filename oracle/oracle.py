"""ctypes front end of the CPU oracle (oracle.c, gen.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg as the checker.  Every function restates a reference routine; the
C source cites the GPUGraphs.jl file:line for each.  Inputs are numpy arrays with
1-based Int32 index arrays, as in the reference.
"""
import ctypes
import os

import numpy as np

from . import build as _build

BOOL, INT32, INT64, FLOAT32, FLOAT64 = 1, 2, 3, 4, 5
(FIRST, SECOND, ANY, PAIR, ADD, SAFE_ADD, MINUS, RMINUS, MUL, MIN, MAX, LOR, LAND, BOR,
 BAND, BXOR, FIRSTI, FIRSTJ, SECONDI, SECONDJ) = range(1, 21)
OK, DIM, ARG, TYPE, UNSUPPORTED, ASSERT = 0, 1, 2, 3, 4, 9

_NP2T = {np.dtype(np.bool_): BOOL, np.dtype(np.int32): INT32, np.dtype(np.int64): INT64,
         np.dtype(np.float32): FLOAT32, np.dtype(np.float64): FLOAT64}
_T2NP = {v: k for k, v in _NP2T.items()}

_lib = None
P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
U64 = ctypes.c_uint64
D = ctypes.c_double


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        sig = {
            "orc_csr_spmv": [I64, I64, P, P, P, I32, P, I32, P, I32, P, I32, I64, I64, I32, I32, I32],
            "orc_sell_sizes": [I64, P, I64, I64, P, P, P, P],
            "orc_sell_fill": [I64, P, P, P, I32, I64, I64, P, P, P, P],
            "orc_sell_spmv": [I64, I64, I64, I64, P, P, P, I32, P, P, I32, P, I32, P, I32, I64, I64,
                              I32, I32, I32],
            "orc_csr_spmm": [I64, P, P, P, I32, P, I32, I64, P, I32, I64, I64, I32, P, I32, I64, I64,
                             I32, I32, I32],
            "orc_sell_spmm": [I64, I64, I64, P, P, P, I32, P, P, I32, I64, P, I32, I64, I64, I32, P,
                              I32, I64, I64, I32, I32, I32],
            "orc_bfs_levels": [I64, P, P, P, I32, I64, P, I64],
            "orc_bfs_parents": [I64, P, P, I64, I32, P],
            "orc_sssp": [I64, P, P, P, I32, P, I64, P, I32, I64],
            "orc_csr_spmv_plus_times_f32": [I64, P, P, P, P, P],
            "orc_csr_spmv_plus_times_f32_rows": [I64, I64, P, P, P, P, P],
            "orc_gen_rmat": [I32, I64, D, D, D, U64, I32, P, P, P],
            "orc_gen_er": [I64, I64, U64, I32, P, P, P],
            "orc_gen_grid": [I64, I64, U64, I32, P, P, P],
            "orc_gen_uniform_f32": [I64, U64, P],
            "orc_coo_to_csr": [I64, I64, P, P, P, I32, I32, I32, P, P, P, P],
            "orc_csr_spmspv": [I64, I64, P, P, P, I32, P, I32, P, P, I32, I64, I32, I32, I32, P,
                               P],
            "orc_csr_spmv_rows": [I64, P, P, P, I32, P, I32, P, I32, P, I64, I32, I32, I32],
            "orc_ewise": [I32, P, I32, P, I32, P, I32, I64, P, I32],
            "orc_apply": [I32, P, I32, P, I32, P, I32, I32, I64, P, I32],
            "orc_reduce": [I32, P, I32, I64, P],
            "orc_bfs_levels_fast": [I64, P, P, P, I32, I64, P, I32],
            "orc_bfs_parents_from_levels": [I64, P, P, P, I64, I32, P],
            "orc_bfs_levels_multi": [I64, P, P, P, I64, P, I64, P, I32],
            "orc_sssp_dijkstra": [I64, P, P, P, I32, I64, P, I32],
            "orc_num_threads": [],
            "orc_set_num_threads": [I32],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = I64 if name in ("orc_bfs_levels", "orc_bfs_parents", "orc_sssp",
                                        "orc_bfs_levels_fast") else I32
        L.orc_set_num_threads.restype = None
        L.orc_bfs_parents_from_levels.restype = None
        L.orc_csr_spmv_plus_times_f32.restype = None
        L.orc_csr_spmv_plus_times_f32_rows.restype = None
        for g in ("orc_gen_rmat", "orc_gen_er", "orc_gen_grid", "orc_gen_uniform_f32"):
            getattr(L, g).restype = None
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def tcode(a):
    return _NP2T[np.asarray(a).dtype]


def npdtype(code):
    return _T2NP[code]


def _c(a, dt=None):
    a = np.ascontiguousarray(a if dt is None else np.asarray(a, dtype=dt))
    return a


def _range(rng):
    if rng is None:
        return 0, 0
    lo, hi = rng
    return int(lo), int(hi)


def csr_spmv(m, n, rowptr, colval, nzval, y, x, mul=MUL, add=ADD, accum=SECOND, mask=None,
             range_=None):
    """gpu_spmv!(y, A::CSR, x; mul, add, accum, range, mask) (src/spmv/CSR.jl:2-29);
    y is updated in place; returns the status code."""
    rowptr, colval, nzval, x = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval), _c(x)
    assert y.flags.c_contiguous
    mask = None if mask is None else _c(mask)
    lo, hi = _range(range_)
    return lib().orc_csr_spmv(m, n, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), _p(y),
                              tcode(y), _p(x), tcode(x), _p(mask),
                              0 if mask is None else tcode(mask), lo, hi, mul, add, accum)


def sell_build(m, rowptr, colval, nzval, slice_size=32, sigma=1):
    """SparseGPUMatrixSELL(transpose(A), backend, slice_size) (src/storage/SELL.jl:99-181),
    plus SELL-C-sigma row sorting when sigma > 1."""
    rowptr, colval, nzval = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval)
    C, ns, nst = I64(), I64(), I64()
    perm = np.zeros(max(m, 1), np.int32)
    lib().orc_sell_sizes(m, _p(rowptr), slice_size, sigma, ctypes.byref(C), ctypes.byref(ns),
                         ctypes.byref(nst), _p(perm))
    slice_ptr = np.zeros(ns.value + 1, np.int32)
    s_col = np.zeros(nst.value, np.int32)
    s_val = np.zeros(nst.value, nzval.dtype)
    if ns.value > 0:
        lib().orc_sell_fill(m, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), C.value, ns.value,
                            _p(perm), _p(slice_ptr), _p(s_col), _p(s_val))
    else:
        slice_ptr[0] = 1
    return dict(m=m, slice_size=C.value, nslices=ns.value, n_stored=nst.value,
                slice_ptr=slice_ptr, colval=s_col, nzval=s_val, perm=perm[:m])


def sell_spmv(S, n, y, x, mul=MUL, add=ADD, accum=SECOND, mask=None, range_=None):
    """gpu_spmv!(y, A::SELL, x; ...) (src/spmv/SELL.jl:2-29)."""
    x = _c(x)
    mask = None if mask is None else _c(mask)
    lo, hi = _range(range_)
    perm = S["perm"] if S["m"] > 0 else np.zeros(1, np.int32)
    return lib().orc_sell_spmv(S["m"], n, S["slice_size"], S["nslices"], _p(S["slice_ptr"]),
                               _p(S["colval"]), _p(S["nzval"]), tcode(S["nzval"]), _p(perm),
                               _p(y), tcode(y), _p(x), tcode(x), _p(mask),
                               0 if mask is None else tcode(mask), lo, hi, mul, add, accum)


def _ld(a, layout):
    # leading dimension of a 2-D numpy array viewed in the given layout
    if layout == 0:
        assert a.flags.f_contiguous
        return a.shape[0]
    assert a.flags.c_contiguous
    return a.shape[1]


def csr_spmm(m, rowptr, colval, nzval, Cm, B, layout=0, mul=MUL, add=ADD, accum=SECOND,
             mask=None, range_=None):
    """gpu_spmm!(C, A::CSR, B; ...) (src/spmm/CSR.jl:111-204); C updated in place."""
    rowptr, colval, nzval = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval)
    mask = None if mask is None else _c(mask)
    lo, hi = _range(range_)
    return lib().orc_csr_spmm(m, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), _p(Cm),
                              tcode(Cm), _ld(Cm, layout), _p(B), tcode(B), _ld(B, layout),
                              B.shape[1], layout, _p(mask), 0 if mask is None else tcode(mask),
                              lo, hi, mul, add, accum)


def sell_spmm(S, Cm, B, layout=0, mul=MUL, add=ADD, accum=SECOND, mask=None, range_=None):
    """gpu_spmm!(C, A::SELL, B; ...) (src/spmm/SELL.jl:84-124)."""
    mask = None if mask is None else _c(mask)
    lo, hi = _range(range_)
    perm = S["perm"] if S["m"] > 0 else np.zeros(1, np.int32)
    return lib().orc_sell_spmm(S["m"], S["slice_size"], S["nslices"], _p(S["slice_ptr"]),
                               _p(S["colval"]), _p(S["nzval"]), tcode(S["nzval"]), _p(perm),
                               _p(Cm), tcode(Cm), _ld(Cm, layout), _p(B), tcode(B),
                               _ld(B, layout), B.shape[1], layout, _p(mask),
                               0 if mask is None else tcode(mask), lo, hi, mul, add, accum)


def bfs_levels(n, rowptr, colval, nzval, source, max_levels=0):
    """bfs_distances(A_T, source) (src/algorithms/bfs.jl:1-73) -> (dist Int32, levels);
    max_levels > 0 stops early and returns -levels."""
    rowptr, colval, nzval = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval)
    dist = np.empty(n, np.int32)
    lv = lib().orc_bfs_levels(n, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), source,
                              _p(dist), max_levels)
    return dist, lv


def bfs_parents(n, rowptr, colval, source, rule):
    """bfs_parents(A_T, source) (src/algorithms/bfs.jl:113-183); rule 1 = CSR (first
    frontier column in storage order), 2 = SELL (largest frontier column)."""
    rowptr, colval = _c(rowptr, np.int32), _c(colval, np.int32)
    par = np.empty(n, np.int32)
    lv = lib().orc_bfs_parents(n, _p(rowptr), _p(colval), source, rule, _p(par))
    return par, lv


def bfs_levels_fast(n, rowptr, colval, nzval, source, symmetric=False):
    """bfs_distances(A_T, source) by frontier BFS (O(nnz); the same levels as
    bfs_levels).  nzval None = every stored entry is an edge; symmetric=True states
    A_T == A (no transpose is built).  Returns (dist, largest level)."""
    rowptr, colval = _c(rowptr, np.int32), _c(colval, np.int32)
    nzval = None if nzval is None else _c(nzval)
    dist = np.empty(n, np.int32)
    lv = lib().orc_bfs_levels_fast(n, _p(rowptr), _p(colval), _p(nzval),
                                   0 if nzval is None else tcode(nzval), source, _p(dist),
                                   int(bool(symmetric and nzval is None)))
    if lv < 0:
        raise MemoryError("orc_bfs_levels_fast")
    return dist, lv


def bfs_parents_fast(n, rowptr, colval, source, rule, dist=None, symmetric=False):
    """bfs_parents(A_T, source) from the pattern's hop distances (O(nnz); the same
    parents as bfs_parents)."""
    rowptr, colval = _c(rowptr, np.int32), _c(colval, np.int32)
    if dist is None:
        dist, _ = bfs_levels_fast(n, rowptr, colval, None, source, symmetric)
    dist = _c(dist, np.int32)
    par = np.empty(n, np.int32)
    lib().orc_bfs_parents_from_levels(n, _p(rowptr), _p(colval), _p(dist), source, rule, _p(par))
    return par


def bfs_levels_multi(n, rowptr, colval, sources, rows, symmetric=False):
    """Hop distances of every source (shortest_path(A_T, sources) with Bool A_T) on
    the listed 0-based rows: (len(rows), S) array, column q for sources[q]."""
    rowptr, colval = _c(rowptr, np.int32), _c(colval, np.int32)
    src = _c(np.atleast_1d(sources), np.int64)
    rows = _c(rows, np.int64)
    out = np.empty((len(rows), len(src)), dtype=np.int32, order="F")
    rc = lib().orc_bfs_levels_multi(n, _p(rowptr), _p(colval), _p(src), len(src), _p(rows),
                                    len(rows), _p(out), int(bool(symmetric)))
    if rc != OK:
        raise MemoryError("orc_bfs_levels_multi")
    return out


def sssp_dijkstra(n, rowptr, colval, nzval, source, symmetric=False):
    """shortest_path(A_T, source) by Dijkstra (Bool / Int32 / Float32 values, all
    non-negative): the Jacobi fixpoint of sssp bit for bit.  Returns dist (Int32
    for Bool / Int32, Float32 for Float32)."""
    rowptr, colval, nzval = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval)
    td = dist_type(tcode(nzval))
    dist = np.empty(n, dtype=npdtype(td))
    rc = lib().orc_sssp_dijkstra(n, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), source,
                                 _p(dist), int(bool(symmetric)))
    if rc != OK:
        raise ValueError("orc_sssp_dijkstra: status %d (negative / NaN weights or overflow)" % rc)
    return dist


def dist_type(tv):
    """T_dist = Int32 for Bool matrices, else the value type (shortest_path.jl:18)."""
    return INT32 if tv == BOOL else tv


def sssp(n, rowptr, colval, nzval, sources, max_rounds=0):
    """shortest_path(A_T, source | sources) (src/algorithms/shortest_path.jl:12-161).
    Returns (dist n x S column-major, rounds)."""
    rowptr, colval, nzval = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval)
    src = _c(np.atleast_1d(sources), np.int64)
    td = dist_type(tcode(nzval))
    dist = np.empty((n, len(src)), dtype=npdtype(td), order="F")
    rounds = lib().orc_sssp(n, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), _p(src), len(src),
                            _p(dist), td, max_rounds)
    return dist, rounds


def csr_spmspv(m, n, rowptr, colval, nzval, y, x_ind, x_val, mul=MUL, add=ADD, accum=SECOND):
    """SpMSpV (src/spmspv.jl:1-54 over CSR): y updated in place on the rows reached;
    returns (status, 1-based rows written ascending)."""
    rowptr, colval, nzval = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval)
    x_ind, x_val = _c(x_ind, np.int32), _c(x_val)
    assert y.flags.c_contiguous
    out = np.zeros(max(m, 1), dtype=np.int32)
    cnt = ctypes.c_int64(0)
    rc = lib().orc_csr_spmspv(m, n, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), _p(y),
                              tcode(y), _p(x_ind), _p(x_val), tcode(x_val), len(x_ind), mul,
                              add, accum, _p(out), ctypes.byref(cnt))
    return rc, out[:cnt.value].copy()


def csr_spmv_rows(m, rowptr, colval, nzval, y, x, rows, mul=MUL, add=ADD, accum=SECOND):
    """sparse_masked_csr_spmv_kernel! (src/spmv/CSR.jl:90-115): the listed 1-based rows."""
    rowptr, colval, nzval, x = _c(rowptr, np.int32), _c(colval, np.int32), _c(nzval), _c(x)
    rows = _c(rows, np.int32)
    assert y.flags.c_contiguous
    return lib().orc_csr_spmv_rows(m, _p(rowptr), _p(colval), _p(nzval), tcode(nzval), _p(y),
                                   tcode(y), _p(x), tcode(x), _p(rows), len(rows), mul, add,
                                   accum)


def ewise(op, z, x, y, mask=None):
    """z[i] = op(x[i], y[i]) where mask[i] != 0; z updated in place; returns the status."""
    x, y = _c(x), _c(y)
    mask = None if mask is None else _c(mask)
    assert z.flags.c_contiguous
    return lib().orc_ewise(op, _p(z), tcode(z), _p(x), tcode(x), _p(y), tcode(y), len(x), _p(mask),
                           0 if mask is None else tcode(mask))


def apply_scalar(op, z, x, s, s_first=False, mask=None):
    """z[i] = op(x[i], s) or op(s, x[i]); s a numpy scalar; returns the status."""
    x = _c(x)
    sv = np.array([s], dtype=np.asarray(s).dtype)
    mask = None if mask is None else _c(mask)
    return lib().orc_apply(op, _p(z), tcode(z), _p(x), tcode(x), _p(sv), tcode(sv),
                           1 if s_first else 0, len(x), _p(mask), 0 if mask is None else tcode(mask))


def reduce(add, x):
    """(status, add over x in the library's fixed chunk / butterfly order)."""
    x = _c(x)
    out = np.zeros(1, dtype=x.dtype)
    rc = lib().orc_reduce(add, _p(x), tcode(x), len(x), _p(out))
    return rc, out[0]


def spmv_plus_times_f32(rowptr, colval, nzval, x, y, rows=None):
    """csr_spmv_kernel! with (mul, add, second) on Float32 (src/spmv/CSR.jl:31-54),
    OpenMP over rows; rows=(r0, r1) restricts to a 0-based row window."""
    m = len(rowptr) - 1
    if rows is None:
        lib().orc_csr_spmv_plus_times_f32(m, _p(rowptr), _p(colval), _p(nzval), _p(x), _p(y))
    else:
        lib().orc_csr_spmv_plus_times_f32_rows(rows[0], rows[1], _p(rowptr), _p(colval),
                                               _p(nzval), _p(x), _p(y))


WEIGHT_DTYPE = {0: np.bool_, 1: np.float32, 2: np.int32, 3: np.float32}


def gen_rmat(scale, nedges, a, b, c, seed, wkind):
    s = np.empty(nedges, np.int32)
    d = np.empty(nedges, np.int32)
    w = np.empty(nedges, WEIGHT_DTYPE[wkind])
    lib().orc_gen_rmat(scale, nedges, a, a + b, a + b + c, seed, wkind, _p(s), _p(d), _p(w))
    return s, d, w


def gen_er(n, nedges, seed, wkind):
    s = np.empty(nedges, np.int32)
    d = np.empty(nedges, np.int32)
    w = np.empty(nedges, WEIGHT_DTYPE[wkind])
    lib().orc_gen_er(n, nedges, seed, wkind, _p(s), _p(d), _p(w))
    return s, d, w


def gen_grid(H, W, seed, wkind):
    ne = H * (W - 1) + (H - 1) * W
    s = np.empty(ne, np.int32)
    d = np.empty(ne, np.int32)
    w = np.empty(ne, WEIGHT_DTYPE[wkind])
    lib().orc_gen_grid(H, W, seed, wkind, _p(s), _p(d), _p(w))
    return s, d, w


def gen_uniform_f32(length, seed):
    out = np.empty(length, np.float32)
    lib().orc_gen_uniform_f32(length, seed, _p(out))
    return out


def coo_to_csr(n, src, dst, w, symmetrize, drop_loops):
    """CSR assembly rule of gen.c: stable (row, column) order, first duplicate kept."""
    src, dst, w = _c(src, np.int32), _c(dst, np.int32), _c(w)
    nnz = I64()
    lib().orc_coo_to_csr(n, len(src), _p(src), _p(dst), _p(w), w.itemsize, int(symmetrize),
                         int(drop_loops), None, None, None, ctypes.byref(nnz))
    rowptr = np.empty(n + 1, np.int32)
    colval = np.empty(nnz.value, np.int32)
    nzval = np.empty(nnz.value, w.dtype)
    lib().orc_coo_to_csr(n, len(src), _p(src), _p(dst), _p(w), w.itemsize, int(symmetrize),
                         int(drop_loops), _p(rowptr), _p(colval), _p(nzval), ctypes.byref(nnz))
    return rowptr, colval, nzval


def num_threads():
    return lib().orc_num_threads()


def set_num_threads(t):
    lib().orc_set_num_threads(int(t))
