"""GPU parity of gpu_spmv_ / gpu_spmm_ and the storage types against the CPU oracle,
the reference's golden vectors and an FP64 oracle.

Tolerance: integer, Bool, min/max/any/or semirings and every row folded in storage
order (CSR rows of at most 32 entries, SELL rows of at most 128, SpMM rows of at
most 256) are compared bit for bit.  Float32 plus-times rows that the kernels reduce in parallel
(CSR rows longer than 32 entries) are compared with rtol 1e-5 against the FP64
product (the reference's own isapprox tests use rtol ~3.4e-4)."""
import itertools

import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from gpugraphs import core
from oracle import oracle as O
from helpers import csr_from_scipy, golden_json, sprand_csr

pytestmark = pytest.mark.gpu
RTOL = 1e-5
SELL_CHUNK = 128  # slice columns one SELL thread folds in storage order
SEG_MM = 256  # SpMM rows longer than this are folded in pieces


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def nan_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if np.issubdtype(a.dtype, np.floating):
        return np.array_equal(np.isnan(a), np.isnan(b)) and (a[~np.isnan(a)] == b[~np.isnan(b)]).all()
    return np.array_equal(a, b)


def power_law_csr(m, seed, dtype=np.float32):
    """Rows with 0 .. ~5000 entries: exercises short-row blocks, empty rows and
    long-row segments."""
    rng = np.random.default_rng(seed)
    deg = np.minimum((rng.pareto(1.2, m) * 3).astype(np.int64), m // 2)
    deg[:3] = [m // 2, min(3000, m - 1), min(300, m - 1)]
    deg[rng.random(m) < 0.2] = 0
    rows, cols = [], []
    for r in range(m):
        c = rng.choice(m, deg[r], replace=False)
        rows.append(np.full(deg[r], r))
        cols.append(c)
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    vals = rng.random(len(rows)).astype(dtype)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(m, m))
    return csr_from_scipy(A) + (A,)


# --------------------------------------------------------------------------------
# storage
# --------------------------------------------------------------------------------

def test_csr_fields_roundtrip():
    """test/structs.jl:30-78: fields equal the reference arrays, getindex agrees."""
    rowptr, colval, nzval, A = sprand_csr(10, 10, 0.5, seed=1)
    for B in (G.SparseGPUMatrixCSR(10, 10, rowptr, colval, nzval),
              G.SparseGPUMatrixCSR.from_scipy(A),
              G.SparseGPUMatrixCSR.from_dense(A.toarray()),
              G.SparseGPUMatrixCSR(10, 10, dev(rowptr), dev(colval), dev(nzval))):
        assert B.size() == (10, 10) and B.length() == 100 and B.nnz() == A.nnz
        assert (host(B.rowptr) == rowptr).all()
        assert (host(B.colval) == colval).all()
        assert (host(B.nzval) == nzval).all()
        D = A.toarray()
        for i, j in [(1, 1), (3, 7), (10, 10), (5, 2)]:
            assert B[i, j] == D[i - 1, j - 1]
        with pytest.raises(G.BoundsError):
            B[11, 1]
    E = G.SparseGPUMatrixCSR.empty(0, 0)
    assert E.size() == (0, 0) and E.nnz() == 0


def test_csr_constructor_errors_golden():
    """test/structs.jl:79-149: every case throws ArgumentError."""
    for case in golden_json("csr_errors.json")["cases"]:
        with pytest.raises(G.ArgumentError):
            G.SparseGPUMatrixCSR(case["m"], case["n"], np.array(case["rowptr"]),
                                 np.array(case["colval"]), np.array(case["nzval"], np.float32))
    # device arrays go through the library's own checks
    case = golden_json("csr_errors.json")["cases"][5]
    with pytest.raises(G.ArgumentError):
        G.SparseGPUMatrixCSR(3, 10, dev(np.array(case["rowptr"], np.int32)),
                             dev(np.array(case["colval"], np.int32)),
                             dev(np.array(case["nzval"], np.float32)))


def test_sell_layout_golden_gpu():
    """test/structs.jl:176-207 through the device SELL builder."""
    g = golden_json("sell_4x4.json")
    D = np.array(g["dense"], np.float32)
    for S in (G.SparseGPUMatrixSELL(sp.csc_matrix(D)), G.SparseGPUMatrixSELL(D)):
        assert S.size() == (4, 4) and S.nnz() == g["nnz"] and S.slice_size == 4
        assert host(S.slice_ptr).tolist() == g["slice_ptr"]
        assert host(S.colval).tolist() == g["colval"]
        assert host(S.nzval).tolist() == g["nzval"]
        for i in range(1, 5):
            for j in range(1, 5):
                assert S[i, j] == D[i - 1, j - 1]


@pytest.mark.parametrize("C,sigma", [(32, 1), (8, 1), (16, 64), (32, 1024), (7, 3)])
def test_sell_layout_matches_oracle(C, sigma):
    rowptr, colval, nzval, A = power_law_csr(600, 2)
    ref = O.sell_build(600, rowptr, colval, nzval, slice_size=C, sigma=sigma)
    S = G.SparseGPUMatrixSELL(G.SparseGPUMatrixCSR(600, 600, rowptr, colval, nzval), C, sigma)
    assert S.n_stored == ref["n_stored"] and S.nslices == ref["nslices"]
    assert (host(S.slice_ptr) == ref["slice_ptr"]).all()
    assert (host(S.colval) == ref["colval"]).all()
    assert (host(S.nzval) == ref["nzval"]).all()
    assert (host(S.perm) == ref["perm"]).all()


# --------------------------------------------------------------------------------
# plus-times Float32 (the headline path)
# --------------------------------------------------------------------------------

@pytest.mark.parametrize("m,p,seed", [(10, 0.5, 1), (1000, 0.2, 2)])
def test_spmv_plus_times_reference_sizes(m, p, seed):
    """test/spmv.jl:10-70 sizes; CSR rows of <= 32 entries and SELL rows of <= 128
    are folded in storage order -> bit-exact."""
    rowptr, colval, nzval, A = sprand_csr(m, m, p, seed=seed)
    x = np.random.default_rng(seed).random(m, dtype=np.float32)
    yo = np.zeros(m, np.float32)
    O.csr_spmv(m, m, rowptr, colval, nzval, yo, x)
    B = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    S = G.SparseGPUMatrixSELL(B)
    ref64 = A.astype(np.float64) @ x.astype(np.float64)
    for M in (B, S):
        y = torch.zeros(m, dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, M, dev(x))
        yh = host(y)
        np.testing.assert_allclose(yh, ref64, rtol=RTOL, atol=1e-6)
        exact = np.diff(rowptr) <= (SELL_CHUNK if M is S else 32)
        assert (yh[exact] == yo[exact]).all()


def test_spmv_plus_times_long_rows():
    m = 6000
    rowptr, colval, nzval, A = power_law_csr(m, 3)
    x = np.random.default_rng(3).random(m, dtype=np.float32)
    yo = np.zeros(m, np.float32)
    O.csr_spmv(m, m, rowptr, colval, nzval, yo, x)
    ref64 = A.astype(np.float64) @ x.astype(np.float64)
    B = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    deg = np.diff(rowptr)
    for rep in range(3):  # the long-row counters reset themselves between launches
        y = torch.full((m,), -1.0, dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, B, dev(x))
        yh = host(y)
        short = deg <= 32
        assert (yh[short] == yo[short]).all()
        np.testing.assert_allclose(yh, ref64, rtol=RTOL, atol=1e-6)
    for C, sigma in ((32, 1), (8, 256), (16, m)):
        S = G.SparseGPUMatrixSELL(B, C, sigma)
        y = torch.zeros(m, dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, S, dev(x))
        yh = host(y)
        # SELL folds each row in storage order within chunks of 128 slice columns;
        # longer rows combine the chunk sums in order
        exact = deg <= SELL_CHUNK
        assert (yh[exact] == yo[exact]).all()
        np.testing.assert_allclose(yh, ref64, rtol=RTOL, atol=1e-6)


def test_spmv_masked_and_range():
    """test/spmv.jl:72-170 plus the range variants (CSR.jl:224-313, SELL.jl:176-283)."""
    m = 1000
    rowptr, colval, nzval, A = sprand_csr(m, m, 0.2, seed=4)
    rng = np.random.default_rng(4)
    x = rng.random(m, dtype=np.float32)
    mask = rng.random(m) < 0.5
    B = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    S = G.SparseGPUMatrixSELL(B, 32, 64)
    ref64 = (A.astype(np.float64) @ x.astype(np.float64))
    for M in (B, S):
        for mk, rg in ((mask, None), (None, range(100, 301)), (mask, (5, 900)), (None, range(7, 7))):
            y = torch.full((m,), -3.0, dtype=torch.float32, device="cuda")
            G.gpu_spmv_(y, M, dev(x), mask=None if mk is None else dev(mk), range=rg)
            sel = np.ones(m, bool) if mk is None else mk.copy()
            if rg is not None:
                lo, hi = (rg.start, rg.stop - 1) if isinstance(rg, range) else rg
                r = np.zeros(m, bool)
                r[lo - 1:hi] = True
                sel &= r
            yh = host(y)
            assert (yh[~sel] == -3.0).all()
            np.testing.assert_allclose(yh[sel], ref64[sel], rtol=RTOL, atol=1e-6)


# --------------------------------------------------------------------------------
# generic semirings: bit parity with the oracle (status codes included)
# --------------------------------------------------------------------------------

SEMIRINGS = [
    (O.MUL, O.ADD, O.SECOND), (O.SAFE_ADD, O.MIN, O.MIN), (O.BAND, O.BOR, O.SECOND),
    (O.SECONDI, O.ANY, O.SECOND), (O.MUL, O.MAX, O.SECOND), (O.PAIR, O.ADD, O.SECOND),
    (O.FIRST, O.MIN, O.MAX), (O.SECOND, O.ANY, O.SECOND), (O.MINUS, O.MAX, O.ADD),
    (O.FIRSTI, O.MIN, O.SECOND), (O.FIRSTJ, O.MAX, O.SECOND), (O.SECONDJ, O.ADD, O.SECOND),
    (O.LAND, O.LOR, O.SECOND), (O.MUL, O.MUL, O.SECOND), (O.BXOR, O.BAND, O.MIN),
    (O.ADD, O.SAFE_ADD, O.SECOND), (O.RMINUS, O.MIN, O.FIRST), (O.MUL, O.BXOR, O.SECOND),
]
TYPES = [(np.bool_, np.bool_), (np.int32, np.int32), (np.int32, np.bool_),
         (np.float32, np.float32), (np.int64, np.int32), (np.float64, np.float32),
         (np.bool_, np.int32), (np.float32, np.int32)]
OPS = {v.code: v for v in G.algebra.OPERATORS.values()}
STATUS_EXC = {O.TYPE: G.ArgumentError, O.UNSUPPORTED: G.UnsupportedError}


def _values(rng, n, dt):
    if dt == np.bool_:
        return rng.random(n) < 0.6
    if np.issubdtype(dt, np.integer):
        v = rng.integers(-4, 9, n).astype(dt)
        v[rng.random(n) < 0.05] = np.iinfo(dt).max
        return v
    v = (rng.random(n) * 4 - 1).astype(dt)
    v[rng.random(n) < 0.05] = np.inf
    return v


def _run_gpu(M, mul, add, accum, y0, x, mask, rng_):
    y = dev(y0)
    kw = dict(mul=OPS[mul], add=OPS[add], accum=OPS[accum])
    if mask is not None:
        kw["mask"] = dev(mask)
    if rng_ is not None:
        kw["range"] = rng_
    # the C ABI accepts y wider than promote_type; call it directly to test the kernels
    L = core.lib()
    mp = core.ptr(kw["mask"]) if mask is not None else None
    lo, hi = rng_ if rng_ is not None else (0, 0)
    rc = L.gg_spmv(core.ctx(), M.handle, mul, add, accum, core.ptr(y), core.dtype_code(y),
                   y.numel(), core.ptr(kw.get("x", dev(x))), core.dtype_code(torch.from_numpy(x)),
                   x.size, mp, 0 if mask is None else core.dtype_code(torch.from_numpy(mask)),
                   0 if mask is None else mask.size, lo, hi)
    return rc, host(y)


@pytest.mark.parametrize("fmt", ["csr", "sell"])
def test_spmv_semiring_grid(fmt):
    rng = np.random.default_rng(7)
    m = 180
    base = sp.random(m, m, density=0.06, random_state=rng, format="csr")
    base.sort_indices()
    rowptr = (base.indptr + 1).astype(np.int32)
    colval = (base.indices + 1).astype(np.int32)
    mask = rng.random(m) < 0.5
    fails = []
    for (tv, tx), (mul, add, accum) in itertools.product(TYPES, SEMIRINGS):
        nz = _values(rng, len(colval), tv)
        x = _values(rng, m, tx)
        ty = np.result_type(tv, tx) if not (tv == np.bool_ and tx == np.bool_) else np.bool_
        if mul in (O.SECONDI, O.FIRSTJ) and ty == np.bool_:
            ty = np.int32
        if mul in (O.FIRSTI, O.SECONDJ) and np.dtype(ty).itemsize < 8:
            ty = np.int64 if not np.issubdtype(ty, np.floating) else np.float64
        y0 = _values(rng, m, ty)
        Bc = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nz)
        M = Bc if fmt == "csr" else G.SparseGPUMatrixSELL(Bc, 8, 4)
        S = O.sell_build(m, rowptr, colval, nz, 8, 4)
        for mk, rg in ((None, None), (mask, None), (None, (20, 150)), (mask, (3, 177))):
            yo = y0.copy()
            if fmt == "csr":
                st = O.csr_spmv(m, m, rowptr, colval, nz, yo, x, mul, add, accum, mk, rg)
            else:
                st = O.sell_spmv(S, m, yo, x, mul, add, accum, mk, rg)
            rc, yg = _run_gpu(M, mul, add, accum, y0, x, mk, rg)
            tag = (fmt, np.dtype(tv).name, np.dtype(tx).name, mul, add, accum, mk is not None, rg)
            if rc != st:
                fails.append(("status", tag, rc, st))
                continue
            if st != O.OK:
                continue
            float_add = np.issubdtype(np.result_type(tv, tx), np.floating) and add in (O.ADD, O.SAFE_ADD, O.MUL)
            parallel = fmt == "csr" and bool((np.diff(rowptr) > 32).any())
            if float_add and parallel:
                ok = np.allclose(yg.astype(np.float64), yo.astype(np.float64), rtol=RTOL,
                                 atol=1e-6, equal_nan=True)
            else:
                ok = nan_equal(yg, yo)
            if not ok:
                fails.append(("value", tag))
    assert not fails, fails[:10]


def test_spmv_errors():
    """_validate_args (src/spmv/CSR.jl:358-408) error classes."""
    rowptr, colval, nzval, A = sprand_csr(20, 30, 0.3, seed=5)
    B = G.SparseGPUMatrixCSR(20, 30, rowptr, colval, nzval)
    x = torch.ones(30, dtype=torch.float32, device="cuda")
    y = torch.zeros(20, dtype=torch.float32, device="cuda")
    with pytest.raises(G.DimensionMismatch):
        G.gpu_spmv_(y, B, torch.ones(29, device="cuda"))
    with pytest.raises(G.DimensionMismatch):
        G.gpu_spmv_(torch.zeros(21, device="cuda"), B, x)
    with pytest.raises(G.ArgumentError):
        G.gpu_spmv_(torch.zeros(20, dtype=torch.int32, device="cuda"), B, x)
    with pytest.raises(G.ArgumentError):
        G.gpu_spmv_(y, B, torch.ones(30))
    with pytest.raises(G.DimensionMismatch):
        G.gpu_spmv_(y, B, x, mask=torch.ones(19, dtype=torch.bool, device="cuda"))
    with pytest.raises(G.UnsupportedError):
        G.gpu_spmv_(y, B, x, mul=G.GPUGraphs_band, add=G.GPUGraphs_bor)
    with pytest.raises(G.ArgumentError):
        G.gpu_spmv_(y, B, x, mul=lambda *a: 0)


# --------------------------------------------------------------------------------
# SpMM
# --------------------------------------------------------------------------------

@pytest.mark.parametrize("layout", [0, 1])
def test_spmm_plus_times(layout):
    """test/spmm.jl:10-73 sizes: each (row, column) is folded in storage order, so the
    result equals the reference's sequential fold bit for bit."""
    for m, k, p, seed in ((10, 5, 0.5, 1), (1000, 20, 0.2, 2), (700, 40, 0.05, 3)):
        rowptr, colval, nzval, A = sprand_csr(m, m, p, seed=seed)
        Bh = np.random.default_rng(seed).random((m, k), dtype=np.float32)
        Bh = np.asfortranarray(Bh) if layout == 0 else np.ascontiguousarray(Bh)
        Co = np.zeros((m, k), np.float32, order="F" if layout == 0 else "C")
        O.csr_spmm(m, rowptr, colval, nzval, Co, Bh, layout=layout)
        ref64 = A.astype(np.float64) @ Bh.astype(np.float64)
        Bc = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
        for M in (Bc, G.SparseGPUMatrixSELL(Bc)):
            if layout == 0:
                Bd = torch.from_numpy(np.ascontiguousarray(Bh.T)).cuda().T
                Cd = torch.zeros((k, m), dtype=torch.float32, device="cuda").T
            else:
                Bd = dev(Bh)
                Cd = torch.zeros((m, k), dtype=torch.float32, device="cuda")
            G.gpu_spmm_(Cd, M, Bd)
            Ch = host(Cd)
            np.testing.assert_allclose(Ch, ref64, rtol=RTOL, atol=1e-5)
            assert (Ch == Co).all()


def test_spmm_min_plus_masked_range():
    m, k = 300, 33
    rng = np.random.default_rng(8)
    base = sp.random(m, m, density=0.05, random_state=rng, format="csr")
    base.sort_indices()
    rowptr = (base.indptr + 1).astype(np.int32)
    colval = (base.indices + 1).astype(np.int32)
    nz = rng.integers(1, 20, len(colval)).astype(np.int32)
    Bh = rng.integers(0, 100, (m, k)).astype(np.int32)
    Bh[rng.random((m, k)) < 0.3] = np.iinfo(np.int32).max
    mask = rng.random(m) < 0.5
    Bc = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nz)
    S = O.sell_build(m, rowptr, colval, nz, 32, 16)
    for fmt, M in (("csr", Bc), ("sell", G.SparseGPUMatrixSELL(Bc, 32, 16))):
        for layout in (0, 1):
            for mk, rg in ((None, None), (mask, None), (None, (10, 250))):
                C0 = rng.integers(0, 50, (m, k)).astype(np.int32)
                C0 = np.asfortranarray(C0) if layout == 0 else np.ascontiguousarray(C0)
                Bl = np.asfortranarray(Bh) if layout == 0 else np.ascontiguousarray(Bh)
                Co = C0.copy(order="K")
                if fmt == "csr":
                    O.csr_spmm(m, rowptr, colval, nz, Co, Bl, layout, O.SAFE_ADD, O.MIN, O.MIN, mk, rg)
                else:
                    O.sell_spmm(S, Co, Bl, layout, O.SAFE_ADD, O.MIN, O.MIN, mk, rg)
                if layout == 0:
                    Bd = torch.from_numpy(np.ascontiguousarray(Bl.T)).cuda().T
                    Cd = torch.from_numpy(np.ascontiguousarray(C0.T)).cuda().T
                else:
                    Bd, Cd = dev(Bl), dev(C0)
                G.gpu_spmm_(Cd, M, Bd, mul=G.GPUGraphs_safe_add, add=G.GPUGraphs_min,
                            accum=G.GPUGraphs_min, mask=None if mk is None else dev(mk), range=rg)
                assert (host(Cd) == Co).all(), (fmt, layout, mk is not None, rg)


def test_spmm_long_rows_power_law():
    """Hub rows (up to m/2 entries) are folded in pieces of 256 by separate warps and
    combined in order: exact for min-plus on Int32, exact for Float32 plus-times rows
    of <= 256 entries, within rtol 1e-5 of FP64 for the others."""
    m, k = 3000, 40
    rowptr, colval, nzval, A = power_law_csr(m, 11)
    deg = np.diff(rowptr)
    assert deg.max() > 4 * SEG_MM
    rng = np.random.default_rng(11)
    Bf = rng.random((m, k), dtype=np.float32)
    ref64 = A.astype(np.float64) @ Bf.astype(np.float64)
    Bc = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    for M in (Bc, G.SparseGPUMatrixSELL(Bc, 32, m), G.SparseGPUMatrixSELL(Bc, 8, 1)):
        for layout in (0, 1):
            Bl = np.asfortranarray(Bf) if layout == 0 else np.ascontiguousarray(Bf)
            Co = np.zeros((m, k), np.float32, order="F" if layout == 0 else "C")
            O.csr_spmm(m, rowptr, colval, nzval, Co, Bl, layout=layout)
            # C starts as NaN: every row (the 20% empty ones too) must be written
            if layout == 0:
                Bd = torch.from_numpy(np.ascontiguousarray(Bf.T)).cuda().T
                Cd = torch.full((k, m), float("nan"), dtype=torch.float32, device="cuda").T
            else:
                Bd = dev(Bf)
                Cd = torch.full((m, k), float("nan"), dtype=torch.float32, device="cuda")
            for rep in range(2):
                G.gpu_spmm_(Cd, M, Bd)
                Ch = host(Cd)
                np.testing.assert_allclose(Ch, ref64, rtol=RTOL, atol=1e-5)
                short = deg <= SEG_MM
                assert (Ch[short] == Co[short]).all()
    # min-plus on Int32 with a mask and a row range: exact on every row
    nzi = rng.integers(1, 50, len(colval)).astype(np.int32)
    Bi = rng.integers(0, 1000, (m, k)).astype(np.int32)
    Bi[rng.random((m, k)) < 0.2] = np.iinfo(np.int32).max
    mask = rng.random(m) < 0.6
    mask[:3] = True
    Ci = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzi)
    S = O.sell_build(m, rowptr, colval, nzi, 32, m)
    for fmt, M in (("csr", Ci), ("sell", G.SparseGPUMatrixSELL(Ci, 32, m))):
        for mk, rg in ((None, None), (mask, None), (None, (1, 2000))):
            C0 = rng.integers(0, 5000, (m, k)).astype(np.int32)
            Co = C0.copy()
            if fmt == "csr":
                O.csr_spmm(m, rowptr, colval, nzi, Co, Bi, 1, O.SAFE_ADD, O.MIN, O.MIN, mk, rg)
            else:
                O.sell_spmm(S, Co, Bi, 1, O.SAFE_ADD, O.MIN, O.MIN, mk, rg)
            Cd = dev(C0)
            G.gpu_spmm_(Cd, M, dev(Bi), mul=G.GPUGraphs_safe_add, add=G.GPUGraphs_min,
                        accum=G.GPUGraphs_min, mask=None if mk is None else dev(mk), range=rg)
            assert (host(Cd) == Co).all(), (fmt, mk is not None, rg)


def test_spmm_assertions():
    rowptr, colval, nzval, A = sprand_csr(20, 30, 0.3, seed=5)
    B = G.SparseGPUMatrixCSR(20, 30, rowptr, colval, nzval)
    with pytest.raises(G.SpmmAssertionError):
        G.gpu_spmm_(torch.zeros((20, 4), device="cuda"), B, torch.zeros((29, 4), device="cuda"))
    with pytest.raises(G.SpmmAssertionError):
        G.gpu_spmm_(torch.zeros((20, 4), device="cuda"), B, torch.zeros((30, 5), device="cuda"))
    with pytest.raises(G.SpmmAssertionError):
        G.gpu_spmm_(torch.zeros((20, 4), device="cuda"), B, torch.zeros((30, 4), device="cuda"),
                    mask=torch.ones(20, device="cuda"), range=(1, 3))


def test_spmv_generic_semirings_on_rmat():
    """Long rows (segments) and short-row blocks of an R-MAT graph through the
    generic-semiring kernels, against the oracle."""
    from gpugraphs import generators as gen
    A = gen.rmat(14, 16, seed=12, wkind=gen.W_INT_1_255)
    rowptr, colval, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    n = A.n
    x = np.random.default_rng(12).integers(0, 1000, n).astype(np.int32)
    for mul, add, accum in ((O.SAFE_ADD, O.MIN, O.MIN), (O.MUL, O.MAX, O.SECOND), (O.BAND, O.BOR, O.SECOND)):
        y0 = np.full(n, 7, np.int32)
        yo = y0.copy()
        assert O.csr_spmv(n, n, rowptr, colval, nz, yo, x, mul, add, accum) == O.OK
        y = dev(y0)
        G.gpu_spmv_(y, A, dev(x), mul=OPS[mul], add=OPS[add], accum=OPS[accum])
        assert (host(y) == yo).all()
    # plus-times Float32 on the same structure (long rows within tolerance)
    B = G.SparseGPUMatrixCSR(n, n, rowptr, colval, nz.astype(np.float32))
    xf = np.random.default_rng(13).random(n, dtype=np.float32)
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, B, dev(xf))
    ref = B.to_scipy().astype(np.float64) @ xf.astype(np.float64)
    np.testing.assert_allclose(host(y), ref, rtol=RTOL, atol=1e-6)


def test_spmv_plus_times_large_csr_sorted_sell_path():
    """CSR of >= 65536 rows, SELL layout chosen: plus-times runs on a SELL-32 copy with rows
    sorted by length, relabelled columns and the hot part of x in shared memory
    (narrow slices grouped per warp, wide ones in chunks; matrix stream staged by bulk
    copies or loaded into registers).  Rows of <= 128 entries are
    folded in storage order -> bit-exact against the oracle; all rows within rtol 1e-5
    of FP64; repeated calls give identical results."""
    from gpugraphs import generators as gen
    A = gen.rmat(17, 16, seed=14, wkind=gen.W_U01_F32)
    rowptr, colval, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    n = A.n
    x = np.random.default_rng(14).random(n, dtype=np.float32)
    yo = np.zeros(n, np.float32)
    O.csr_spmv(n, n, rowptr, colval, nz, yo, x)
    ref = A.to_scipy().astype(np.float64) @ x.astype(np.float64)
    deg = np.diff(rowptr)
    first = None
    from gpugraphs import tuning
    # register loads, bulk-copy staging and hub rows from column windows: the same bits
    # for every row of <= 128 entries; long rows within rounding, and the register and
    # bulk-copy kernels (the same chunk tree) bit for bit; every kernel gives the same
    # bits twice
    seen = {}
    for variant in ["registers", "registers", "bulk_copy", "bulk_copy",
                    "hub_windows", "hub_windows"]:
        tuning.apply(A, {"spmv_kernel": "sell", "slice_size": 32, "sigma": n,
                         "sell_variant": variant})
        y = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, A, dev(x))
        yh = host(y)
        exact = deg <= SELL_CHUNK
        assert (yh[exact] == yo[exact]).all()
        np.testing.assert_allclose(yh, ref, rtol=RTOL, atol=1e-6)
        if variant in seen:
            assert (yh == seen[variant]).all()
        seen[variant] = yh
    assert (seen["bulk_copy"] == seen["registers"]).all()


def test_spmv_long_rows_keep_the_absorb_stop():
    """CSR row blocks (m < 65536): rows longer than 32 entries are reduced by warp
    segments in tree order; a row whose sum is NaN there is folded again in storage
    order with the stop at +Inf, so every row has the oracle's NaN / +Inf / -Inf
    pattern (plain plus-times and the generic masked kernel)."""
    m = 6000
    rowptr, colval, nzval, A = power_law_csr(m, 41)
    rng = np.random.default_rng(41)
    cc = np.bincount(colval - 1, minlength=m)
    x = rng.random(m, dtype=np.float32)
    order = np.argsort(-cc, kind="stable")
    x[order[0]] = np.inf
    x[order[5:400:9]] = np.nan
    x[order[7:400:11]] = -np.inf
    B = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    deg = np.diff(rowptr)
    mask = np.ones(m, np.float32)
    mask[::7] = 0
    for mk in (None, mask):
        y0 = np.full(m, 3.0, np.float32)
        yo = y0.copy()
        O.csr_spmv(m, m, rowptr, colval, nzval, yo, x, mask=mk)
        with np.errstate(invalid="ignore"):
            ref = A.astype(np.float64) @ x.astype(np.float64)
        stop = np.isposinf(yo) & np.isnan(ref)
        assert (stop & (deg > 32)).any() and (stop & (deg <= 32)).any()
        y = dev(y0)
        if mk is None:
            G.gpu_spmv_(y, B, dev(x))
        else:
            G.gpu_spmv_(y, B, dev(x), mask=dev(mk))
        yh = host(y)
        for f in (np.isnan, np.isposinf, np.isneginf):
            assert np.array_equal(f(yh), f(yo)), (f.__name__, mk is None)
        short = deg <= 32
        np.testing.assert_array_equal(yh[short], yo[short])
        fin = np.isfinite(yo)
        if mk is not None:
            fin &= mask != 0
            np.testing.assert_array_equal(yh[mask == 0], y0[mask == 0])
        np.testing.assert_allclose(yh[fin], ref[fin], rtol=RTOL, atol=1e-6)


def special_x(A, seed):
    """x in [0, 1) with +Inf on the most frequent column and on a late column, NaN on
    a light column and -Inf on another: rows reach +Inf before or after the NaN /
    -Inf terms in storage order, in short rows and in hub rows."""
    n = A.n
    colval = host(A.colval)
    cc = np.bincount(colval - 1, minlength=n)
    x = np.random.default_rng(seed).random(n, dtype=np.float32)
    hub = int(np.argmax(cc))
    late = int(np.flatnonzero(cc >= 8)[-1])  # a +Inf column near the end of most rows
    light = [int(c) for c in np.flatnonzero(cc == 1)[:2]]
    mid = np.flatnonzero((cc >= 4) & (cc <= 64))
    x[hub] = np.inf
    x[late] = np.inf
    x[light[0]] = np.nan
    x[light[1]] = -np.inf
    x[mid[1::97][:24]] = np.nan
    x[mid[50::97][:24]] = -np.inf
    return x


@pytest.mark.parametrize("layout", ["registers", "bulk_copy", "window_tiles", "built_in"])
def test_spmv_large_csr_keeps_the_absorb_stop(layout):
    """A CSR of >= 65536 rows runs plus-times on its SELL-32 copy (register or
    bulk-copy staging) or on column-window tiles; the result still follows the
    reference's CSR kernel, whose fold stops once the sum reaches the absorbing +Inf
    (csr_spmv_kernel!, src/spmv/CSR.jl:47-52; monoid_absorb(GPUGraphs_add) = typemax,
    src/algebra.jl:45).  With +Inf, NaN and -Inf in x: every row of at most 128
    entries equals the oracle bit for bit on the SELL copy, every row has the oracle's
    NaN / +Inf / -Inf pattern on every layout, finite rows are within rtol 1e-5 of
    FP64; two calls give the same bits."""
    from gpugraphs import generators as gen
    from gpugraphs import tuning
    A = gen.rmat(17, 16, seed=31, wkind=gen.W_U01_F32)
    n = A.n
    rowptr, colval, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    if layout == "window_tiles":
        tuning.apply(A, {"spmv_kernel": "window_tiles"})
    elif layout != "built_in":
        tuning.apply(A, {"spmv_kernel": "sell", "slice_size": 32, "sigma": n,
                         "sell_variant": layout})
    x = special_x(A, 31)
    yo = np.zeros(n, np.float32)
    assert O.csr_spmv(n, n, rowptr, colval, nz, yo, x) == O.OK
    # the cases the test is about are present
    deg = np.diff(rowptr)
    short = deg <= SELL_CHUNK
    with np.errstate(invalid="ignore"):
        ref = A.to_scipy().astype(np.float64) @ x.astype(np.float64)
    stop = np.isposinf(yo) & np.isnan(ref)  # +Inf reached, then NaN or -Inf
    assert (stop & short).sum() >= 10 and (stop & ~short).sum() >= 1
    assert (np.isnan(yo) & short).any() and (np.isneginf(yo) & short).any()
    first = None
    for _ in range(2):
        y = torch.full((n,), -7.0, dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, A, dev(x))
        yh = host(y)
        if first is None:
            first = yh
        else:
            assert np.array_equal(yh.view(np.int32), first.view(np.int32))
    assert G.spmv_layout(A) == ("window_tiles" if layout == "window_tiles" else "sell")
    for f in (np.isnan, np.isposinf, np.isneginf):
        assert np.array_equal(f(yh), f(yo)), f.__name__
    if layout != "window_tiles":
        np.testing.assert_array_equal(yh[short], yo[short])
    fin = np.isfinite(yo)
    np.testing.assert_allclose(yh[fin], ref[fin], rtol=RTOL, atol=1e-6)
    # the NaN rows the fast fold leaves are refolded like the oracle on long rows too
    np.testing.assert_array_equal(yh[stop], yo[stop])


@pytest.mark.parametrize("scale,seed", [(16, 21), (17, 14), (18, 22)])
def test_spmv_plus_times_window_tiles(scale, seed):
    """Plus-times over column-window tiles of a large power-law CSR (rows
    sorted by length in tiles of 8192, x windows of 16384 relabelled columns staged in
    shared memory, tail ranges gathered, heavy tiles split into units whose partial
    rows are combined in order).  Every row within rtol 1e-5 of FP64 (empty rows 0,
    rows through hubs included); repeated calls give identical bits; NaN and Inf in x
    propagate like the FP64 sums."""
    from gpugraphs import generators as gen
    from gpugraphs import tuning
    A = gen.rmat(scale, 16, seed=seed, wkind=gen.W_U01_F32)
    n = A.n
    tuning.apply(A, {"spmv_kernel": "window_tiles"})
    S = A.to_scipy().astype(np.float64)
    x = np.random.default_rng(seed).random(n, dtype=np.float32)
    ref = S @ x.astype(np.float64)
    first = None
    for _ in range(3):
        y = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, A, dev(x))
        yh = host(y)
        np.testing.assert_allclose(yh, ref, rtol=RTOL, atol=1e-6)
        if first is None:
            first = yh
        else:
            assert (yh == first).all()
    deg = np.diff(host(A.rowptr))
    assert (first[deg == 0] == 0).all()
    # special values: one NaN column, one +Inf column.  A CSR row follows
    # csr_spmv_kernel!'s storage-order fold with its stop at +Inf (CSR.jl:47-52): a row
    # holding the +Inf column before the NaN one is +Inf, after it NaN -- the oracle's
    # pattern, not the FP64 product's
    colcount = np.bincount(host(A.colval) - 1, minlength=n)
    hub = int(np.argmax(colcount))
    light = int(np.flatnonzero(colcount == 1)[0])
    xs = x.copy()
    xs[hub] = np.inf
    xs[light] = np.nan
    yo = np.zeros(n, np.float32)
    O.csr_spmv(n, n, host(A.rowptr), host(A.colval), host(A.nzval), yo, xs)
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, A, dev(xs))
    yh = host(y)
    assert (np.isnan(yh) == np.isnan(yo)).all()
    assert (np.isposinf(yh) == np.isposinf(yo)).all()
    with np.errstate(invalid="ignore"):
        ref_s = S @ xs.astype(np.float64)
    fin = np.isfinite(yo)
    np.testing.assert_allclose(yh[fin], ref_s[fin], rtol=RTOL, atol=1e-6)


def test_spmv_layout_choices_on_large_csr():
    """The built-in choice for a large CSR is the sorted SELL-32 copy; window tiles run
    when chosen and the column frequencies are skewed, else the SELL copy runs."""
    from gpugraphs import generators as gen
    from gpugraphs import tuning
    B = gen.rmat(16, 16, seed=23, wkind=gen.W_U01_F32)
    C = gen.rmat(16, 16, seed=23, wkind=gen.W_U01_F32)  # untouched handle: built-in rule
    assert G.spmv_layout(C) is None
    tuning.apply(B, {"spmv_kernel": "window_tiles"})
    x = np.random.default_rng(23).random(B.n, dtype=np.float32)
    y1 = torch.zeros(B.n, dtype=torch.float32, device="cuda")
    y2 = torch.zeros(B.n, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y1, B, dev(x))
    G.gpu_spmv_(y2, C, dev(x))
    assert G.spmv_layout(B) == "window_tiles" and G.spmv_layout(C) == "sell"
    ref = C.to_scipy().astype(np.float64) @ x.astype(np.float64)
    np.testing.assert_allclose(host(y1), ref, rtol=RTOL, atol=1e-6)
    np.testing.assert_allclose(host(y2), ref, rtol=RTOL, atol=1e-6)
    # a matrix without skewed columns falls back to the SELL copy
    E = gen.erdos_renyi(1 << 16, 16, seed=24, wkind=gen.W_U01_F32)
    tuning.apply(E, {"spmv_kernel": "window_tiles"})
    G.gpu_spmv_(torch.zeros(E.m, device="cuda"), E, dev(np.ones(E.n, np.float32)))
    assert G.spmv_layout(E) == "sell"


@pytest.mark.parametrize("k", [4, 32, 36])
def test_spmm_special_values_fold_like_the_reference(k):
    """Row-major plus-times SpMM with +Inf, -Inf and NaN in B: every row of <= 256
    entries (short rows, medium rows of the four-items-per-warp kernel) equals the
    oracle's sequential fold, including its stop at +Inf (NaN-aware comparison)."""
    m = 3000
    rowptr, colval, nzval, A = power_law_csr(m, 31)
    rng = np.random.default_rng(k)
    B = rng.random((m, k), dtype=np.float32)
    B[rng.random((m, k)) < 0.002] = np.inf
    B[rng.random((m, k)) < 0.001] = -np.inf
    B[rng.random((m, k)) < 0.001] = np.nan
    Co = np.zeros((m, k), np.float32)
    O.csr_spmm(m, rowptr, colval, nzval, Co, B, layout=1)
    M = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    Cd = torch.zeros((m, k), dtype=torch.float32, device="cuda")
    G.gpu_spmm_(Cd, M, dev(B))
    Ch = host(Cd)
    short = np.diff(rowptr) <= SEG_MM
    np.testing.assert_array_equal(Ch[short], Co[short])
    assert (np.isposinf(Co) & short[:, None]).any() and (np.isnan(Co) & short[:, None]).any()


@pytest.mark.parametrize("k", [1, 4, 6, 32])
def test_spmm_writes_every_row(k):
    """Row-major plus-times SpMM with 20% empty rows into a NaN-filled C: every row is
    written (empty rows get the neutral 0), for column counts on and off the
    four-column kernel's alignment."""
    m = 2000
    rowptr, colval, nzval, A = power_law_csr(m, 12)
    B = np.random.default_rng(k).random((m, k), dtype=np.float32)
    Co = np.zeros((m, k), np.float32)
    O.csr_spmm(m, rowptr, colval, nzval, Co, B, layout=1)
    M = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    Cd = torch.full((m, k), float("nan"), dtype=torch.float32, device="cuda")
    G.gpu_spmm_(Cd, M, dev(B))
    Ch = host(Cd)
    assert not np.isnan(Ch).any()
    short = np.diff(rowptr) <= SEG_MM
    assert (Ch[short] == Co[short]).all()
    np.testing.assert_allclose(Ch, Co, rtol=1e-4, atol=1e-4)


def test_spmm_wide_operand_power_law():
    """R-MAT 17 times a 132-column row-major operand (larger than L2; 4-column lanes
    over 33 column groups): sampled rows of <= 256 entries equal the oracle's
    storage-order fold (NaN / Inf in B included, refolded with the stop at +Inf), every
    sampled row is within rtol 1e-5 of FP64 where finite, and two calls give the same
    bits."""
    from gpugraphs import generators as gen
    A = gen.rmat(17, 16, seed=33, wkind=gen.W_U01_F32)
    n, k = A.n, 132
    rp, cv, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    rng = np.random.default_rng(33)
    B = rng.random((n, k), dtype=np.float32)
    B[rng.random((n, k)) < 1e-4] = np.inf
    B[rng.random((n, k)) < 5e-5] = np.nan
    Bd = dev(B)
    first = None
    for _ in range(2):
        C = torch.full((n, k), -3.0, dtype=torch.float32, device="cuda")
        G.gpu_spmm_(C, A, Bd)
        Ch = host(C)
        if first is None:
            first = Ch
        else:
            assert np.array_equal(Ch.view(np.int32), first.view(np.int32))
    deg = np.diff(rp)
    rows = np.unique(np.concatenate([np.argsort(-deg)[:64], rng.integers(0, n, 1500)]))
    short = rows[deg[rows] <= SEG_MM]
    srp = np.concatenate([[1], 1 + np.cumsum(deg[short])]).astype(np.int32)
    idx = np.concatenate([np.arange(rp[r] - 1, rp[r + 1] - 1) for r in short])
    Co = np.zeros((len(short), k), np.float32)
    O.csr_spmm(len(short), srp, cv[idx], nz[idx], Co, B, layout=1)
    np.testing.assert_array_equal(Ch[short], Co)
    with np.errstate(invalid="ignore"):
        ref = A.to_scipy().astype(np.float64)[rows] @ B.astype(np.float64)
    fin = np.isfinite(ref)
    np.testing.assert_allclose(Ch[rows][fin], ref[fin], rtol=RTOL, atol=1e-6)


def test_spmm_one_column_large_csr_equals_the_wide_fold():
    """One dense column on a CSR of >= 65536 rows runs over the SELL-32 copy with
    256-column chunks; it must fold exactly like the 32-column SpMM (rows of <= 256
    entries in storage order, longer rows in pieces of 256 added in order, NaN pieces
    refolded with the stop at +Inf): every column of a 32-column product equals the
    one-column product of that column bit for bit, with +Inf, -Inf and NaN in B, in
    both dense layouts; sampled rows of <= 256 entries equal the oracle."""
    from gpugraphs import generators as gen
    A = gen.rmat(17, 16, seed=35, wkind=gen.W_U01_F32)
    n = A.n
    rp, cv, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    rng = np.random.default_rng(35)
    B = rng.random((n, 32), dtype=np.float32)
    cc = np.bincount(cv - 1, minlength=n)
    order = np.argsort(-cc, kind="stable")
    B[order[0], :8] = np.inf             # a hub column: many rows reach +Inf
    B[order[3:300:7], 8:16] = np.nan
    B[order[5:300:11], 16:24] = -np.inf
    Bd = dev(B)
    C = torch.zeros((n, 32), dtype=torch.float32, device="cuda")
    G.gpu_spmm_(C, A, Bd)
    Ch = host(C)
    for j in (0, 3, 9, 17, 30):
        for col in (Bd[:, j:j + 1].contiguous(), Bd[:, j].clone().view(n, 1)):
            y = torch.full((n, 1), -5.0, dtype=torch.float32, device="cuda")
            G.gpu_spmm_(y, A, col)
            yh = host(y)[:, 0]
            assert np.array_equal(np.isnan(yh), np.isnan(Ch[:, j]))
            fin = ~np.isnan(yh)
            assert np.array_equal(yh[fin].view(np.int32), Ch[fin, j].view(np.int32)), j
    deg = np.diff(rp)
    rows = np.unique(rng.integers(0, n, 800))
    short = rows[deg[rows] <= SEG_MM]
    srp = np.concatenate([[1], 1 + np.cumsum(deg[short])]).astype(np.int32)
    idx = np.concatenate([np.arange(rp[r] - 1, rp[r + 1] - 1) for r in short])
    Co = np.zeros((len(short), 32), np.float32)
    O.csr_spmm(len(short), srp, cv[idx], nz[idx], Co, B, layout=1)
    np.testing.assert_array_equal(Ch[short], Co)
