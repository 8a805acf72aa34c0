"""GPU parity of gpu_spmspv_ / gpu_spmv_rows_ / gpu_ewise_ / gpu_apply_ / gpu_reduce
against the CPU oracle.

Every comparison is bit for bit: SpMSpV and the row-list SpMV fold each row in storage
order on the GPU as in the oracle (a thread per row of at most 32 entries, a warp per
longer row that adds the present products in lane order), e-wise / apply are one
operation per entry, and the reduction follows the same chunk / butterfly order in both."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from oracle import oracle as O
from helpers import sprand_csr

pytestmark = pytest.mark.gpu

OPS = {O.ADD: G.GPUGraphs_add, O.MUL: G.GPUGraphs_mul, O.MIN: G.GPUGraphs_min,
       O.MAX: G.GPUGraphs_max, O.SECOND: G.GPUGraphs_second, O.ANY: G.GPUGraphs_any,
       O.BAND: G.GPUGraphs_band, O.BOR: G.GPUGraphs_bor, O.SECONDI: G.GPUGraphs_secondi,
       O.SAFE_ADD: G.GPUGraphs_safe_add, O.LOR: G.GPUGraphs_lor, O.LAND: G.GPUGraphs_land,
       O.MINUS: G.GPUGraphs_minus, O.RMINUS: G.GPUGraphs_rminus, O.FIRSTI: G.GPUGraphs_firsti,
       O.FIRST: G.GPUGraphs_first, O.PAIR: G.GPUGraphs_pair}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if np.issubdtype(a.dtype, np.floating):
        return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])
    return np.array_equal(a, b)


def rmat_csr(scale, ef, seed, wkind):
    n = 1 << scale
    s, d, w = O.gen_rmat(scale, ef * n, 0.57, 0.19, 0.19, seed, wkind)
    rp, cv, nz = O.coo_to_csr(n, s, d, w, symmetrize=True, drop_loops=True)
    return n, rp, cv, nz


def sparse_x(n, k, seed, dtype):
    rng = np.random.default_rng(seed)
    ind = np.sort(rng.choice(n, size=k, replace=False)).astype(np.int32) + 1
    if dtype == np.bool_:
        val = np.ones(k, np.bool_)
    elif np.issubdtype(dtype, np.integer):
        val = rng.integers(0, 200, k).astype(dtype)
    else:
        val = (rng.random(k) + 0.25).astype(dtype)
    return ind, val


def run_spmspv(m, n, rp, cv, nz, ind, val, y0, mul, add, accum):
    A = G.SparseGPUMatrixCSR(m, n, rp, cv, nz)
    y = dev(y0.copy())
    rows = G.gpu_spmspv_(y, A, G.SparseGPUVector(n, ind, val), mul=OPS[mul], add=OPS[add],
                         accum=OPS[accum])
    yr = y0.copy()
    rc, want = O.csr_spmspv(m, n, rp, cv, nz, yr, ind, val, mul=mul, add=add, accum=accum)
    assert rc == 0
    return host(y), host(rows), yr, want, A


SEMIRINGS = [
    # (value dtype, mul, add, accum)
    (np.float32, O.MUL, O.ADD, O.SECOND),
    (np.float32, O.ADD, O.MIN, O.MIN),
    (np.int32, O.SAFE_ADD, O.MIN, O.MIN),
    (np.int32, O.SECONDI, O.ANY, O.SECOND),
    (np.bool_, O.BAND, O.BOR, O.SECOND),
    (np.float64, O.MUL, O.ADD, O.ADD),
]


@pytest.mark.parametrize("dtype,mul,add,accum", SEMIRINGS)
@pytest.mark.parametrize("density", [0.001, 0.05, 1.0])
def test_spmspv_matches_oracle_on_rmat(dtype, mul, add, accum, density):
    wk = 2 if dtype == np.int32 else (0 if dtype == np.bool_ else 1)
    n, rp, cv, nz = rmat_csr(12, 16, 21, wk)
    nz = nz.astype(dtype)
    assert np.diff(rp).max() > 32  # long rows take the warp path
    k = max(1, int(density * n))
    ind, val = sparse_x(n, k, 22, dtype)
    ty = np.float32 if dtype == np.float32 else dtype
    if mul == O.SECONDI:
        val = val.astype(np.int32)
    y0 = np.zeros(n, ty) if accum == O.SECOND else np.full(n, 50, ty)
    got, rows, want_y, want_rows, _ = run_spmspv(n, n, rp, cv, nz, ind, val, y0, mul, add, accum)
    assert np.array_equal(rows, want_rows)
    assert same(got, want_y)


def test_spmspv_rectangular_special_values_and_reuse():
    m, n = 700, 1300
    rp, cv, nz, _ = sprand_csr(m, n, 0.04, np.float32, seed=31)
    ind, val = sparse_x(n, 200, 32, np.float32)
    val[3], val[10], val[11] = np.inf, np.nan, -np.inf
    A = G.SparseGPUMatrixCSR(m, n, rp, cv, nz)
    for trial in range(3):  # the bitmaps must be clean between calls
        sel = np.sort(np.random.default_rng(40 + trial).choice(len(ind), 60 + 50 * trial, replace=False))
        y = dev(np.zeros(m, np.float32))
        rows = G.gpu_spmspv_(y, A, G.SparseGPUVector(n, ind[sel], val[sel]))
        yr = np.zeros(m, np.float32)
        rc, want = O.csr_spmspv(m, n, rp, cv, nz, yr, ind[sel], val[sel])
        assert rc == 0
        assert np.array_equal(host(rows), want)
        assert same(host(y), yr)


def test_spmspv_allocating_form_and_empty_x():
    m, n = 300, 200
    rp, cv, nz, _ = sprand_csr(m, n, 0.03, np.float32, seed=33)
    A = G.SparseGPUMatrixCSR(m, n, rp, cv, nz)
    ind, val = sparse_x(n, 15, 34, np.float32)
    v = G.gpu_spmspv(A, G.SparseGPUVector(n, ind, val))
    yr = np.zeros(m, np.float32)
    rc, want = O.csr_spmspv(m, n, rp, cv, nz, yr, ind, val)
    assert np.array_equal(host(v.nzind), want)
    assert same(host(v.nzval), yr[want - 1])
    y = dev(np.full(m, 3.0, np.float32))
    rows = G.gpu_spmspv_(y, A, G.SparseGPUVector(n, np.zeros(0, np.int32), np.zeros(0, np.float32)))
    assert rows.numel() == 0 and (host(y) == 3.0).all()


def test_spmspv_errors():
    rp, cv, nz, _ = sprand_csr(50, 40, 0.1, np.float32, seed=35)
    A = G.SparseGPUMatrixCSR(50, 40, rp, cv, nz)
    y = dev(np.zeros(50, np.float32))
    with pytest.raises(G.DimensionMismatch):
        G.gpu_spmspv_(y, A, G.SparseGPUVector(41, [1], np.ones(1, np.float32)))
    with pytest.raises(G.DimensionMismatch):
        G.gpu_spmspv_(dev(np.zeros(49, np.float32)), A, G.SparseGPUVector(40, [1], np.ones(1, np.float32)))
    for bad in ([5, 3], [2, 2], [0], [41]):
        with pytest.raises(G.ArgumentError):
            G.gpu_spmspv_(y, A, G.SparseGPUVector(40, bad, np.ones(len(bad), np.float32)))
    assert (host(y) == 0).all()
    # after rejected calls the next call still sees clean bitmaps
    rows = G.gpu_spmspv_(y, A, G.SparseGPUVector(40, [7], np.ones(1, np.float32)))
    yr = np.zeros(50, np.float32)
    _, want = O.csr_spmspv(50, 40, rp, cv, nz, yr, np.array([7], np.int32), np.ones(1, np.float32))
    assert np.array_equal(host(rows), want) and same(host(y), yr)
    with pytest.raises(G.ArgumentError):
        G.gpu_spmspv_(y, G.SparseGPUMatrixSELL(A), G.SparseGPUVector(40, [1], np.ones(1, np.float32)))


@pytest.mark.parametrize("dtype,mul,add", [(np.float32, O.MUL, O.ADD), (np.int32, O.SAFE_ADD, O.MIN),
                                           (np.bool_, O.BAND, O.BOR)])
def test_spmv_rows_matches_oracle(dtype, mul, add):
    wk = 2 if dtype == np.int32 else (0 if dtype == np.bool_ else 1)
    n, rp, cv, nz = rmat_csr(11, 16, 23, wk)
    nz = nz.astype(dtype)
    rng = np.random.default_rng(24)
    x = (rng.random(n) + 0.5).astype(dtype) if dtype == np.float32 else rng.integers(0, 2 if dtype == np.bool_ else 100, n).astype(dtype)
    rows = (rng.choice(n, 300, replace=False) + 1).astype(np.int32)
    rows = np.concatenate([rows, np.argsort(-np.diff(rp))[:20].astype(np.int32) + 1])
    rows = np.unique(rows)[rng.permutation(len(np.unique(rows)))].astype(np.int32)
    A = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    y0 = np.zeros(n, dtype)
    y = dev(y0)
    G.gpu_spmv_rows_(y, A, dev(x), dev(rows), mul=OPS[mul], add=OPS[add])
    yr = y0.copy()
    assert O.csr_spmv_rows(n, rp, cv, nz, yr, x, rows, mul=mul, add=add) == 0
    assert same(host(y), yr)
    with pytest.raises(G.BoundsError):
        G.gpu_spmv_rows_(y, A, dev(x), dev(np.array([1, n + 1], np.int32)), mul=OPS[mul], add=OPS[add])


EW = [(O.ADD, np.float32), (O.MUL, np.float32), (O.MIN, np.float32), (O.MAX, np.float64),
      (O.MINUS, np.float32), (O.RMINUS, np.int32), (O.ADD, np.int32), (O.MIN, np.int64),
      (O.SAFE_ADD, np.int32), (O.LOR, np.bool_), (O.LAND, np.bool_), (O.ANY, np.int32),
      (O.PAIR, np.float32), (O.SECOND, np.float32), (O.SECONDI, np.int64), (O.FIRSTI, np.int64),
      (O.MIN, np.float64)]


def ew_input(dtype, n, seed):
    rng = np.random.default_rng(seed)
    if dtype == np.bool_:
        return rng.integers(0, 2, n).astype(np.bool_)
    if np.issubdtype(dtype, np.integer):
        v = rng.integers(-1000, 1000, n).astype(dtype)
        v[:4] = [np.iinfo(dtype).max, np.iinfo(dtype).min, 0, -1]
        return v
    v = (rng.random(n) * 10 - 5).astype(dtype)
    v[:6] = [np.nan, np.inf, -np.inf, 0.0, -0.0, 1e-30]
    return v


@pytest.mark.parametrize("op,dtype", EW)
def test_ewise_matches_oracle(op, dtype):
    n = 100_003
    x, y = ew_input(dtype, n, 1), ew_input(dtype, n, 2)
    mask = (np.arange(n) % 3 != 0)
    for msk in (None, mask):
        z0 = ew_input(dtype, n, 3)
        z = dev(z0)
        G.gpu_ewise_(z, dev(x), dev(y), OPS[op], mask=None if msk is None else dev(msk))
        zr = z0.copy()
        assert O.ewise(op, zr, x, y, mask=msk) == 0
        assert same(host(z), zr)


def test_ewise_index_operator_and_mixed_types():
    n = 5000
    x = ew_input(np.int32, n, 4)
    y = ew_input(np.float32, n, 5)
    z = dev(np.zeros(n, np.float32))
    G.gpu_ewise_(z, dev(x), dev(y), G.GPUGraphs_add)
    zr = np.zeros(n, np.float32)
    assert O.ewise(O.ADD, zr, x, y) == 0
    assert same(host(z), zr)
    zi = dev(np.zeros(n, np.int64))
    G.gpu_ewise_(zi, dev(x), dev(x), G.GPUGraphs_firsti)
    assert (host(zi) == np.arange(1, n + 1)).all()
    with pytest.raises(G.ArgumentError):
        G.gpu_ewise_(dev(np.zeros(n, np.int32)), dev(x), dev(y), G.GPUGraphs_add)
    with pytest.raises(G.UnsupportedError):
        G.gpu_ewise_(dev(np.zeros(n, np.float32)), dev(y), dev(y), G.GPUGraphs_bor)


@pytest.mark.parametrize("op,dtype,first", [(O.MINUS, np.float32, False), (O.MINUS, np.float32, True),
                                            (O.MIN, np.int32, False), (O.SAFE_ADD, np.int32, True),
                                            (O.LOR, np.bool_, False), (O.MUL, np.float64, True)])
def test_apply_matches_oracle(op, dtype, first):
    n = 70_001
    x = ew_input(dtype, n, 6)
    s = np.asarray(ew_input(dtype, 8, 7)[7]).astype(dtype)[()]
    mask = np.arange(n) % 5 != 1
    z0 = ew_input(dtype, n, 8)
    z = dev(z0)
    G.gpu_apply_(z, dev(x), s, OPS[op], bind_first=first, s_dtype=dtype, mask=dev(mask))
    zr = z0.copy()
    assert O.apply_scalar(op, zr, x, np.asarray(s, dtype=dtype)[()], s_first=first, mask=mask) == 0
    assert same(host(z), zr)


@pytest.mark.parametrize("add,dtype,n", [(O.ADD, np.float32, 1), (O.ADD, np.float32, 8191),
                                         (O.ADD, np.float32, 3_000_017), (O.MUL, np.float64, 100_000),
                                         (O.ADD, np.int32, 1_000_003), (O.MIN, np.float32, 500_000),
                                         (O.MAX, np.int64, 77_777), (O.LOR, np.bool_, 123_457),
                                         (O.ANY, np.int32, 1000), (O.ADD, np.float32, 0)])
def test_reduce_matches_oracle(add, dtype, n):
    rng = np.random.default_rng(9)
    if dtype == np.bool_:
        x = np.zeros(n, np.bool_)
        if n > 1000:
            x[n - 3] = True
    elif add == O.MUL:
        x = (1.0 + (rng.random(n) - 0.5) * 1e-5).astype(dtype)
    elif np.issubdtype(dtype, np.integer):
        x = rng.integers(-2**30, 2**30, n).astype(dtype)
    else:
        x = rng.random(n).astype(dtype)
    got = G.gpu_reduce(dev(x) if n else torch.zeros(0, dtype=torch.float32, device="cuda"), OPS[add])
    rc, want = O.reduce(add, x)
    assert rc == 0
    assert same(np.array([got]), np.array([want]))


def test_reduce_multi_pass_order():
    # more than 8192 chunks: the chunk totals are reduced in a second pass
    n = 8192 * 8192 + 12_345
    x = O.gen_uniform_f32(n, 77)
    got = G.gpu_reduce(dev(x), G.GPUGraphs_add)
    rc, want = O.reduce(O.ADD, x)
    assert rc == 0 and got == want
    assert abs(float(got) - x.astype(np.float64).sum()) <= 1e-5 * x.astype(np.float64).sum()


@pytest.mark.parametrize("mul,add", [(O.MUL, O.ADD), (O.ADD, O.MIN)])
def test_spmspv_hub_rows_span_several_pieces(mul, add):
    # rows of 20000 and 5000 entries (pieces of 2048), an absorbing +Inf inside a hub
    m, n = 300, 20000
    rng = np.random.default_rng(50)
    D = sp.random(m, n, density=0.002, format="lil", random_state=rng, dtype=np.float64)
    D[5, :] = rng.random(n) + 0.1
    D[7, rng.choice(n, 5000, replace=False)] = 1.0
    A = sp.csr_matrix(D).astype(np.float32)
    A.sort_indices()
    rp, cv, nz = (A.indptr + 1).astype(np.int32), (A.indices + 1).astype(np.int32), A.data.copy()
    for density, special in ((0.3, False), (0.05, True), (1.0, False)):
        ind, val = sparse_x(n, int(density * n), 51, np.float32)
        if special:
            val[len(val) // 2] = np.inf
            val[len(val) // 2 + 3] = np.nan
        y0 = np.zeros(m, np.float32)
        got, rows, want_y, want_rows, _ = run_spmspv(m, n, rp, cv, nz, ind, val, y0, mul, add, O.SECOND)
        assert np.array_equal(rows, want_rows)
        assert same(got, want_y)


def test_spmspv_hub_columns_pushed_by_the_grid():
    # columns of 10000 and 6000 entries (longer than one warp's push share)
    m, n = 10000, 500
    rng = np.random.default_rng(60)
    D = sp.random(m, n, density=0.004, format="lil", random_state=rng, dtype=np.float64)
    D[:, 3] = rng.random((m, 1)) + 0.1
    D[rng.choice(m, 6000, replace=False), 11] = 2.0
    A = sp.csr_matrix(D).astype(np.float32)
    A.sort_indices()
    rp, cv, nz = (A.indptr + 1).astype(np.int32), (A.indices + 1).astype(np.int32), A.data.copy()
    ind = np.array([3, 4, 11, 12, 100, 499], np.int32) + 1
    val = (rng.random(len(ind)) + 0.5).astype(np.float32)
    for mul, add in ((O.MUL, O.ADD), (O.ADD, O.MIN)):
        got, rows, want_y, want_rows, _ = run_spmspv(m, n, rp, cv, nz, ind, val, np.zeros(m, np.float32),
                                                     mul, add, O.SECOND)
        assert np.array_equal(rows, want_rows)
        assert same(got, want_y)
