"""GPU parity of the CSC SpMV (gpu_spmv_ on SparseGPUMatrixCSC, i.e. gg_spmv_t on the
CSR storage of the transpose) and of derived-copy invalidation after value writes.

Oracle: the CSR of the CSC matrix with rows in ascending column order, folded by the
oracle's CSR SpMV.  Integer, Bool and min/max semirings and rows of at most 32 entries
are compared bit for bit; Float32 plus-times rows longer than 32 entries (reduced in
parallel) within rtol 1e-5 of the FP64 product."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def csr_arrays(B):
    B = sp.csr_matrix(B)
    B.sort_indices()
    return (B.indptr + 1).astype(np.int32), (B.indices + 1).astype(np.int32), np.ascontiguousarray(B.data)


def rmat(scale, seed, wkind):
    n = 1 << scale
    s, d, w = O.gen_rmat(scale, 16 * n, 0.57, 0.19, 0.19, seed, wkind)
    rp, cv, nz = O.coo_to_csr(n, s, d, w, symmetrize=False, drop_loops=False)
    return sp.csr_matrix((nz, cv - 1, rp - 1), shape=(n, n))


def check_close(got, want, rp, B64, x):
    short = np.diff(rp) <= 32
    assert np.array_equal(got[short], want[short])
    ref = B64 @ x.astype(np.float64)
    assert np.allclose(got, ref, rtol=RTOL, atol=1e-6)


@pytest.mark.parametrize("m,n", [(900, 1300), (1 << 12, 1 << 12)])
def test_csc_plus_times_float32(m, n):
    rng = np.random.default_rng(3)
    B = sp.random(m, n, density=0.01, format="csc", random_state=rng, dtype=np.float64).astype(np.float32)
    if m == n:
        B = rmat(12, 5, 1).tocsc().astype(np.float32)
    A = G.SparseGPUMatrixCSC.from_scipy(B)
    assert A.size() == B.shape
    x = rng.random(B.shape[1]).astype(np.float32)
    y = dev(np.zeros(B.shape[0], np.float32))
    G.gpu_spmv_(y, A, dev(x))
    rp, cv, nz = csr_arrays(B)
    want = np.zeros(B.shape[0], np.float32)
    assert O.csr_spmv(B.shape[0], B.shape[1], rp, cv, nz, want, x) == 0
    check_close(host(y), want, rp, B.astype(np.float64), x)


def test_csc_large_plus_times_uses_the_copy_and_stays_close():
    B = rmat(17, 9, 1).tocsc().astype(np.float32)
    A = G.SparseGPUMatrixCSC.from_scipy(B)
    x = O.gen_uniform_f32(B.shape[1], 10)
    y = dev(np.zeros(B.shape[0], np.float32))
    G.gpu_spmv_(y, A, dev(x))
    rp, cv, nz = csr_arrays(B)
    want = np.zeros(B.shape[0], np.float32)
    assert O.csr_spmv(B.shape[0], B.shape[1], rp, cv, nz, want, x) == 0
    check_close(host(y), want, rp, B.astype(np.float64), x)


@pytest.mark.parametrize("dtype,mul,add,accum,gm,ga,gc", [
    (np.int32, O.SAFE_ADD, O.MIN, O.MIN, G.GPUGraphs_safe_add, G.GPUGraphs_min, G.GPUGraphs_min),
    (np.bool_, O.BAND, O.BOR, O.SECOND, G.GPUGraphs_band, G.GPUGraphs_bor, G.GPUGraphs_second),
    (np.int32, O.SECONDI, O.ANY, O.SECOND, G.GPUGraphs_secondi, G.GPUGraphs_any, G.GPUGraphs_second),
    (np.float32, O.ADD, O.MIN, O.MIN, G.GPUGraphs_add, G.GPUGraphs_min, G.GPUGraphs_min),
])
def test_csc_semirings_mask_and_range_exact(dtype, mul, add, accum, gm, ga, gc):
    B = rmat(11, 7, 2 if dtype == np.int32 else (0 if dtype == np.bool_ else 1)).tocsc()
    B.data = B.data.astype(dtype)
    m, n = B.shape
    rng = np.random.default_rng(8)
    if dtype == np.bool_:
        x = rng.integers(0, 2, n).astype(np.bool_)
    elif dtype == np.int32:
        x = rng.integers(0, 300, n).astype(np.int32)
    else:
        x = (rng.random(n) * 10).astype(np.float32)
    A = G.SparseGPUMatrixCSC.from_scipy(B, dtype=dtype)
    rp, cv, nz = csr_arrays(B)
    nz = nz.astype(dtype)
    mask = (rng.random(m) < 0.6).astype(np.int32)
    for kw, okw in (({}, {}), ({"mask": mask}, {"mask": mask}), ({"range": (100, 1500)}, {"range_": (100, 1500)})):
        y0 = np.full(m, 7, dtype) if dtype != np.bool_ else np.zeros(m, np.bool_)
        y = dev(y0)
        gkw = dict(kw)
        if "mask" in gkw:
            gkw["mask"] = dev(gkw["mask"])
        G.gpu_spmv_(y, A, dev(x), mul=gm, add=ga, accum=gc, **gkw)
        want = y0.copy()
        assert O.csr_spmv(m, n, rp, cv, nz, want, x, mul=mul, add=add, accum=accum, **okw) == 0
        assert np.array_equal(host(y), want)


def test_csc_dimension_checks():
    B = sp.random(30, 20, density=0.2, format="csc", random_state=np.random.default_rng(1), dtype=np.float32)
    A = G.SparseGPUMatrixCSC.from_scipy(B)
    with pytest.raises(G.DimensionMismatch):
        G.gpu_spmv_(dev(np.zeros(30, np.float32)), A, dev(np.zeros(21, np.float32)))
    with pytest.raises(G.DimensionMismatch):
        G.gpu_spmv_(dev(np.zeros(20, np.float32)), A, dev(np.zeros(20, np.float32)))
    with pytest.raises(G.ArgumentError):
        G.SparseGPUMatrixCSC(30, 20, np.ones(20, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    with pytest.raises(G.ArgumentError):
        G.SparseGPUMatrixCSC(3, 2, np.array([1, 2, 3], np.int32), np.array([1, 4], np.int32),
                             np.ones(2, np.float32))
    with pytest.raises(G.ArgumentError):
        G.gpu_spmm_(dev(np.zeros((30, 2), np.float32)), A, dev(np.zeros((20, 2), np.float32)))


def test_value_writes_drop_derived_copies():
    # m >= 65536: plus-times runs on the SELL-32 copy; a write must not leave it stale
    B = rmat(16, 12, 1).astype(np.float32)
    rp, cv, nz = csr_arrays(B)
    n = B.shape[0]
    A = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    x = O.gen_uniform_f32(n, 13)
    y = dev(np.zeros(n, np.float32))
    G.gpu_spmv_(y, A, dev(x))
    r = int(np.argmax(np.diff(rp) == 3)) + 1
    j = int(cv[rp[r - 1] - 1])
    A[r, j] = 1000.0
    nz2 = nz.copy()
    nz2[rp[r - 1] - 1] = 1000.0
    G.gpu_spmv_(y, A, dev(x))
    want = np.zeros(n, np.float32)
    assert O.csr_spmv(n, n, rp, cv, nz2, want, x) == 0
    got = host(y)
    assert got[r - 1] == want[r - 1]
    short = np.diff(rp) <= 32
    assert np.array_equal(got[short], want[short])
    # the same through the transposed copy of a CSC matrix
    C = G.SparseGPUMatrixCSC(n, n, rp, cv, nz)  # the transpose of B, as CSC
    yt = dev(np.zeros(n, np.float32))
    G.gpu_spmv_(yt, C, dev(x))
    C.nzval[rp[r - 1] - 1] = 1000.0
    C.values_changed()
    G.gpu_spmv_(yt, C, dev(x))
    Bt = sp.csr_matrix((nz2, cv - 1, rp - 1), shape=(n, n)).T.tocsr()
    rpt, cvt, nzt = csr_arrays(Bt)
    want_t = np.zeros(n, np.float32)
    assert O.csr_spmv(n, n, rpt, cvt, nzt, want_t, x) == 0
    got_t = host(yt)
    st = np.diff(rpt) <= 32
    assert np.array_equal(got_t[st], want_t[st])
    assert np.allclose(got_t, Bt.astype(np.float64) @ x.astype(np.float64), rtol=RTOL, atol=1e-6)
