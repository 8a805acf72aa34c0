"""Plus-times Float32 SpMV whose hub rows are folded from shared-memory column windows.

With the "hub_windows" SELL-32 variant, a large skewed matrix's sorted SELL-32 layout
takes its longest rows (more than 128 entries, in groups dense enough) out of the
SELL-32 kernel and folds them window by window from x values staged in shared memory
(gg_spmv_hub.cu).  Checked here:
the path is taken (gg_spmv_hub_rows), every row of at most 128 entries still equals
the oracle bit for bit, every row is within rtol 1e-5 of the FP64 product, repeated
calls give identical bits, rows with repeated columns and user-built SELL-32
handles work, and the CSR handle keeps the reference's stop at +Inf
(csr_spmv_kernel!, src/spmv/CSR.jl:47-52) on hub rows."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from gpugraphs import tuning
from oracle import oracle as O
from helpers import csr_from_scipy

pytestmark = pytest.mark.gpu
RTOL = 1e-5
SELL_CHUNK = 128


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def hub_windows(A):
    """Select the hub-window variant on a CSR handle (its SELL-32 copy sorted by row
    length) or on a SELL-32 handle."""
    if isinstance(A, G.SparseGPUMatrixCSR):
        tuning.apply(A, {"spmv_kernel": "sell", "slice_size": 32, "sigma": A.m,
                         "sell_variant": "hub_windows"})
    else:
        tuning.apply(A, {"sell_variant": "hub_windows"})


def check_against_oracle(A, x, yh, sell=None):
    rowptr, colval, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    n = A.n
    yo = np.zeros(n, np.float32)
    assert O.csr_spmv(A.m, n, rowptr, colval, nz, yo, x) == O.OK
    deg = np.diff(rowptr)
    short = deg <= SELL_CHUNK
    np.testing.assert_array_equal(yh[short], yo[short])
    ref = A.to_scipy().astype(np.float64) @ x.astype(np.float64)
    np.testing.assert_allclose(yh, ref, rtol=RTOL, atol=1e-6)
    return deg


@pytest.mark.parametrize("scale,seed", [(17, 5), (18, 6)])
def test_hub_rows_from_windows_rmat(scale, seed):
    A = gen.rmat(scale, 16, seed=seed, wkind=gen.W_U01_F32)
    n = A.n
    hub_windows(A)
    x = np.random.default_rng(seed).random(n, dtype=np.float32)
    outs = []
    for _ in range(2):
        y = torch.full((n,), -3.0, dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, A, dev(x))
        outs.append(host(y))
    hub = G.spmv_hub_rows(A)
    deg = check_against_oracle(A, x, outs[0])
    assert G.spmv_hub_rows(gen.rmat(12, 16, seed=seed, wkind=gen.W_U01_F32)) == 0
    assert G.spmv_layout(A) == "sell"
    # the hub rows are the longest rows, all above 128 entries
    assert hub >= 32 and hub % 32 == 0
    assert hub <= int((deg > SELL_CHUNK).sum())
    assert np.array_equal(outs[0].view(np.int32), outs[1].view(np.int32))
    # the register kernel for every row: the same bits on short rows, rounding on hub rows
    tuning.apply(A, {"sell_variant": "registers"})
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, A, dev(x))
    y2 = host(y)
    short = deg <= SELL_CHUNK
    np.testing.assert_array_equal(y2[short], outs[0][short])
    np.testing.assert_allclose(y2, outs[0], rtol=2 * RTOL, atol=1e-6)


def test_hub_rows_with_repeated_columns():
    """Rows that repeat a column more often than a window is wide (the CSR handle
    keeps duplicates, as the reference's constructor does)."""
    m = 70000
    rng = np.random.default_rng(12)
    rows, cols = [], []
    for r in range(96):  # hub rows with random columns
        d = int(rng.integers(6500, 8000))
        rows.append(np.full(d, r))
        cols.append(rng.choice(m, d, replace=False))
    rows.append(np.full(12000, 0))  # row 0: column 6 repeated 12000 times
    cols.append(np.full(12000, 5))
    # skewed columns (80% of the light entries on 500 columns), so the layout ranks
    # columns by frequency, which the window path needs
    light = np.where(rng.random(8 * m) < 0.8, rng.integers(0, 500, size=8 * m),
                     rng.integers(0, m, size=8 * m))
    rows.append(np.repeat(np.arange(m), 8))
    cols.append(light)
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    order = np.lexsort((np.arange(len(r)), r))  # row order, generation order in a row
    r, c = r[order], c[order]
    v = rng.random(len(r)).astype(np.float32)
    rowptr = np.concatenate([[1], 1 + np.cumsum(np.bincount(r, minlength=m))]).astype(np.int32)
    A = G.SparseGPUMatrixCSR(m, m, rowptr, (c + 1).astype(np.int32), v)
    hub_windows(A)
    x = rng.random(m, dtype=np.float32)
    y = torch.zeros(m, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, A, dev(x))
    yh = host(y)
    assert G.spmv_hub_rows(A) > 0
    yo = np.zeros(m, np.float32)
    assert O.csr_spmv(m, m, rowptr, (c + 1).astype(np.int32), v, yo, x) == O.OK
    deg = np.diff(rowptr)
    np.testing.assert_array_equal(yh[deg <= SELL_CHUNK], yo[deg <= SELL_CHUNK])
    ref = sp.csr_matrix((v.astype(np.float64), c, rowptr - 1), shape=(m, m)) @ x.astype(np.float64)
    np.testing.assert_allclose(yh, ref, rtol=RTOL, atol=1e-6)


def test_hub_rows_on_a_sell_handle():
    """A user-built SELL-32 handle with rows sorted by length (sigma = m) takes the same
    path; SELL semantics (no early exit, src/spmv/SELL.jl:31-63)."""
    A = gen.rmat(17, 16, seed=8, wkind=gen.W_U01_F32)
    n = A.n
    S = G.SparseGPUMatrixSELL(A, slice_size=32, sigma=n)
    hub_windows(S)
    x = np.random.default_rng(8).random(n, dtype=np.float32)
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, S, dev(x))
    yh = host(y)
    assert G.spmv_hub_rows(S) > 0
    check_against_oracle(A, x, yh)


def test_hub_rows_keep_the_absorb_stop():
    """+Inf in x on a hub column, NaN / -Inf on others: hub rows get the oracle's
    NaN / +Inf / -Inf pattern (the NaN rows of the fast fold are folded again in storage
    order with the stop at +Inf) and finite rows stay within rtol 1e-5."""
    A = gen.rmat(17, 16, seed=33, wkind=gen.W_U01_F32)
    n = A.n
    hub_windows(A)
    rowptr, colval, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    cc = np.bincount(colval - 1, minlength=n)
    order = np.argsort(-cc, kind="stable")
    x = np.random.default_rng(33).random(n, dtype=np.float32)
    x[order[3]] = np.inf
    x[order[40000:40400:7]] = np.nan
    x[order[50000:50400:5]] = -np.inf
    x[order[2000:2100:9]] = np.inf
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, A, dev(x))
    yh = host(y)
    hub = G.spmv_hub_rows(A)
    assert hub > 0
    yo = np.zeros(n, np.float32)
    assert O.csr_spmv(n, n, rowptr, colval, nz, yo, x) == O.OK
    with np.errstate(invalid="ignore"):
        ref = A.to_scipy().astype(np.float64) @ x.astype(np.float64)
    deg = np.diff(rowptr)
    long_ = deg > SELL_CHUNK
    stop = np.isposinf(yo) & np.isnan(ref)
    assert (stop & long_).sum() >= 1
    for f in (np.isnan, np.isposinf, np.isneginf):
        assert np.array_equal(f(yh), f(yo)), f.__name__
    np.testing.assert_array_equal(yh[stop], yo[stop])
    np.testing.assert_array_equal(yh[~long_], yo[~long_])
    fin = np.isfinite(yo)
    np.testing.assert_allclose(yh[fin], ref[fin], rtol=RTOL, atol=1e-6)
