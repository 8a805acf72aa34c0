"""CPU checks of the oracle's SpMSpV, row-list SpMV, e-wise, apply and reduce.

The reference has no tests for these paths (src/spmspv.jl was never finished and
e_wise_ops.jl / map_and_reduce.jl are empty), so they are pinned by their defining
properties: SpMSpV with every entry of x present equals the oracle's dense SpMV (itself
pinned by the reference's golden vectors) on every non-empty row; plus-times equals
scipy's FP64 product on the rows reached; min-plus equals a dense restatement; e-wise /
apply match numpy; exact reductions match numpy and float sums stay within rounding of
an FP64 sum."""
import numpy as np
import pytest

from helpers import sprand_csr
from oracle import oracle as O


def sparse_x(n, k, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    ind = np.sort(rng.choice(n, size=k, replace=False)).astype(np.int32) + 1
    val = rng.random(k).astype(dtype) + 0.5
    return ind, val


def test_spmspv_full_x_equals_dense_spmv():
    m, n = 120, 90
    rp, cv, nz, A = sprand_csr(m, n, 0.05, np.float32, seed=3)
    x = (np.random.default_rng(4).random(n).astype(np.float32) + 0.25)
    y1 = np.full(m, -7.0, np.float32)
    rc, rows = O.csr_spmspv(m, n, rp, cv, nz, y1, np.arange(1, n + 1, dtype=np.int32), x)
    assert rc == 0
    y2 = np.full(m, -7.0, np.float32)
    assert O.csr_spmv(m, n, rp, cv, nz, y2, x) == 0
    nonempty = np.flatnonzero(np.diff(rp) > 0) + 1
    assert np.array_equal(rows, nonempty)
    assert np.array_equal(y1[rows - 1], y2[rows - 1])
    empty = np.diff(rp) == 0
    assert (y1[empty] == -7.0).all()


def test_spmspv_plus_times_matches_scipy():
    m, n = 300, 250
    rp, cv, nz, A = sprand_csr(m, n, 0.03, np.float64, seed=5)
    ind, val = sparse_x(n, 25, 6)
    y = np.zeros(m)
    rc, rows = O.csr_spmspv(m, n, rp, cv, nz, y, ind, val)
    assert rc == 0
    sub = A[:, ind - 1]
    want_rows = np.flatnonzero(np.diff(sub.tocsr().indptr) > 0) + 1
    assert np.array_equal(rows, want_rows)
    ref = sub @ val
    np.testing.assert_allclose(y[rows - 1], ref[rows - 1], rtol=1e-12)
    others = np.setdiff1d(np.arange(1, m + 1), rows)
    assert (y[others - 1] == 0).all()


def test_spmspv_min_plus_matches_dense():
    m, n = 80, 70
    rp, cv, nz, A = sprand_csr(m, n, 0.1, np.int32, seed=7,
                               values=lambda rng, k: rng.integers(1, 50, k).astype(np.float64))
    ind, _ = sparse_x(n, 12, 8)
    val = np.random.default_rng(9).integers(0, 100, len(ind)).astype(np.int32)
    y = np.full(m, 1000, np.int32)
    rc, rows = O.csr_spmspv(m, n, rp, cv, nz, y, ind, val, mul=O.ADD, add=O.MIN, accum=O.MIN)
    assert rc == 0
    D = A.toarray()
    xs = dict(zip(ind - 1, val))
    for i in range(m):
        terms = [D[i, j] + xs[j] for j in cv[rp[i] - 1:rp[i + 1] - 1] - 1 if j in xs]
        if terms:
            assert i + 1 in rows
            assert y[i] == min(1000, min(terms))
        else:
            assert i + 1 not in rows and y[i] == 1000


def test_spmspv_rejects_bad_indices():
    rp, cv, nz, _ = sprand_csr(10, 10, 0.3, np.float32, seed=1)
    y = np.zeros(10, np.float32)
    for ind in ([3, 2], [1, 1], [0, 4], [4, 11]):
        rc, _ = O.csr_spmspv(10, 10, rp, cv, nz, y, np.array(ind, np.int32),
                             np.ones(len(ind), np.float32))
        assert rc == O.ARG
    assert (y == 0).all()


def test_spmv_rows_equals_dense_rows():
    m, n = 150, 140
    rp, cv, nz, _ = sprand_csr(m, n, 0.05, np.float32, seed=11)
    x = np.random.default_rng(12).random(n).astype(np.float32)
    rows = np.array([150, 3, 77, 1, 42], np.int32)
    y1 = np.full(m, 2.0, np.float32)
    assert O.csr_spmv_rows(m, rp, cv, nz, y1, x, rows) == 0
    y2 = np.full(m, 2.0, np.float32)
    assert O.csr_spmv(m, n, rp, cv, nz, y2, x) == 0
    assert np.array_equal(y1[rows - 1], y2[rows - 1])
    rest = np.setdiff1d(np.arange(m), rows - 1)
    assert (y1[rest] == 2.0).all()
    assert O.csr_spmv_rows(m, rp, cv, nz, y1, x, np.array([0, 2], np.int32)) == O.ARG


@pytest.mark.parametrize("op,fn", [(O.ADD, np.add), (O.MUL, np.multiply), (O.MIN, np.minimum),
                                   (O.MAX, np.maximum), (O.MINUS, np.subtract)])
def test_ewise_float32_matches_numpy(op, fn):
    rng = np.random.default_rng(13)
    x = (rng.random(1000) * 4 - 2).astype(np.float32)
    y = (rng.random(1000) * 4 - 2).astype(np.float32)
    x[5], y[9] = np.nan, np.inf
    z = np.zeros(1000, np.float32)
    assert O.ewise(op, z, x, y) == 0
    want = fn(x, y)
    assert np.array_equal(np.isnan(z), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.array_equal(z[ok], want[ok])


def test_ewise_int32_wraps_and_masks():
    x = np.array([2**31 - 1, 5, -3, 7], np.int32)
    y = np.array([1, 6, -4, 1], np.int32)
    z = np.full(4, 9, np.int32)
    mask = np.array([1, 1, 0, 1], np.bool_)
    assert O.ewise(O.ADD, z, x, y, mask=mask) == 0
    assert z.tolist() == [-2**31, 11, 9, 8]
    zb = np.zeros(4, np.bool_)
    assert O.ewise(O.LOR, zb, np.array([0, 1, 0, 1], np.bool_), np.array([0, 0, 1, 1], np.bool_)) == 0
    assert zb.tolist() == [False, True, True, True]
    zi = np.zeros(4, np.int64)
    assert O.ewise(O.FIRSTI, zi, x, y) == 0
    assert zi.tolist() == [1, 2, 3, 4]
    assert O.ewise(O.ADD, np.zeros(4, np.int32), x, y.astype(np.float32)) == O.TYPE
    assert O.ewise(O.BOR, np.zeros(4, np.float32), x.astype(np.float32), y.astype(np.float32)) == O.UNSUPPORTED


def test_apply_scalar_both_sides():
    x = np.array([1.5, -2.0, 3.25], np.float32)
    z = np.zeros(3, np.float32)
    assert O.apply_scalar(O.MINUS, z, x, np.float32(1.0)) == 0
    assert z.tolist() == [0.5, -3.0, 2.25]
    assert O.apply_scalar(O.MINUS, z, x, np.float32(1.0), s_first=True) == 0
    assert z.tolist() == [-0.5, 3.0, -2.25]
    assert O.apply_scalar(O.MIN, z, x, np.float32(0.0), mask=np.array([1, 0, 1], np.int32)) == 0
    assert z.tolist() == [0.0, 3.0, 0.0]


def test_reduce_exact_monoids_and_float_sum():
    rng = np.random.default_rng(14)
    xi = rng.integers(-2**31, 2**31 - 1, 3 * 8192 + 17, dtype=np.int64).astype(np.int32)
    rc, s = O.reduce(O.ADD, xi)
    wrapped = (int(xi.astype(np.int64).sum()) + 2**31) % 2**32 - 2**31
    assert rc == 0 and int(s) == wrapped
    assert O.reduce(O.MIN, xi)[1] == xi.min()
    assert O.reduce(O.MAX, xi)[1] == xi.max()
    xf = rng.random(5 * 8192 + 3).astype(np.float32)
    rc, sf = O.reduce(O.ADD, xf)
    assert rc == 0
    assert abs(float(sf) - xf.astype(np.float64).sum()) <= 1e-5 * xf.astype(np.float64).sum()
    assert O.reduce(O.ADD, np.zeros(0, np.float32))[1] == 0.0
    assert O.reduce(O.MIN, np.zeros(0, np.int32))[1] == np.iinfo(np.int32).max
    xb = np.zeros(100, np.bool_)
    assert not O.reduce(O.LOR, xb)[1]
    xb[37] = True
    assert O.reduce(O.LOR, xb)[1] and not O.reduce(O.LAND, xb)[1]
    assert O.reduce(O.BOR, xb)[0] == 0
    assert O.reduce(O.ADD, xb)[0] == O.UNSUPPORTED


def _reduce_order_py(x):
    """The library's reduction order restated with numpy Float32 scalars: chunks of 8192,
    thread t of 256 folds t, t+256, ... left to right, xor butterflies over each warp's 32
    lanes (lane l takes v[l] + v[l ^ o]) and over the 8 warp totals, chunk totals again."""
    vals = [np.float32(v) for v in x]
    while len(vals) > 1 or not vals:
        if not vals:
            return np.float32(0)
        out = []
        for c0 in range(0, len(vals), 8192):
            th = []
            for t in range(256):
                acc = np.float32(0)
                for u in range(32):
                    i = c0 + t + 256 * u
                    if i < len(vals):
                        acc = np.float32(acc + vals[i])
                th.append(acc)
            tot = []
            for w in range(8):
                v = th[32 * w:32 * w + 32]
                for o in (16, 8, 4, 2, 1):
                    v = [np.float32(v[l] + v[l ^ o]) for l in range(32)]
                tot.append(v[0])
            v = tot + [np.float32(0)] * 24
            for o in (16, 8, 4, 2, 1):
                v = [np.float32(v[l] + v[l ^ o]) for l in range(32)]
            out.append(v[0])
        vals = out
        if len(vals) == 1:
            break
    return vals[0]


def test_reduce_order_pinned_by_an_independent_restatement():
    rng = np.random.default_rng(21)
    for n in (1, 255, 8192, 8193, 20000):
        x = (rng.random(n) * 2 - 0.5).astype(np.float32)
        rc, got = O.reduce(O.ADD, x)
        assert rc == 0
        assert np.float32(got).tobytes() == _reduce_order_py(x).tobytes(), n
