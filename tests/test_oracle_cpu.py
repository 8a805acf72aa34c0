"""Pins the CPU oracle against the reference's golden vectors and test oracles
(no GPU needed).  Each test names the reference test it restates."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from helpers import (bfs_levels_scipy, golden_graphs, golden_json, sprand_csr,
                     undirected_csr, csr_from_scipy)

I32MAX = np.iinfo(np.int32).max


def test_sell_layout_golden():
    """test/structs.jl:176-207: SELL layout of the 4x4 known answer."""
    g = golden_json("sell_4x4.json")
    A = sp.csr_matrix(np.array(g["dense"], np.float32))
    rowptr, colval, nzval = csr_from_scipy(A)
    S = O.sell_build(4, rowptr, colval, nzval, slice_size=32)
    assert S["slice_size"] == 4 and S["nslices"] == 1
    assert S["slice_ptr"].tolist() == g["slice_ptr"]
    assert S["colval"].tolist() == g["colval"]
    assert S["nzval"].tolist() == g["nzval"]
    assert (S["perm"] == np.arange(1, 5)).all()


@pytest.mark.parametrize("m,p,seed", [(10, 0.5, 1), (1000, 0.2, 2)])
def test_csr_spmv_vs_fp64(m, p, seed):
    """test/spmv.jl:10-70: plus-times SpMV against SparseArrays A*b."""
    rowptr, colval, nzval, A = sprand_csr(m, m, p, seed=seed)
    x = np.random.default_rng(seed).random(m, dtype=np.float32)
    y = np.zeros(m, np.float32)
    assert O.csr_spmv(m, m, rowptr, colval, nzval, y, x) == O.OK
    ref = A.astype(np.float64) @ x.astype(np.float64)
    np.testing.assert_allclose(y, ref, rtol=1e-5, atol=1e-6)
    y2 = np.zeros(m, np.float32)
    O.spmv_plus_times_f32(rowptr, colval, nzval, x, y2)
    assert (y2 == y).all()


@pytest.mark.parametrize("C,sigma", [(32, 1), (8, 1), (4, 16), (32, 64)])
def test_sell_spmv_matches_csr_order(C, sigma):
    """SELL and CSR accumulate each row in the same storage order, so Float32
    plus-times results agree bit for bit (src/spmv/SELL.jl:31-63 vs CSR.jl:31-54)."""
    m = 300
    rowptr, colval, nzval, A = sprand_csr(m, m, 0.05, seed=5)
    x = np.random.default_rng(5).random(m, dtype=np.float32)
    y = np.zeros(m, np.float32)
    O.csr_spmv(m, m, rowptr, colval, nzval, y, x)
    S = O.sell_build(m, rowptr, colval, nzval, slice_size=C, sigma=sigma)
    ys = np.zeros(m, np.float32)
    assert O.sell_spmv(S, m, ys, x) == O.OK
    assert (ys == y).all()


def test_masked_spmv():
    """test/spmv.jl:72-170: dense Bool mask; masked-out rows keep their old value."""
    m = 1000
    rowptr, colval, nzval, A = sprand_csr(m, m, 0.2, seed=3)
    rng = np.random.default_rng(3)
    x = rng.random(m, dtype=np.float32)
    mask = rng.random(m) < 0.5
    ref = (A.astype(np.float64) @ x) * mask
    y = np.zeros(m, np.float32)
    O.csr_spmv(m, m, rowptr, colval, nzval, y, x, mask=mask)
    np.testing.assert_allclose(y, ref, rtol=1e-5, atol=1e-6)
    S = O.sell_build(m, rowptr, colval, nzval)
    ys = np.zeros(m, np.float32)
    O.sell_spmv(S, m, ys, x, mask=mask)
    assert (ys == y).all()
    # range + mask: rows outside the range keep the sentinel
    y3 = np.full(m, -7.0, np.float32)
    O.csr_spmv(m, m, rowptr, colval, nzval, y3, x, mask=mask, range_=(100, 200))
    sel = np.zeros(m, bool)
    sel[99:200] = True
    sel &= mask
    assert (y3[~sel] == -7.0).all()
    np.testing.assert_allclose(y3[sel], ref[sel], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("layout", [0, 1])
def test_spmm_vs_fp64(layout):
    """test/spmm.jl:10-73: CSR / SELL SpMM against SparseArrays A*B."""
    m, k = 1000, 20
    rowptr, colval, nzval, A = sprand_csr(m, m, 0.2, seed=4)
    rng = np.random.default_rng(4)
    B = rng.random((m, k), dtype=np.float32)
    B = np.asfortranarray(B) if layout == 0 else np.ascontiguousarray(B)
    ref = A.astype(np.float64) @ B.astype(np.float64)
    Cm = np.zeros((m, k), np.float32, order="F" if layout == 0 else "C")
    assert O.csr_spmm(m, rowptr, colval, nzval, Cm, B, layout=layout) == O.OK
    np.testing.assert_allclose(Cm, ref, rtol=1e-5, atol=1e-5)
    S = O.sell_build(m, rowptr, colval, nzval)
    C2 = np.zeros_like(Cm)
    assert O.sell_spmm(S, C2, B, layout=layout) == O.OK
    assert (C2 == Cm).all()


def test_semiring_scalars():
    """Julia semantics of src/algebra.jl on single-entry matrices."""
    rowptr = np.array([1, 2], np.int32)
    colval = np.array([1], np.int32)

    def one(a, xv, yinit, mul, add, accum, tx=None):
        nz = np.array([a])
        x = np.array([xv], dtype=tx or nz.dtype)
        y = np.array([yinit], dtype=np.result_type(nz.dtype, x.dtype))
        rc = O.csr_spmv(1, 1, rowptr, colval, nz, y, x, mul=mul, add=add, accum=accum)
        return rc, y[0]

    imax = np.int32(I32MAX)
    assert one(np.int32(5), imax, imax, O.SAFE_ADD, O.MIN, O.MIN)[1] == I32MAX
    assert one(np.int32(5), np.int32(7), imax, O.SAFE_ADD, O.MIN, O.MIN)[1] == 12
    assert one(np.float32(5), np.float32(np.inf), np.float32(np.inf), O.SAFE_ADD, O.MIN,
               O.MIN)[1] == np.inf
    # Int32 wraps like Julia
    assert one(np.int32(2 ** 30), np.int32(4), np.int32(0), O.MUL, O.ADD, O.SECOND)[1] == 0
    # min propagates NaN (Julia), unlike fmin
    rc, v = one(np.float32(np.nan), np.float32(1), np.float32(0), O.MUL, O.MIN, O.SECOND)
    assert np.isnan(v)
    # Bool + Bool is Int in Julia: no Bool plus monoid
    assert one(np.bool_(True), np.bool_(True), np.bool_(False), O.MUL, O.ADD,
               O.SECOND)[0] == O.UNSUPPORTED
    # bitwise operators on floats have no method
    assert one(np.float32(1), np.float32(1), np.float32(0), O.BAND, O.BOR,
               O.SECOND)[0] == O.UNSUPPORTED
    # secondi = column * y
    assert one(np.int32(9), np.int32(1), np.int32(0), O.SECONDI, O.ANY, O.SECOND)[1] == 1
    # result type narrower than promote_type(Tv, Tx)
    nz = np.array([1.0], np.float32)
    y = np.zeros(1, np.int32)
    assert O.csr_spmv(1, 1, rowptr, colval, nz, y, np.ones(1, np.float32)) == O.TYPE


def test_any_first_hit_vs_max():
    """CSR any kernel takes the first frontier column (src/spmv/CSR.jl:147-171);
    SELL any is max (src/algebra.jl:35); rows without a hit are left untouched."""
    # row 1: in-neighbours 2, 3, 4 (all in frontier); row 2: none in frontier
    rowptr = np.array([1, 4, 5, 5, 5], np.int32)
    colval = np.array([2, 3, 4, 1], np.int32)
    nz = np.ones(4, np.int32)
    x = np.array([0, 1, 1, 1], np.int32)
    mask = np.ones(4, np.int32)
    y = np.full(4, -5, np.int32)
    O.csr_spmv(4, 4, rowptr, colval, nz, y, x, mul=O.SECONDI, add=O.ANY, mask=mask)
    assert y.tolist() == [2, -5, -5, -5]
    S = O.sell_build(4, rowptr, colval, nz)
    ys = np.full(4, -5, np.int32)
    O.sell_spmv(S, 4, ys, x, mul=O.SECONDI, add=O.ANY, mask=mask)
    assert ys.tolist() == [4, 0, 0, 0]


@pytest.mark.parametrize("name", ["ba30", "dm30"])
def test_bfs_levels_golden(name):
    """test/bfs.jl:10-46: bfs_distances on Bool and Int32 0/1 matrices == gdistances."""
    g = golden_graphs()
    n = g[name + "_hop"].shape[0]
    for dt in (np.bool_, np.int32):
        rowptr, colval, nzval = undirected_csr(g[name + "_edges"], n, dtype=dt)
        for s in (1, 7, n):
            dist, _ = O.bfs_levels(n, rowptr, colval, nzval, s)
            assert (dist == g[name + "_hop"][:, s - 1]).all()


def test_bfs_levels_directed_unreachable():
    rng = np.random.default_rng(9)
    n = 400
    A = sp.random(n, n, density=0.004, random_state=rng, format="csr")
    A.data[:] = 1
    AT = A.T.tocsr()
    rowptr, colval, nzval = csr_from_scipy(AT.astype(np.bool_))
    for s in (1, 50):
        dist, _ = O.bfs_levels(n, rowptr, colval, nzval, s)
        assert (dist == bfs_levels_scipy(rowptr, colval, n, s)).all()
        assert (dist == I32MAX).any()


def test_bfs_levels_band_quirk():
    """Levels BFS uses band(A, curr): an Int32 edge with an even value is inactive."""
    rowptr = np.array([1, 1, 2, 3], np.int32)  # A_T rows: 1:{} 2:{1} 3:{2}
    colval = np.array([1, 2], np.int32)
    dist, _ = O.bfs_levels(3, rowptr, colval, np.array([1, 2], np.int32), 1)
    assert dist.tolist() == [0, 1, I32MAX]
    dist, _ = O.bfs_levels(3, rowptr, colval, np.array([3, 5], np.int32), 1)
    assert dist.tolist() == [0, 1, 2]


@pytest.mark.parametrize("rule", [1, 2])
def test_bfs_parents_rule(rule):
    g = golden_graphs()
    n = g["ba30_hop"].shape[0]
    rowptr, colval, nzval = undirected_csr(g["ba30_edges"], n, dtype=np.int32)
    par, _ = O.bfs_parents(n, rowptr, colval, 1, rule)
    lev = g["ba30_hop"][:, 0]
    assert par[0] == 0
    for v in range(1, n):
        nb = colval[rowptr[v] - 1:rowptr[v + 1] - 1]
        cand = [c for c in nb if lev[c - 1] == lev[v] - 1]
        assert par[v] == (min(cand) if rule == 1 else max(cand))


@pytest.mark.parametrize("name", ["ba30", "dm30"])
def test_shortest_path_golden(name):
    """test/shortest_path.jl:77-172: single and all-source Bellman-Ford == gdistances
    (Bool / Int32 0-1) and == dijkstra (Int32 weights)."""
    g = golden_graphs()
    n = g[name + "_hop"].shape[0]
    for dt in (np.bool_, np.int32):
        rowptr, colval, nzval = undirected_csr(g[name + "_edges"], n, dtype=dt)
        d, _ = O.sssp(n, rowptr, colval, nzval, [1])
        assert d.dtype == np.int32 and (d[:, 0] == g[name + "_hop"][:, 0]).all()
        d, _ = O.sssp(n, rowptr, colval, nzval, np.arange(1, n + 1))
        assert (d == g[name + "_hop"]).all()
    rowptr, colval, nzval = undirected_csr(g[name + "_edges"], n, weights=g[name + "_w"])
    d, _ = O.sssp(n, rowptr, colval, nzval, np.arange(1, n + 1))
    assert (d == g[name + "_dijkstra"]).all()


def test_shortest_path_float_vs_dijkstra():
    from scipy.sparse.csgraph import dijkstra
    rng = np.random.default_rng(11)
    n = 300
    A = sp.random(n, n, density=0.02, random_state=rng, format="csr")
    A.data = (1.0 + 9.0 * rng.random(A.nnz)).astype(np.float32)
    rowptr, colval, nzval = csr_from_scipy(A.T.tocsr().astype(np.float32))
    d, _ = O.sssp(n, rowptr, colval, nzval.astype(np.float32), [1, 17])
    ref = dijkstra(A.astype(np.float64), indices=[0, 16]).T
    fin = np.isfinite(ref)
    assert (np.isfinite(d) == fin).all()
    np.testing.assert_allclose(d[fin], ref[fin], rtol=1e-5)


def test_generators_and_assembly():
    s, d, w = O.gen_rmat(10, 16 * 1024, 0.57, 0.19, 0.19, 7, 1)
    assert s.min() >= 1 and s.max() <= 1024 and d.min() >= 1 and d.max() <= 1024
    rowptr, colval, nzval = O.coo_to_csr(1024, s, d, w, symmetrize=True, drop_loops=True)
    AT = sp.csr_matrix((nzval, colval - 1, rowptr - 1), shape=(1024, 1024))
    assert (AT != AT.T).nnz == 0           # symmetric, mirrored weights
    assert AT.diagonal().sum() == 0        # no self-loops
    # deduplicated, sorted columns
    for r in range(0, 1024, 37):
        c = colval[rowptr[r] - 1:rowptr[r + 1] - 1]
        assert (np.diff(c) > 0).all()
    # first duplicate kept: compare with an explicit dict build
    first = {}
    for e in range(len(s)):
        for a, b in ((s[e], d[e]), (d[e], s[e])):
            if a != b and (a, b) not in first:
                first[(a, b)] = w[e]
    assert len(first) == len(colval)
    r0 = int(s[0])
    for k in range(rowptr[r0 - 1] - 1, rowptr[r0] - 1):
        assert nzval[k] == first[(r0, colval[k])]
    gs, gd, gw = O.gen_grid(4, 5, 3, 3)
    assert len(gs) == 4 * 4 + 3 * 5 and gw.min() >= 1.0 and gw.max() < 10.0
    x = O.gen_uniform_f32(1000, 5)
    assert x.min() >= 0 and x.max() < 1


# --------------------------------------------------------------------------------
# full-size cross-checks (frontier BFS, parents from levels, multi-source BFS,
# Dijkstra) against the restated level-synchronous / Jacobi loops
# --------------------------------------------------------------------------------

def _graphs_for_cross_checks():
    """Directed and symmetric graphs with unreachable parts, hubs and a grid."""
    out = []
    s, d, w = O.gen_rmat(11, 8 * 2048, 0.57, 0.19, 0.19, 5, 2)  # Int32 1..255
    out.append(("rmat11_sym",) + O.coo_to_csr(2048, s, d, w, True, True))
    out.append(("rmat11_dir",) + O.coo_to_csr(2048, s, d, w, False, False))
    s, d, w = O.gen_er(3000, 3 * 3000, 6, 1)  # sparse directed ER, Float32 [0,1)
    out.append(("er3000_dir",) + O.coo_to_csr(3000, s, d, w, False, False))
    s, d, w = O.gen_grid(40, 37, 7, 3)  # Float32 [1, 10)
    out.append(("grid40x37",) + O.coo_to_csr(40 * 37, s, d, w, True, True))
    return out


def test_frontier_bfs_equals_level_synchronous_bfs():
    for name, rowptr, colval, nzval in _graphs_for_cross_checks():
        n = len(rowptr) - 1
        pat = np.ones(len(colval), np.bool_)
        for src in (1, n // 3 + 1, n):
            ref, _ = O.bfs_levels(n, rowptr, colval, pat, src)
            got, lv = O.bfs_levels_fast(n, rowptr, colval, None, src)
            assert (got == ref).all(), name
            assert lv == ref[ref != I32MAX].max()
            if "dir" not in name:  # symmetric: rows are their own out-edge lists
                got, _ = O.bfs_levels_fast(n, rowptr, colval, None, src, symmetric=True)
                assert (got == ref).all(), name
            if nzval.dtype == np.int32:  # only odd stored values are edges
                ref, _ = O.bfs_levels(n, rowptr, colval, nzval, src)
                got, _ = O.bfs_levels_fast(n, rowptr, colval, nzval, src)
                assert (got == ref).all(), name
            for rule in (1, 2):
                par_ref, _ = O.bfs_parents(n, rowptr, colval, src, rule)
                assert (O.bfs_parents_fast(n, rowptr, colval, src, rule) == par_ref).all(), name


def test_multi_source_bfs_equals_shortest_path_on_bool():
    for name, rowptr, colval, _ in _graphs_for_cross_checks()[:3]:
        n = len(rowptr) - 1
        src = np.array([1, 5, n // 2, n], np.int64)
        rows = np.arange(0, n, 3, dtype=np.int64)
        ref, _ = O.sssp(n, rowptr, colval, np.ones(len(colval), np.bool_), src)
        got = O.bfs_levels_multi(n, rowptr, colval, src, rows)
        assert (got == ref[rows]).all(), name
        if "dir" not in name:
            got = O.bfs_levels_multi(n, rowptr, colval, src, rows, symmetric=True)
            assert (got == ref[rows]).all(), name


def test_dijkstra_equals_jacobi_bellman_ford_bit_for_bit():
    """Int32 and Float32 weights: Dijkstra's distances equal the Jacobi fixpoint of
    shortest_path! bit for bit (Float32 sums rounded once per step in both)."""
    for name, rowptr, colval, nzval in _graphs_for_cross_checks():
        n = len(rowptr) - 1
        for src in (1, n // 2):
            ref, _ = O.sssp(n, rowptr, colval, nzval, [src])
            got = O.sssp_dijkstra(n, rowptr, colval, nzval, src)
            assert got.dtype == ref.dtype
            assert np.array_equal(got.view(np.int32), ref[:, 0].view(np.int32)), name
            if "dir" not in name:
                got = O.sssp_dijkstra(n, rowptr, colval, nzval, src, symmetric=True)
                assert np.array_equal(got.view(np.int32), ref[:, 0].view(np.int32)), name
    # Bool A_T: hop counts
    name, rowptr, colval, _ = _graphs_for_cross_checks()[1]
    n = len(rowptr) - 1
    pat = np.ones(len(colval), np.bool_)
    assert (O.sssp_dijkstra(n, rowptr, colval, pat, 3) == O.sssp(n, rowptr, colval, pat, [3])[0][:, 0]).all()
    with pytest.raises(ValueError):
        O.sssp_dijkstra(3, np.array([1, 2, 3, 3], np.int32), np.array([2, 3], np.int32),
                        np.array([1.0, -1.0], np.float32), 1)
