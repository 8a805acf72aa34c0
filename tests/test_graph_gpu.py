"""GPU parity of bfs_distances / bfs_parents / shortest_path and of the synthetic
graph generators against the CPU oracle and the golden fixtures.

Every comparison here is exact: BFS levels and parents are integers, and the
Bellman-Ford fixpoint is order independent, so Int32 and Float32 distances must
match bit for bit."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from oracle import oracle as O
from helpers import csr_from_scipy, golden_graphs, undirected_csr

pytestmark = pytest.mark.gpu
I32MAX = np.iinfo(np.int32).max


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def csr_host(A):
    return host(A.rowptr), host(A.colval), host(A.nzval)


@pytest.mark.parametrize("name", ["ba30", "dm30"])
def test_bfs_golden(name):
    """test/bfs.jl:10-46 (CSR, Bool and Int32 0/1) plus SELL."""
    g = golden_graphs()
    n = g[name + "_hop"].shape[0]
    for dt in (np.bool_, np.int32):
        rp, cv, nz = undirected_csr(g[name + "_edges"], n, dtype=dt)
        B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
        for M in (B, G.SparseGPUMatrixSELL(B), G.SparseGPUMatrixSELL(B, 8, 16)):
            for s in (1, 5, n):
                assert (host(G.bfs_distances(M, s)) == g[name + "_hop"][:, s - 1]).all()


@pytest.mark.parametrize("fmt", ["csr", "sell"])
def test_bfs_parents_rules(fmt):
    g = golden_graphs()
    for name in ("ba30", "dm30"):
        n = g[name + "_hop"].shape[0]
        rp, cv, nz = undirected_csr(g[name + "_edges"], n, dtype=np.int32)
        B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
        M = B if fmt == "csr" else G.SparseGPUMatrixSELL(B, 8, 4)
        for s in (1, 9):
            ref, _ = O.bfs_parents(n, rp, cv, s, 1 if fmt == "csr" else 2)
            assert (host(G.bfs_parents(M, s)) == ref).all()


def _directed(n, density, seed, dtype=np.bool_):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=density, random_state=rng, format="csr")
    A.data[:] = 1
    return csr_from_scipy(A.T.tocsr().astype(dtype))


def test_bfs_directed_unreachable_and_inplace():
    n = 3000
    rp, cv, nz = _directed(n, 0.0012, 3)
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    for s in (1, 77, 2999):
        ref, _ = O.bfs_levels(n, rp, cv, nz, s)
        got = host(G.bfs_distances(B, s))
        assert (got == ref).all()
        assert (got == I32MAX).any()
        # in-place form leaves unreached entries untouched
        d = torch.full((n,), -9, dtype=torch.int32, device="cuda")
        G.bfs_distances_(B, s, d)
        dh = host(d)
        assert (dh[ref != I32MAX] == ref[ref != I32MAX]).all() and (dh[ref == I32MAX] == -9).all()
        for rule, fmt_rule in ((1, G.algorithms.PARENT_FIRST_IN_ROW), (2, G.algorithms.PARENT_MAX_INDEX)):
            pref, _ = O.bfs_parents(n, rp, cv, s, rule)
            assert (host(G.bfs_parents(B, s, rule=fmt_rule)) == pref).all()


def test_bfs_band_quirk_int32_values():
    """Levels use band(A, curr): Int32 edges with even values are inactive, while
    parents (secondi / any) use every stored edge."""
    n = 2000
    rng = np.random.default_rng(5)
    rp, cv, nz = _directed(n, 0.004, 5, dtype=np.int32)
    nz = rng.integers(1, 5, len(cv)).astype(np.int32)
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    for s in (1, 100):
        ref, _ = O.bfs_levels(n, rp, cv, nz, s)
        assert (host(G.bfs_distances(B, s)) == ref).all()
        pref, _ = O.bfs_parents(n, rp, cv, s, 1)
        assert (host(G.bfs_parents(B, s)) == pref).all()


@pytest.mark.parametrize("scale", [12, 16])
def test_bfs_rmat_push_pull(scale):
    """R-MAT graphs large enough to leave the single-CTA path and switch between
    top-down and bottom-up levels."""
    A = gen.rmat(scale, 16, seed=3, wkind=gen.W_PATTERN)
    rp, cv, nz = csr_host(A)
    n = A.n
    deg = np.diff(rp)
    for s in (int(np.argmax(deg)) + 1, int(np.nonzero(deg)[0][-1]) + 1):
        ref, _ = O.bfs_levels(n, rp, cv, nz, s)
        assert (host(G.bfs_distances(A, s)) == ref).all()
        pref, _ = O.bfs_parents(n, rp, cv, s, 1)
        assert (host(G.bfs_parents(A, s)) == pref).all()
    S = G.SparseGPUMatrixSELL(A, 32, 256)
    s = int(np.argmax(deg)) + 1
    ref, _ = O.bfs_levels(n, rp, cv, nz, s)
    assert (host(G.bfs_distances(S, s)) == ref).all()
    pref, _ = O.bfs_parents(n, rp, cv, s, 2)
    assert (host(G.bfs_parents(S, s)) == pref).all()


def test_bfs_grid_high_diameter():
    A = gen.grid(300, 200, seed=4, wkind=gen.W_PATTERN)
    rp, cv, nz = csr_host(A)
    for s in (1, 300 * 200, 12345):
        ref, lv = O.bfs_levels(A.n, rp, cv, nz, s)
        assert (host(G.bfs_distances(A, s)) == ref).all()


@pytest.mark.parametrize("name", ["ba30", "dm30"])
def test_shortest_path_golden(name):
    """test/shortest_path.jl:77-172: SELL (and CSR) single / all sources, Bool / Int32
    0-1 against gdistances and Int32 weights against dijkstra."""
    g = golden_graphs()
    n = g[name + "_hop"].shape[0]
    for dt in (np.bool_, np.int32):
        rp, cv, nz = undirected_csr(g[name + "_edges"], n, dtype=dt)
        B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
        for M in (B, G.SparseGPUMatrixSELL(B)):
            d1 = host(G.shortest_path(M, 1))
            assert d1.dtype == np.int32 and (d1 == g[name + "_hop"][:, 0]).all()
            dall = G.shortest_path(M, np.arange(1, n + 1, dtype=np.int32))
            assert dall.shape == (n, n) and (host(dall) == g[name + "_hop"]).all()
    rp, cv, nz = undirected_csr(g[name + "_edges"], n, weights=g[name + "_w"])
    M = G.SparseGPUMatrixSELL(G.SparseGPUMatrixCSR(n, n, rp, cv, nz))
    assert (host(G.shortest_path(M, np.arange(1, n + 1))) == g[name + "_dijkstra"]).all()


def test_shortest_path_float_grid_exact():
    A = gen.grid(120, 90, seed=6, wkind=gen.W_F32_1_10)
    rp, cv, nz = csr_host(A)
    for s in (1, 5000):
        ref, _ = O.sssp(A.n, rp, cv, nz, [s])
        got = host(G.shortest_path(A, s))
        assert got.dtype == np.float32 and (got == ref[:, 0]).all()


def test_shortest_path_int_rmat_exact():
    A = gen.rmat(13, 16, seed=7, wkind=gen.W_INT_1_255)
    rp, cv, nz = csr_host(A)
    deg = np.diff(rp)
    srcs = [int(np.argmax(deg)) + 1, int(np.nonzero(deg)[0][7]) + 1, 1]
    ref, _ = O.sssp(A.n, rp, cv, nz, srcs)
    got = host(G.shortest_path(A, np.array(srcs)))
    assert (got == ref).all()
    S = G.SparseGPUMatrixSELL(A, 16, 64)
    assert (host(G.shortest_path(S, srcs[0])) == ref[:, 0]).all()


def test_shortest_path_directed_float():
    n = 2500
    rng = np.random.default_rng(8)
    A = sp.random(n, n, density=0.002, random_state=rng, format="csr")
    A.data = (rng.random(A.nnz) * 3).astype(np.float32)
    rp, cv, nz = csr_from_scipy(A.T.tocsr().astype(np.float32))
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    ref, _ = O.sssp(n, rp, cv, nz, [1, 400])
    assert (host(G.shortest_path(B, [1, 400])) == ref).all()


def _reference_inplace(n, rp, cv, nz, s, dist0, next0):
    """The loop of shortest_path! (shortest_path.jl:34-83) on the oracle's SpMV."""
    dist, nxt = dist0.copy(), next0.copy()
    dist[s - 1] = 0
    nxt[s - 1] = 0
    for _ in range(4 * n):
        O.csr_spmv(n, n, rp, cv, nz, nxt, dist, O.SAFE_ADD, O.MIN, O.MIN)
        changed = (nxt < dist).any()
        dist[:] = nxt
        if not changed:
            break
    return dist


def test_shortest_path_inplace_caller_state():
    n = 400
    rng = np.random.default_rng(9)
    A = sp.random(n, n, density=0.01, random_state=rng, format="csr")
    A.data = rng.integers(1, 9, A.nnz).astype(np.int32)
    rp, cv, nz = csr_from_scipy(A.T.tocsr().astype(np.int32))
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    dist0 = np.full(n, I32MAX, np.int32)
    next0 = np.full(n, I32MAX, np.int32)
    dist0[10], next0[20], dist0[30], next0[30] = 5, 7, 100, 2
    ref = _reference_inplace(n, rp, cv, nz, 3, dist0, next0)
    d = torch.from_numpy(dist0).cuda()
    x = torch.from_numpy(next0).cuda()
    G.shortest_path_(B, 3, d, x)
    assert (host(d) == ref).all() and (host(x) == ref).all()


def test_shortest_path_negative_weights_jacobi():
    n = 300
    rng = np.random.default_rng(10)
    A = sp.random(n, n, density=0.01, random_state=rng, format="csr")
    A.data = rng.integers(1, 9, A.nnz).astype(np.int32)
    A = sp.triu(A, 1).tocsr()  # a DAG: negative weights without negative cycles
    A.data[::5] *= -1
    rp, cv, nz = csr_from_scipy(A.T.tocsr().astype(np.int32))
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    ref, _ = O.sssp(n, rp, cv, nz, [1, 2])
    assert (host(G.shortest_path(B, [1, 2])) == ref).all()


def test_graph_errors():
    g = golden_graphs()
    rp, cv, nz = undirected_csr(g["ba30_edges"], 30, dtype=np.float32)
    B = G.SparseGPUMatrixCSR(30, 30, rp, cv, nz)
    with pytest.raises(G.BoundsError):
        G.bfs_distances(B, 31)
    with pytest.raises(G.BoundsError):
        G.shortest_path(B, 0)
    with pytest.raises(G.UnsupportedError):
        G.bfs_distances(B, 1)  # band has no Float32 method
    R = G.SparseGPUMatrixCSR(2, 3, np.array([1, 2, 3]), np.array([1, 3]), np.ones(2, np.bool_))
    with pytest.raises(G.DimensionMismatch):
        G.bfs_distances(R, 1)


def test_generators_match_oracle():
    for wk in (gen.W_PATTERN, gen.W_U01_F32, gen.W_INT_1_255, gen.W_F32_1_10):
        s, d, w = gen.rmat_edges(10, 5000, seed=11, wkind=wk)
        os_, od, ow = O.gen_rmat(10, 5000, 0.57, 0.19, 0.19, 11, wk)
        assert (host(s) == os_).all() and (host(d) == od).all() and (host(w) == ow).all()
    s, d, w = gen.er_edges(777, 4000, seed=12, wkind=gen.W_U01_F32)
    os_, od, ow = O.gen_er(777, 4000, 12, 1)
    assert (host(s) == os_).all() and (host(d) == od).all() and (host(w) == ow).all()
    s, d, w = gen.grid_edges(17, 23, seed=13, wkind=gen.W_F32_1_10)
    os_, od, ow = O.gen_grid(17, 23, 13, 3)
    assert (host(s) == os_).all() and (host(d) == od).all() and (host(w) == ow).all()
    assert (host(gen.uniform_vector(1000, seed=14)) == O.gen_uniform_f32(1000, 14)).all()
    # CSR assembly: device (torch sort) == oracle (counting sort)
    A = gen.rmat(11, 16, seed=15, wkind=gen.W_INT_1_255)
    s, d, w = O.gen_rmat(11, 16 * 2048, 0.57, 0.19, 0.19, 15, 2)
    rp, cv, nz = O.coo_to_csr(2048, s, d, w, symmetrize=True, drop_loops=True)
    grp, gcv, gnz = csr_host(A)
    assert (grp == rp).all() and (gcv == cv).all() and (gnz == nz).all()
    E = gen.erdos_renyi(1500, 16, seed=16)
    s, d, w = O.gen_er(1500, 1500 * 16, 16, 1)
    rp, cv, nz = O.coo_to_csr(1500, s, d, w, symmetrize=False, drop_loops=False)
    grp, gcv, gnz = csr_host(E)
    assert (grp == rp).all() and (gcv == cv).all() and (gnz == nz).all()


@pytest.mark.parametrize("wkind", [gen.W_F32_1_10, gen.W_INT_1_255])
def test_grid_persistent_paths_exact(wkind):
    """Grids of >= 65536 vertices (out-degree <= 4) run BFS levels through the
    persistent cooperative kernel and shortest paths as one near-far ordered
    persistent search: both equal the oracle exactly."""
    A = gen.grid(300, 250, seed=61, wkind=wkind)
    rp, cv, nz = csr_host(A)
    for s in (1, 37000, 75000):
        ref, _ = O.sssp(A.n, rp, cv, nz, [s])
        got = host(G.shortest_path(A, s))
        assert (got == ref[:, 0]).all(), s
    P = G.SparseGPUMatrixCSR(A.m, A.n, A.rowptr, A.colval,
                             torch.ones(A.nnz(), dtype=torch.bool, device="cuda"))
    pr, pc, pn = csr_host(P)
    for s in (1, 40000):
        lv, _ = O.bfs_levels(A.n, pr, pc, pn, s)
        assert (host(G.bfs_distances(P, s)) == lv).all(), s


@pytest.mark.parametrize("wkind,directed", [(gen.W_INT_1_255, False), (gen.W_U01_F32, False),
                                            (gen.W_INT_1_255, True)])
def test_sssp_large_csr_pull_rounds(wkind, directed):
    """CSR handles of >= 65536 rows run their pull rounds over a SELL-32 copy (every
    in-edge, atomic min, in place); distances equal Dijkstra's bit for bit (Int32 and
    Float32 weights; a directed R-MAT whose A_T differs from A), two sources each."""
    A = gen.rmat(17, 16, seed=41, wkind=wkind, symmetrize=not directed, drop_loops=not directed)
    rp, cv, nz = csr_host(A)
    n = A.n
    deg = np.diff(rp)
    for s in (int(np.argmax(deg)) + 1, int(np.flatnonzero(deg > 0)[len(deg) // 3]) + 1):
        d = host(G.shortest_path(A, s))
        ref = O.sssp_dijkstra(n, rp, cv, nz, s, symmetric=not directed)
        assert d.dtype == ref.dtype
        assert np.array_equal(d.view(np.int32), ref.view(np.int32))
