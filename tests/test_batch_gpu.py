"""GPU parity of the batched engines (many sources in one pass): batched BFS levels
and batched shortest paths equal the per-source results column by column, exactly."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from oracle import oracle as O
from helpers import csr_from_scipy, golden_graphs, undirected_csr

pytestmark = pytest.mark.gpu


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def csr_host(A):
    return host(A.rowptr), host(A.colval), host(A.nzval)


def test_bfs_batch_rmat_two_groups():
    A = gen.rmat(13, 16, seed=31, wkind=gen.W_PATTERN)
    rp, cv, nz = csr_host(A)
    n = A.n
    rng = np.random.default_rng(31)
    src = rng.integers(1, n + 1, 300)  # two groups: 256 + 44
    D = host(G.bfs_distances_batch(A, src))
    assert D.shape == (n, 300)
    for q in list(range(0, 300, 23)) + [255, 256, 299]:
        ref, _ = O.bfs_levels(n, rp, cv, nz, int(src[q]))
        assert (D[:, q] == ref).all(), q
    S = G.SparseGPUMatrixSELL(A, 32, 64)
    D2 = host(G.bfs_distances_batch(S, src[:40]))
    assert (D2 == D[:, :40]).all()


def test_bfs_batch_odd_values_and_directed():
    n = 2500
    rng = np.random.default_rng(32)
    M = sp.random(n, n, density=0.003, random_state=rng, format="csr")
    M.data = rng.integers(1, 5, M.nnz).astype(np.int32)
    rp, cv, nz = csr_from_scipy(M.T.tocsr().astype(np.int32))
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    src = np.arange(1, n + 1, 97)
    D = host(G.bfs_distances_batch(B, src))
    for q, s in enumerate(src):
        ref, _ = O.bfs_levels(n, rp, cv, nz, int(s))
        assert (D[:, q] == ref).all()


@pytest.mark.parametrize("name", ["ba30", "dm30"])
def test_sssp_batch_golden_all_sources(name):
    g = golden_graphs()
    n = g[name + "_hop"].shape[0]
    rp, cv, nz = undirected_csr(g[name + "_edges"], n, weights=g[name + "_w"])
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    L = G.core.lib()
    d = torch.empty((n, n), dtype=torch.int32, device="cuda").T.contiguous().T
    src = np.arange(1, n + 1, dtype=np.int64)
    import ctypes
    rc = L.gg_sssp_batch(G.core.ctx(), B.handle, src.ctypes.data_as(ctypes.c_void_p), n,
                         G.core.ptr(d), 2, n, None)
    assert rc == 0
    assert (host(d) == g[name + "_dijkstra"]).all()


def test_sssp_batch_int_rmat_and_float_grid():
    A = gen.rmat(12, 16, seed=33, wkind=gen.W_INT_1_255)
    rp, cv, nz = csr_host(A)
    rng = np.random.default_rng(33)
    src = rng.integers(1, A.n + 1, 40)
    ref, _ = O.sssp(A.n, rp, cv, nz, src)
    assert (host(G.shortest_path(A, src)) == ref).all()  # routed to the batched engine
    Gf = gen.grid(60, 50, seed=34, wkind=gen.W_F32_1_10)
    rp, cv, nz = csr_host(Gf)
    src = rng.integers(1, Gf.n + 1, 33)
    ref, _ = O.sssp(Gf.n, rp, cv, nz, src)
    got = host(G.shortest_path(Gf, src))
    assert got.dtype == np.float32 and (got == ref).all()
    S = G.SparseGPUMatrixSELL(Gf, 16, 32)
    assert (host(G.shortest_path(S, src)) == ref).all()


def hub_graph(n, seed, dtype):
    """Directed graph with two hubs of 6000 and 9000 in-edges (split into pieces), a
    vertex of 1500 in-edges (whole-warp scan) and a sparse random remainder."""
    rng = np.random.default_rng(seed)
    M = sp.random(n, n, density=3.0 / n, random_state=rng, format="coo")
    rows, cols = [M.row], [M.col]
    for v, d in ((0, 6000), (1, 9000), (2, 1500)):
        rows.append(np.full(d, v))
        cols.append(rng.choice(n, d, replace=False))
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    if dtype == np.float32:
        vals = rng.uniform(1, 10, len(rows)).astype(np.float32)
    else:
        vals = rng.integers(1, 6, len(rows)).astype(dtype)
    A_T = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))  # row v lists in-neighbours
    A_T.sum_duplicates()
    A_T.sort_indices()
    return csr_from_scipy(A_T)


def test_bfs_batch_hubs():
    n = 12000
    rp, cv, nz = hub_graph(n, 41, np.int32)
    assert np.diff(rp).max() > 2048
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    rng = np.random.default_rng(41)
    src = np.concatenate([[1, 2, 3], rng.integers(1, n + 1, 97)])
    for rep in range(2):  # hub accumulators are cleared for the next call
        D = host(G.bfs_distances_batch(B, src))
        for q in list(range(0, 100, 7)) + [0, 1, 2, 99]:
            ref, _ = O.bfs_levels(n, rp, cv, nz, int(src[q]))
            assert (D[:, q] == ref).all(), (rep, q)


@pytest.mark.parametrize("dtype", [np.int32, np.float32])
def test_sssp_batch_hubs(dtype):
    n = 12000
    rp, cv, nz = hub_graph(n, 42, dtype)
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    rng = np.random.default_rng(42)
    src = np.concatenate([[1, 2, 3], rng.integers(1, n + 1, 37)]).astype(np.int64)
    ref, _ = O.sssp(n, rp, cv, nz, src)
    got = host(G.shortest_path(B, src))
    assert (got == ref).all()


@pytest.mark.parametrize("dtype", [np.int32, np.float32])
def test_single_source_hub_pieces(dtype):
    """Single-source BFS and shortest paths where frontier vertices have thousands of
    out-edges (push pieces) and in-edges (pull pieces), on a directed graph and on its
    symmetrised version."""
    n = 12000
    rp, cv, nz = hub_graph(n, 43, dtype)
    A = sp.csr_matrix((nz, cv - 1, rp - 1), shape=(n, n))
    for M in (A, (A + A.T).tocsr()):
        M.sort_indices()
        rp2, cv2, nz2 = csr_from_scipy(M)
        B = G.SparseGPUMatrixCSR(n, n, rp2, cv2, nz2)
        for s in (1, 2, 3, 77, 5000):
            ref, _ = O.sssp(n, rp2, cv2, nz2, np.array([s], np.int64))
            got = host(G.shortest_path(B, s))
            assert (got == ref[:, 0] if ref.ndim == 2 else got == ref).all(), s
            if dtype == np.int32:
                lv, _ = O.bfs_levels(n, rp2, cv2, nz2, s)
                assert (host(G.bfs_distances(B, s)) == lv).all(), s


@pytest.mark.parametrize("dtype", [np.int32, np.float32])
def test_sssp_batch_sell_full_rounds(dtype):
    """Graphs of at least 65536 vertices: the batched rounds that visit every vertex run
    over the SELL-32 copy (32 rows x 32 source columns of minima per warp, hubs as row
    chunks lowered with atomic min).  R-MAT scale 16 (Int32 1..255 or Float32 [1,10))
    with 40 sources (two groups) and a directed graph with hubs of 6000 / 9000 in-edges,
    every column equal to the oracle."""
    wk = gen.W_INT_1_255 if dtype == np.int32 else gen.W_F32_1_10
    A = gen.rmat(16, 16, seed=35, wkind=wk)
    rp, cv, nz = csr_host(A)
    rng = np.random.default_rng(35)
    src = rng.integers(1, A.n + 1, 40)
    ref, _ = O.sssp(A.n, rp, cv, nz, src)
    got = host(G.shortest_path(A, src))
    assert got.dtype == dtype and (got == ref).all()
    n = 70000
    rp, cv, nz = hub_graph(n, 44, dtype)
    B = G.SparseGPUMatrixCSR(n, n, rp, cv, nz)
    src = np.concatenate([[1, 2, 3], rng.integers(1, n + 1, 34)]).astype(np.int64)
    ref, _ = O.sssp(n, rp, cv, nz, src)
    for rep in range(2):
        got = host(G.shortest_path(B, src))
        assert (got == ref).all(), rep

