"""GPU parity at the benchmark configurations' own sizes, against the CPU oracle.

* Erdős–Rényi directed graph, n = 16384, average out-degree 16 (duplicates merged,
  self-loops kept), values and x uniform [0, 1): plus-times SpMV on CSR and SELL.
* R-MAT scale 22 (a, b, c = .57, .19, .19, edge factor 16, symmetrised, self-loops
  removed), the benchmark's seeds: every row of the plus-times SpMV against FP64
  and the oracle, SpMM rows against FP64, BFS levels and parents from 4 sources,
  Int32 shortest paths from 2 sources, all 256 columns of the batched BFS.
* 1024 x 1024 4-neighbour grid with Float32 weights [1, 10): shortest paths and
  BFS levels.

Tolerances: bit-exact for BFS levels / parents, Int32 and Float32 shortest paths
(the Bellman-Ford fixpoint is order independent), and plus-times rows folded in
storage order (CSR rows of at most 32 entries on the row-block kernel, rows of at
most 128 on the SELL copy); every plus-times row within rtol 1e-5 of FP64."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-5
I32MAX = np.iinfo(np.int32).max
RMAT_SEED = 1  # the benchmark's R-MAT seed; x of the SpMV: uniform_vector(seed=2)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def csr_host(A):
    return host(A.rowptr), host(A.colval), host(A.nzval)


def scipy_f64(rp, cv, nz, n):
    return sp.csr_matrix((nz.astype(np.float64), cv - 1, rp - 1), shape=(len(rp) - 1, n))


def sources_for(rp, k, seed):
    """k seeded non-isolated vertices (1-based), the benchmark's rule."""
    nz = np.flatnonzero(np.diff(rp) > 0)
    rng = np.random.default_rng(seed)
    return (nz[rng.integers(0, len(nz), k)] + 1).astype(np.int64)


def rel_err(got, ref):
    ref = np.asarray(ref, np.float64)
    d = np.abs(np.asarray(got, np.float64) - ref)
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(ref != 0, d / np.abs(ref), d)
    return float(r.max()) if r.size else 0.0


# --------------------------------------------------------------------------------
# Erdős–Rényi n = 16384 (the reference's CPU-runnable configuration)
# --------------------------------------------------------------------------------

def test_er16384_spmv_plus_times():
    n = 16384
    A = gen.erdos_renyi(n, 16, seed=1, wkind=gen.W_U01_F32)
    rp, cv, nz = csr_host(A)
    assert A.nnz() > 0.99 * 16 * n and A.nnz() <= 16 * n  # duplicates merged
    assert (cv == np.repeat(np.arange(1, n + 1), np.diff(rp))).any()  # self-loops kept
    x = host(gen.uniform_vector(n, seed=2))
    yo = np.zeros(n, np.float32)
    assert O.csr_spmv(n, n, rp, cv, nz, yo, x) == O.OK
    ref = scipy_f64(rp, cv, nz, n) @ x.astype(np.float64)
    deg = np.diff(rp)
    for M, exact_len in ((A, 32), (G.SparseGPUMatrixSELL(A), 128), (G.SparseGPUMatrixSELL(A, 32, n), 128)):
        y = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, M, torch.from_numpy(x).cuda())
        yh = host(y)
        exact = deg <= exact_len
        assert exact.mean() > 0.99
        np.testing.assert_array_equal(yh[exact], yo[exact])
        assert rel_err(yh, ref) <= RTOL


# --------------------------------------------------------------------------------
# R-MAT scale 22
# --------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def rmat22_f32():
    A = gen.rmat(22, 16, seed=RMAT_SEED, wkind=gen.W_U01_F32)
    x = gen.uniform_vector(A.n, seed=2)
    return A, x, csr_host(A)


@pytest.fixture(scope="module")
def rmat22_pattern():
    P = gen.rmat(22, 16, seed=RMAT_SEED, wkind=gen.W_PATTERN)
    return P, csr_host(P)


def test_rmat22_spmv_every_row(rmat22_f32):
    """The headline SpMV's configuration: all 4,194,304 rows against FP64 (rel err
    <= 1e-5) and every row of <= 128 entries against the oracle bit for bit, on the
    built-in layout (SELL-32 copy) and on a SELL-32 sigma = n handle."""
    A, x, (rp, cv, nz) = rmat22_f32
    n = A.n
    xh = host(x)
    ref = scipy_f64(rp, cv, nz, n) @ xh.astype(np.float64)
    yo = np.empty(n, np.float32)
    O.spmv_plus_times_f32(rp, cv, nz, xh, yo)
    deg = np.diff(rp)
    short = deg <= 128
    for M in (A, G.SparseGPUMatrixSELL(A, 32, n)):
        y = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        G.gpu_spmv_(y, M, x)
        yh = host(y)
        assert rel_err(yh, ref) <= RTOL
        np.testing.assert_array_equal(yh[short], yo[short])
    assert G.spmv_layout(A) == "sell"


def test_rmat22_spmm_rows(rmat22_f32):
    """SpMM with the configuration's 4,194,304 x 32 row-major X: the hub rows and a
    seeded sample of the others against FP64 (rel err <= 1e-5), every sampled row
    of <= 256 entries against the oracle's storage-order fold bit for bit."""
    A, _, (rp, cv, nz) = rmat22_f32
    n = A.n
    X = torch.rand((n, 32), dtype=torch.float32, device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(5))
    Y = torch.full((n, 32), float("nan"), dtype=torch.float32, device="cuda")
    G.gpu_spmm_(Y, A, X)
    deg = np.diff(rp)
    rng = np.random.default_rng(5)
    rows = np.unique(np.concatenate([np.argsort(-deg)[:2048], rng.integers(0, n, 30000)]))
    Xh = host(X)
    Yh = host(Y[torch.from_numpy(rows).cuda()])
    sub = scipy_f64(rp, cv, nz, n)[rows]
    ref = sub @ Xh.astype(np.float64)
    assert rel_err(Yh, ref) <= RTOL
    # oracle over the sampled rows of <= 256 entries: a CSR of those rows
    short = deg[rows] <= 256
    rs = rows[short]
    srp = np.concatenate([[1], 1 + np.cumsum(deg[rs])]).astype(np.int32)
    idx = np.concatenate([np.arange(rp[r] - 1, rp[r + 1] - 1) for r in rs])
    Co = np.zeros((len(rs), 32), np.float32)
    O.csr_spmm(len(rs), srp, cv[idx], nz[idx], Co, Xh, layout=1)
    np.testing.assert_array_equal(Yh[short], Co)


def test_rmat22_bfs_levels_and_parents(rmat22_pattern):
    """BFS levels and parents (CSR first-hit rule) from 4 seeded sources of the
    benchmark's source list, against the restated level-synchronous loops."""
    P, (rp, cv, nz) = rmat22_pattern
    n = P.n
    src = sources_for(rp, 256, 7)
    for s in [int(v) for v in src[:4]]:
        ref, _ = O.bfs_levels(n, rp, cv, nz, s)
        assert (host(G.bfs_distances(P, s)) == ref).all()
        pref, _ = O.bfs_parents(n, rp, cv, s, 1)
        assert (host(G.bfs_parents(P, s)) == pref).all()
    S = G.SparseGPUMatrixSELL(P, 32, n)
    s = int(src[4])
    assert (host(G.bfs_parents(S, s)) == O.bfs_parents(n, rp, cv, s, 2)[0]).all()


def test_rmat22_sssp_int32():
    """Int32 weights 1..255, 2 seeded sources: bit-exact against the restated Jacobi
    Bellman-Ford (one source) and Dijkstra (both)."""
    W = gen.rmat(22, 16, seed=RMAT_SEED, wkind=gen.W_INT_1_255)
    rp, cv, nz = csr_host(W)
    n = W.n
    src = sources_for(rp, 256, 7)[:2]
    d0 = host(G.shortest_path(W, int(src[0])))
    ref, rounds = O.sssp(n, rp, cv, nz, [int(src[0])])
    assert rounds > 0 and (d0 == ref[:, 0]).all()
    for s in src:
        d = host(G.shortest_path(W, int(s)))
        assert (d == O.sssp_dijkstra(n, rp, cv, nz, int(s), symmetric=True)).all()


def test_rmat22_batched_bfs_all_256_columns(rmat22_pattern):
    """bfs_distances_batch with the benchmark's 256 sources: every column against the
    oracle's hop distances on a seeded sample of rows (all hub rows included)."""
    P, (rp, cv, nz) = rmat22_pattern
    n = P.n
    src = sources_for(rp, 256, 7)
    D = G.bfs_distances_batch(P, src)
    deg = np.diff(rp)
    rng = np.random.default_rng(9)
    rows = np.unique(np.concatenate([np.argsort(-deg)[:512], rng.integers(0, n, 16384)]))
    got = host(D[torch.from_numpy(rows).cuda()])
    ref = O.bfs_levels_multi(n, rp, cv, src, rows, symmetric=True)
    assert got.shape == ref.shape == (len(rows), 256)
    assert (got == ref).all()


# --------------------------------------------------------------------------------
# high-diameter grid
# --------------------------------------------------------------------------------

def test_grid1024_float32_sssp_and_bfs():
    """1024 x 1024 4-neighbour grid (hop diameter 2046), Float32 weights [1, 10):
    shortest paths bit-exact against Dijkstra in Float32 (the Jacobi fixpoint, see
    oracle.c), BFS levels against the frontier BFS."""
    A = gen.grid(1024, 1024, seed=4, wkind=gen.W_F32_1_10)
    rp, cv, nz = csr_host(A)
    n = A.n
    for s in (1, 524800, int(sources_for(rp, 64, 11)[0])):
        d = host(G.shortest_path(A, s))
        ref = O.sssp_dijkstra(n, rp, cv, nz, s, symmetric=True)
        assert d.dtype == np.float32
        assert np.array_equal(d.view(np.int32), ref.view(np.int32))
    P = G.SparseGPUMatrixCSR(n, n, A.rowptr, A.colval,
                             torch.ones(A.nnz(), dtype=torch.bool, device="cuda"))
    lv = host(G.bfs_distances(P, 1))
    ref, top = O.bfs_levels_fast(n, rp, cv, None, 1, symmetric=True)
    assert top == 2046 and (lv == ref).all()
