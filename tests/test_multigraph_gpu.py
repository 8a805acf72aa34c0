"""Many graphs in one launch: every graph's SpMV and BFS equal its own single-graph
result (BFS exactly; SpMV within rtol 1e-5 of FP64), launch after launch."""
import numpy as np
import pytest
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from gpugraphs.multigraph import MultiGraph

pytestmark = pytest.mark.gpu


def _graphs(wkind):
    rng = np.random.default_rng(51)
    gs = []
    for i in range(24):
        n = int(10 ** rng.uniform(2, 3.7))
        d = int(rng.integers(2, 16))
        gs.append(gen.erdos_renyi(n, d, seed=100 + i, wkind=wkind, symmetric=True))
    gs.append(gen.grid(30, 20, seed=52, wkind=wkind if wkind != gen.W_INT_1_255 else gen.W_PATTERN))
    return gs


def test_multigraph_bfs_matches_per_graph():
    gs = _graphs(gen.W_PATTERN)
    mg = MultiGraph(gs)
    assert mg.ngraphs == len(gs) and mg.total_n == sum(g.n for g in gs)
    rng = np.random.default_rng(53)
    for rep in range(2):  # second call replays the captured CUDA graph
        src = [int(rng.integers(1, g.n + 1)) for g in gs]
        d = mg.bfs(src)
        torch.cuda.synchronize()
        for g, s, part in zip(gs, src, mg.split(d)):
            assert torch.equal(part, G.bfs_distances(g, s))


def test_multigraph_spmv_matches_per_graph():
    gs = _graphs(gen.W_U01_F32)
    gs = gs[:-1]  # Float32 graphs only
    mg = MultiGraph(gs)
    x = torch.rand(mg.total_n, device="cuda")
    for rep in range(2):
        y = mg.spmv(x)
        torch.cuda.synchronize()
        for g, xp, yp in zip(gs, mg.split(x), mg.split(y)):
            ref = g.to_scipy().astype(np.float64) @ xp.double().cpu().numpy()
            np.testing.assert_allclose(yp.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("wkind", [gen.W_INT_1_255, gen.W_F32_1_10, gen.W_PATTERN])
def test_multigraph_sssp_matches_per_graph(wkind):
    gs = _graphs(wkind)
    if wkind == gen.W_INT_1_255:
        gs = gs[:-1]  # the grid is a Bool pattern there
    mg = MultiGraph(gs)
    rng = np.random.default_rng(54)
    for rep in range(2):
        src = [int(rng.integers(1, g.n + 1)) for g in gs]
        d = mg.sssp(src)
        torch.cuda.synchronize()
        for g, s, part in zip(gs, src, mg.split(d)):
            assert torch.equal(part, G.shortest_path(g, s))


def test_multigraph_bfs_float_graphs_use_the_pattern():
    gs = _graphs(gen.W_U01_F32)[:-1]
    mg = MultiGraph(gs)
    src = [1 for _ in gs]
    d = mg.bfs(src)
    torch.cuda.synchronize()
    for g, part in zip(gs, mg.split(d)):
        P = G.SparseGPUMatrixCSR(g.m, g.n, g.rowptr, g.colval,
                                 torch.ones(g.nnz(), dtype=torch.bool, device="cuda"))
        assert torch.equal(part, G.bfs_distances(P, 1))


def test_multigraph_entry_offsets_past_int32():
    """Six symmetric Erdos-Renyi graphs of 2^22 vertices with about 108 entries per row
    hold more than 2^31 stored entries together, so the last graphs' entry offsets in
    the concatenation exceed Int32 (the 1000-graph configuration holds about 2.6 G).
    Their SpMV (within rtol 1e-5 of FP64), BFS levels (exact, against the oracle's
    frontier BFS) and shortest paths (exact, against the single-graph path) from the
    one-launch structure equal the per-graph results."""
    import scipy.sparse as sp
    from oracle import oracle as O
    n = 1 << 22
    gs = [gen.erdos_renyi(n, 54, seed=70 + i, wkind=gen.W_F32_1_10, symmetric=True) for i in range(6)]
    mg = MultiGraph(gs)
    assert mg.total_nnz > 2 ** 31 and int(mg.offsets[-1]) == 6 * n
    last = gs[-1]
    rp, cv, nz = (t.cpu().numpy() for t in (last.rowptr, last.colval, last.nzval))
    before = sum(g.nnz() for g in gs[:-1])
    assert before > 2 ** 31  # every entry of the last graph sits past Int32 offsets
    x = torch.rand(mg.total_n, device="cuda", generator=torch.Generator(device="cuda").manual_seed(7))
    y = mg.spmv(x)
    xl = mg.split(x)[-1].cpu().numpy().astype(np.float64)
    ref = sp.csr_matrix((nz.astype(np.float64), cv - 1, rp - 1), shape=(n, n)) @ xl
    np.testing.assert_allclose(mg.split(y)[-1].cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
    src = [1 + 97 * i for i in range(len(gs))]
    d = mg.bfs(src)
    torch.cuda.synchronize()
    lv, _ = O.bfs_levels_fast(n, rp, cv, None, src[-1], symmetric=True)
    assert (mg.split(d)[-1].cpu().numpy() == lv).all()
    ds = mg.sssp(src)
    torch.cuda.synchronize()
    for g, s, part in list(zip(gs, src, mg.split(ds)))[-2:]:
        assert torch.equal(part, G.shortest_path(g, s))
