"""Bounded device-side waits run out cleanly.

gg_set_wait_limit lowers the poll limit of the grid barriers of the persistent
kernels to one poll: a barrier that some block reaches before the others then gives
up, every block returns, and the call raises TimeoutError_ (GG_ERR_TIMEOUT).  No GPU
fault is involved.  With the built-in limit restored, the next calls on the same
context succeed and equal the oracle."""
import numpy as np
import pytest
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from gpugraphs.errors import TimeoutError_
from gpugraphs.multigraph import MultiGraph
from gpugraphs.ops import set_wait_limit
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_barrier_waits_run_out_and_the_context_recovers():
    # a hub-free graph of >= 65536 vertices: Float32 shortest paths run as one
    # persistent near-far search with a grid barrier per step
    A = gen.grid(300, 250, seed=3, wkind=gen.W_F32_1_10)
    rp, cv, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    # many graphs: the BFS of all of them is one persistent cooperative launch
    gs = [gen.erdos_renyi(n, 6, seed=60 + i, wkind=gen.W_PATTERN, symmetric=True)
          for i, n in enumerate((500, 1200, 3000, 800))]
    gs.append(gen.grid(30, 20, seed=64, wkind=gen.W_PATTERN))
    mg = MultiGraph(gs)
    src = [1, 7, 100, 5, 300]
    try:
        set_wait_limit(1)
        with pytest.raises(TimeoutError_):
            G.shortest_path(A, 1)
        with pytest.raises(TimeoutError_):
            mg.bfs(src)
    finally:
        set_wait_limit(0)
    # the same context afterwards: correct results
    d = host(G.shortest_path(A, 1))
    ref = O.sssp_dijkstra(A.n, rp, cv, nz, 1, symmetric=True)
    assert np.array_equal(d.view(np.int32), ref.view(np.int32))
    parts = mg.split(mg.bfs(src))
    for g, s, part in zip(gs, src, parts):
        grp, gcv, gnz = host(g.rowptr), host(g.colval), host(g.nzval)
        lv, _ = O.bfs_levels(g.n, grp, gcv, gnz, s)
        assert (host(part) == lv).all()
    y = torch.zeros(A.n, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, A, torch.ones(A.n, dtype=torch.float32, device="cuda"))
    np.testing.assert_allclose(host(y), A.to_scipy().astype(np.float64) @ np.ones(A.n),
                               rtol=1e-5)
    G.synchronize()
