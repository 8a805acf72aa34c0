"""The continuous-batching server: every result equals the single-query path (BFS and
shortest paths exactly; SpMV iterations exactly against the same query run alone on
the server, and within rtol 1e-5 of the FP64 iteration), whatever mix it ran in."""
import numpy as np
import pytest
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from gpugraphs.serving import Server

pytestmark = pytest.mark.gpu


def _graphs():
    return [gen.rmat(12, 16, seed=41, wkind=gen.W_PATTERN),
            gen.rmat(11, 16, seed=42, wkind=gen.W_INT_1_255),
            gen.grid(40, 30, seed=43, wkind=gen.W_F32_1_10),
            gen.rmat(11, 8, seed=44, wkind=gen.W_U01_F32)]


def test_server_mix_equals_single_queries():
    gs = _graphs()
    srv = Server(reserve_bytes=0)
    ids = [srv.add_graph(A) for A in gs]
    rng = np.random.default_rng(45)
    reqs = []
    xs = {}
    for i in range(300):
        kind = i % 3
        if kind == 0:
            g = int(rng.choice([0, 1]))
            s = int(rng.integers(1, gs[g].n + 1))
            reqs.append((srv.submit_bfs(ids[g], s), "bfs", g, s))
        elif kind == 1:
            g = int(rng.choice([1, 2]))
            s = int(rng.integers(1, gs[g].n + 1))
            reqs.append((srv.submit_sssp(ids[g], s), "sssp", g, s))
        else:
            g = 3
            x = torch.rand(gs[g].n, device="cuda")
            rid = srv.submit_spmv_iter(ids[g], x, steps=5)
            xs[rid] = x
            reqs.append((rid, "spmv", g, None))
        if i % 50 == 49:
            time.sleep(0.002)  # let some requests complete while others arrive
    done = srv.wait(timeout=120)
    assert len(done) == len(reqs)
    for rid, kind, g, s in reqs:
        got, lat = done[rid]
        assert lat >= 0
        if kind == "bfs":
            assert torch.equal(got, G.bfs_distances(gs[g], s))
        elif kind == "sssp":
            assert torch.equal(got, G.shortest_path(gs[g], s))
    # SpMV iterations: alone on a fresh server == in the mix; close to FP64
    alone = Server(reserve_bytes=0)
    a_id = alone.add_graph(gs[3])
    A = gs[3].to_scipy().astype(np.float64)
    for rid, x in list(xs.items())[:5]:
        r = alone.submit_spmv_iter(a_id, x, steps=5)
        got_alone = alone.wait(timeout=60)[r][0]
        assert torch.equal(got_alone, done[rid][0])
        ref = x.double().cpu().numpy()
        for _ in range(5):
            ref = A @ ref
        np.testing.assert_allclose(done[rid][0].cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
    st = srv.stats()
    assert st["ticks"] > 0 and st["executor_bytes"] > 0
    srv.close()
    alone.close()


def test_server_admission_waits_for_memory():
    """An executor is not created while free HBM is below its need plus the reserve;
    its requests stay queued (they are served once memory allows)."""
    A = gen.rmat(10, 8, seed=46, wkind=gen.W_PATTERN)
    free, total = torch.cuda.mem_get_info()
    srv = Server(reserve_bytes=free * 2)  # can never be satisfied
    g = srv.add_graph(A)
    srv.submit_bfs(g, 1)
    time.sleep(0.3)
    d, infl = srv.poll()
    assert not d and infl == 1 and srv.stats()["admission_waits"] > 0
    srv.close()


import time  # noqa: E402


def test_server_large_graph_shortest_paths_equal_single():
    """Graphs of at least 65536 vertices: the shortest-path executors' rounds over every
    vertex run on the graph's SELL-32 copy (Int32 and Float32 weights); 40 queries per
    graph, submitted in bursts, each equal to the single-query result."""
    gs = [gen.rmat(16, 16, seed=47, wkind=gen.W_INT_1_255),
          gen.rmat(16, 8, seed=48, wkind=gen.W_F32_1_10)]
    srv = Server(reserve_bytes=0)
    ids = [srv.add_graph(A) for A in gs]
    rng = np.random.default_rng(49)
    reqs = []
    for i in range(80):
        g = i % 2
        s = int(rng.integers(1, gs[g].n + 1))
        reqs.append((srv.submit_sssp(ids[g], s), g, s))
        if i % 20 == 19:
            time.sleep(0.003)
    done = srv.wait(timeout=120)
    assert len(done) == len(reqs)
    for rid, g, s in reqs:
        assert torch.equal(done[rid][0], G.shortest_path(gs[g], s)), (g, s)
    srv.close()

