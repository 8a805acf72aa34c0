"""Writes the golden fixtures under tests/golden/ (run from the repository root:
``python tests/golden/make_golden.py``).

* sell_4x4.json -- the reference's own SELL layout known answer, transcribed from
  GPUGraphs.jl test/structs.jl:176-190 (4x4 matrix, expected slice_ptr / colval /
  nzval with -1 / 0 padding).
* csr_errors.json -- the constructor cases the reference expects to throw
  ArgumentError, transcribed from test/structs.jl:79-149.
* reference_exports.json -- the names the reference module exports
  (src/GPUGraphs.jl:25-51), which the Julia drop-in must export too.
* graphs.npz -- the reference's BFS / shortest-path test graphs rebuilt with the same
  generator families (test/bfs.jl:11-12, test/shortest_path.jl:10-29):
  Barabasi-Albert(30, 3) and Dorogovtsev-Mendes(30), seeded, plus integer weights
  1..10, with expected hop distances (Graphs.gdistances) and weighted distances
  (dijkstra_shortest_paths) from every source computed by networkx.  Julia's RNG
  streams cannot be reproduced here, so the instances differ from the reference's
  while the generators, the checks and the expected-value oracles are the same.
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def sell_4x4():
    return {
        "source": "GPUGraphs.jl test/structs.jl:176-190",
        "dense": [[1, 7, 0, 0], [5, 0, 3, 9], [0, 2, 8, 0], [0, 0, 0, 6]],
        "nnz": 8,
        "slice_ptr": [1, 13],
        "colval": [1, 1, 2, 4, 2, 3, 3, -1, -1, 4, -1, -1],
        "nzval": [1, 5, 2, 6, 7, 3, 8, 0, 0, 9, 0, 0],
    }


def csr_errors():
    cols = list(range(1, 11))
    return {
        "source": "GPUGraphs.jl test/structs.jl:79-149",
        "cases": [
            {"m": 3, "n": 10, "rowptr": [1, 4, 7, 11], "colval": cols, "nzval": cols + [1]},
            {"m": 3, "n": 10, "rowptr": [1, 4, 7, 11], "colval": cols, "nzval": cols[:9]},
            {"m": 4, "n": 10, "rowptr": [1, 4, 7, 11], "colval": cols, "nzval": cols},
            {"m": 2, "n": 10, "rowptr": [1, 4, 7, 11], "colval": cols, "nzval": cols},
            {"m": 3, "n": 10, "rowptr": [-1, 4, 7, 11], "colval": cols, "nzval": cols},
            {"m": 3, "n": 10, "rowptr": [1, 4, 7, 12], "colval": cols, "nzval": cols},
            {"m": 3, "n": 10, "rowptr": [1, 4, 7, 12], "colval": cols[:9] + [15], "nzval": cols},
        ],
    }


def dorogovtsev_mendes(n, rng):
    """Graphs.jl dorogovtsev_mendes: start from a triangle; every new vertex joins
    both ends of a uniformly chosen existing edge."""
    edges = [(0, 1), (1, 2), (0, 2)]
    for v in range(3, n):
        a, b = edges[rng.integers(len(edges))]
        edges.append((a, v))
        edges.append((b, v))
    return edges


def graphs():
    import networkx as nx

    rng = np.random.default_rng(1234)
    out = {}
    ba = nx.barabasi_albert_graph(30, 3, seed=1234)
    dm = nx.Graph()
    dm.add_edges_from(dorogovtsev_mendes(30, rng))
    for name, g in (("ba30", ba), ("dm30", dm)):
        n = g.number_of_nodes()
        e = np.array(sorted((min(u, v), max(u, v)) for u, v in g.edges()), np.int32)
        w = rng.integers(1, 11, len(e)).astype(np.int32)
        hop = np.zeros((n, n), np.int32)
        wd = np.zeros((n, n), np.int32)
        gw = nx.Graph()
        gw.add_nodes_from(range(n))
        for (u, v), ww in zip(e, w):
            gw.add_edge(int(u), int(v), weight=int(ww))
        for s in range(n):
            d = nx.single_source_shortest_path_length(g, s)
            dd = nx.single_source_dijkstra_path_length(gw, s)
            for t in range(n):
                hop[t, s] = d.get(t, np.iinfo(np.int32).max)
                wd[t, s] = dd.get(t, np.iinfo(np.int32).max)
        out[name + "_edges"] = e + 1  # 1-based undirected edge list
        out[name + "_w"] = w
        out[name + "_hop"] = hop      # hop[:, s-1] = gdistances(g, s)
        out[name + "_dijkstra"] = wd  # wd[:, s-1] = dijkstra_shortest_paths(g_w, s).dists
    return out


def reference_exports():
    """The names GPUGraphs.jl exports (src/GPUGraphs.jl:25-51), transcribed: the drop-in
    module must export every one of them."""
    return {
        "source": "GPUGraphs.jl src/GPUGraphs.jl:25-51",
        "exports": [
            "AbstractSparseGPUMatrix", "SparseGPUMatrixCSR", "SparseGPUMatrixCSC",
            "SparseGPUMatrixSELL", "SparseGPUVector", "AbstractSparseGPUVector", "gpu_spmv!",
            "gpu_spmm!", "sprand_gpu", "monoid_neutral", "monoid_absorb", "bfs_distances",
            "bfs_distances!", "bfs_parents", "bfs_parents!", "shortest_path", "shortest_path!",
            "GPUGraphs_add", "GPUGraphs_safe_add", "GPUGraphs_mul", "GPUGraphs_second",
            "GPUGraphs_band", "GPUGraphs_bor", "GPUGraphs_any", "GPUGraphs_secondi",
            "GPUGraphs_max", "GPUGraphs_min",
        ],
    }


def main():
    with open(os.path.join(HERE, "sell_4x4.json"), "w") as f:
        json.dump(sell_4x4(), f, indent=1)
    with open(os.path.join(HERE, "reference_exports.json"), "w") as f:
        json.dump(reference_exports(), f, indent=1)
    with open(os.path.join(HERE, "csr_errors.json"), "w") as f:
        json.dump(csr_errors(), f, indent=1)
    np.savez_compressed(os.path.join(HERE, "graphs.npz"), **graphs())


if __name__ == "__main__":
    main()
