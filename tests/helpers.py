"""Shared helpers for the tests: seeded sparse inputs in the reference's CSR form
(1-based Int32 rowptr / colval) and golden-fixture loaders."""
import json
import os

import numpy as np
import scipy.sparse as sp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sprand_csr(m, n, p, dtype=np.float32, seed=0, values=None):
    """Seeded equivalent of SparseArrays.sprand(T, m, n, p) as a 1-based CSR triple
    (rowptr, colval, nzval) plus the scipy matrix."""
    rng = np.random.default_rng(seed)
    A = sp.random(m, n, density=p, format="csr", random_state=rng, dtype=np.float64)
    A.sort_indices()
    if values is not None:
        A.data = values(rng, A.nnz)
    A = A.astype(dtype)
    rowptr = (A.indptr + 1).astype(np.int32)
    colval = (A.indices + 1).astype(np.int32)
    nzval = np.ascontiguousarray(A.data.astype(dtype))
    return rowptr, colval, nzval, A


def csr_from_scipy(A):
    A = sp.csr_matrix(A)
    A.sort_indices()
    return ((A.indptr + 1).astype(np.int32), (A.indices + 1).astype(np.int32),
            np.ascontiguousarray(A.data))


def undirected_csr(edges1, n, weights=None, dtype=np.int32):
    """Symmetric adjacency (A == A_T) of a 1-based undirected edge list."""
    e = np.asarray(edges1) - 1
    w = np.ones(len(e)) if weights is None else np.asarray(weights)
    r = np.concatenate([e[:, 0], e[:, 1]])
    c = np.concatenate([e[:, 1], e[:, 0]])
    v = np.concatenate([w, w]).astype(dtype)
    A = sp.csr_matrix((v, (r, c)), shape=(n, n))
    return csr_from_scipy(A)


def golden_graphs():
    return dict(np.load(os.path.join(GOLDEN, "graphs.npz")))


def golden_json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def bfs_levels_scipy(rowptr, colval, n, source):
    """Hop distances along in-edges of A_T (row v lists in-neighbours of v), i.e.
    along out-edges of A, computed by scipy.sparse.csgraph; unreachable = Int32 max."""
    from scipy.sparse.csgraph import breadth_first_order, shortest_path

    data = np.ones(len(colval))
    AT = sp.csr_matrix((data, colval - 1, rowptr - 1), shape=(n, n))
    A = AT.T.tocsr()
    d = shortest_path(A, method="D", unweighted=True, indices=source - 1)
    out = np.full(n, np.iinfo(np.int32).max, np.int64)
    fin = np.isfinite(d)
    out[fin] = d[fin].astype(np.int64)
    return out.astype(np.int32)
