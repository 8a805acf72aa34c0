"""gg_bfs_levels_noalloc: BFS levels for callers that cannot allocate device memory
(a host whose allocator owns the whole device, or code that must avoid the
allocator's implicit synchronisation).  It must give exactly what gg_bfs_levels
gives, call after call, although every call reuses the same fixed scratch array.

This file is collected last on purpose: when it fails, a run that stops at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import torch

import gpugraphs as G
from gpugraphs import _lib, core
from gpugraphs import generators as gen

pytestmark = pytest.mark.gpu
I32MAX = np.iinfo(np.int32).max


def _noalloc(A, source, dist):
    L = _lib.load()
    lv = ctypes.c_int64()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.gg_bfs_levels_noalloc(core.ptr(A.rowptr), core.ptr(A.colval), core.ptr(A.nzval),
                                 A.dtype_code, A.n, A.nnz(), source, core.ptr(dist), stream,
                                 ctypes.byref(lv))
    return rc, lv.value


def _graphs():
    out = [gen.rmat(14, 16, seed=21, wkind=gen.W_PATTERN), gen.grid(64, 48, seed=22, wkind=gen.W_PATTERN)]
    rng = np.random.default_rng(23)
    n = 3000
    A = sp.random(n, n, density=0.002, random_state=rng, format="csr")
    A.data = rng.integers(1, 5, A.nnz).astype(np.int32)  # even values are inactive edges
    out.append(G.SparseGPUMatrixCSR.from_scipy(A.T.tocsr(), dtype=np.int32))
    return out


def test_noalloc_matches_bfs_levels_twice():
    for A in _graphs():
        deg = np.diff(A.rowptr.cpu().numpy())
        for s in (int(np.argmax(deg)) + 1, 1):
            ref = G.bfs_distances(A, s)
            torch.cuda.synchronize()
            for _ in range(2):  # the shared scratch keeps the last call's contents
                d = torch.full((A.n,), I32MAX, dtype=torch.int32, device="cuda")
                rc, lv = _noalloc(A, s, d)
                assert rc == 0, _lib.load().gg_last_error()
                torch.cuda.synchronize()
                assert torch.equal(d, ref)


def test_noalloc_rejects_oversize():
    L = _lib.load()
    d = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.gg_bfs_levels_noalloc(core.ptr(d), core.ptr(d), None, 1, 4194305, 0, 1, core.ptr(d),
                                 None, None)
    assert rc == 2 and b"capacity" in L.gg_last_error()
