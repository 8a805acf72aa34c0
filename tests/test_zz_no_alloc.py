"""gg_bfs_levels_noalloc: BFS levels for callers that cannot allocate device memory
(a host whose allocator owns the whole device, or code that must avoid the
allocator's implicit synchronisation).  It must give exactly what gg_bfs_levels
gives -- the levels, the level count and the oracle's levels -- call after call,
although every call reuses the same fixed scratch array, and it must not change the
device's free memory.

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
from oracle import oracle as O

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


def _levels(A, source, dist):
    """gg_bfs_levels on the library's context: (status, level count)."""
    L = _lib.load()
    lv = ctypes.c_int64()
    rc = L.gg_bfs_levels(core.ctx(), A.handle, source, core.ptr(dist), dist.numel(),
                         ctypes.byref(lv))
    torch.cuda.synchronize()
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
        rp, cv, nz = A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy()
        deg = np.diff(rp)
        for s in (int(np.argmax(deg)) + 1, 1):
            ref = torch.full((A.n,), I32MAX, dtype=torch.int32, device="cuda")
            rc, ref_levels = _levels(A, s, ref)
            assert rc == 0, _lib.load().gg_last_error()
            oracle, oracle_levels = O.bfs_levels(A.n, rp, cv, nz, s)
            assert (ref.cpu().numpy() == oracle).all()
            assert ref_levels == oracle_levels  # iterations of bfs.jl:50-71, the last empty
            for _ in range(2):  # the shared scratch keeps the last call's contents
                d = torch.full((A.n,), I32MAX, dtype=torch.int32, device="cuda")
                rc, lv = _noalloc(A, s, d)
                assert rc == 0, _lib.load().gg_last_error()
                torch.cuda.synchronize()
                assert torch.equal(d, ref)
                assert (d.cpu().numpy() == oracle).all()
                assert lv == ref_levels


def test_noalloc_leaves_free_memory_unchanged():
    """After a first call (which may load the library's device code), repeated calls
    change the device's free memory by nothing: no allocation, no pool growth."""
    A = _graphs()[0]
    dists = [torch.full((A.n,), I32MAX, dtype=torch.int32, device="cuda") for _ in range(4)]
    rc, _ = _noalloc(A, 1, dists[0])
    assert rc == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for d in dists[1:]:
        rc, _ = _noalloc(A, 1, d)
        assert rc == 0
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0
    for d in dists[1:]:
        assert torch.equal(d, dists[0])


def test_noalloc_rejects_oversize():
    L = _lib.load()
    d = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.gg_bfs_levels_noalloc(core.ptr(d), core.ptr(d), None, 1, 4194305, 0, 1, core.ptr(d),
                                 None, None)
    assert rc == 2 and b"capacity" in L.gg_last_error()
