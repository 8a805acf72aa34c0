"""Seeded synthetic graphs built on the device: the inputs of the benchmark configs
(Erdos-Renyi, R-MAT, 4-neighbour grid) as SparseGPUMatrixCSR.

Edges come from the library's counter-based generators (gg_gen_*_edges); assembly
into CSR keeps generation order: entries (src, dst) of edge e, then its mirror
(dst, src) when symmetrising, optionally without self-loops, stably sorted by (row,
column) with the first duplicate kept, so mirrored weights stay symmetric."""
import ctypes

import torch

from . import core
from .errors import check
from .storage import SparseGPUMatrixCSR

W_PATTERN, W_U01_F32, W_INT_1_255, W_F32_1_10 = 0, 1, 2, 3
_WDT = {W_PATTERN: torch.bool, W_U01_F32: torch.float32, W_INT_1_255: torch.int32,
        W_F32_1_10: torch.float32}


def _edges(kind, ne, wkind, device, fill):
    src = torch.empty(ne, dtype=torch.int32, device=device)
    dst = torch.empty(ne, dtype=torch.int32, device=device)
    w = torch.empty(ne, dtype=_WDT[wkind], device=device)
    L = core.lib()
    with torch.cuda.device(device):
        c = core.ctx(device)
        check(fill(L, c, src, dst, w), L)
    return src, dst, w


def rmat_edges(scale, nedges, a=0.57, b=0.19, c=0.19, seed=1, wkind=W_U01_F32, device="cuda"):
    dev = torch.device(device)
    return _edges("rmat", nedges, wkind, dev, lambda L, cx, s, d, w: L.gg_gen_rmat_edges(
        cx, scale, nedges, a, b, c, seed, wkind, core.ptr(s), core.ptr(d), core.ptr(w)))


def er_edges(n, nedges, seed=1, wkind=W_U01_F32, device="cuda"):
    dev = torch.device(device)
    return _edges("er", nedges, wkind, dev, lambda L, cx, s, d, w: L.gg_gen_er_edges(
        cx, n, nedges, seed, wkind, core.ptr(s), core.ptr(d), core.ptr(w)))


def grid_edges(H, W, seed=1, wkind=W_F32_1_10, device="cuda"):
    dev = torch.device(device)
    ne = H * (W - 1) + (H - 1) * W
    return _edges("grid", ne, wkind, dev, lambda L, cx, s, d, w: L.gg_gen_grid_edges(
        cx, H, W, seed, wkind, core.ptr(s), core.ptr(d), core.ptr(w)))


def assemble_csr(n, src, dst, w, symmetrize, drop_loops):
    """(rowptr, colval, nzval) device tensors, 1-based, by the assembly rule above."""
    if symmetrize:
        rows = torch.stack([src, dst], 1).reshape(-1)
        cols = torch.stack([dst, src], 1).reshape(-1)
        vals = torch.stack([w, w], 1).reshape(-1)
    else:
        rows, cols, vals = src, dst, w
    if drop_loops:
        keep = rows != cols
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
    key = ((rows.to(torch.int64) - 1) << 32) | (cols.to(torch.int64) - 1)
    del rows, cols
    key, order = torch.sort(key, stable=True)
    first = torch.ones_like(key, dtype=torch.bool)
    if key.numel() > 1:
        first[1:] = key[1:] != key[:-1]
    key = key[first]
    vals = vals[order[first]]
    del order, first
    r = (key >> 32).to(torch.int64)
    counts = torch.bincount(r, minlength=n)
    rowptr = torch.empty(n + 1, dtype=torch.int32, device=key.device)
    rowptr[0] = 1
    rowptr[1:] = (torch.cumsum(counts, 0) + 1).to(torch.int32)
    colval = ((key & 0xFFFFFFFF) + 1).to(torch.int32)
    return rowptr, colval, vals.contiguous()


def _csr(n, src, dst, w, symmetrize, drop_loops):
    rowptr, colval, nzval = assemble_csr(n, src, dst, w, symmetrize, drop_loops)
    del src, dst, w
    return SparseGPUMatrixCSR(n, n, rowptr, colval, nzval, device=rowptr.device)


def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, wkind=W_U01_F32,
         symmetrize=True, drop_loops=True, device="cuda"):
    """R-MAT graph with 2^scale vertices and edge_factor * 2^scale generated edges."""
    n = 1 << scale
    s, d, w = rmat_edges(scale, edge_factor * n, a, b, c, seed, wkind, device)
    return _csr(n, s, d, w, symmetrize, drop_loops)


def erdos_renyi(n, avg_degree=16, seed=1, wkind=W_U01_F32, symmetric=False, device="cuda"):
    """Erdos-Renyi graph with avg_degree * n uniform edges, duplicates merged (first
    kept): directed with self-loops kept, or (symmetric=True) undirected -- each edge
    mirrored, self-loops dropped, about 2 * avg_degree entries per row."""
    s, d, w = er_edges(n, int(round(avg_degree * n)), seed, wkind, device)
    return _csr(n, s, d, w, symmetric, symmetric)


def grid(H, W, seed=1, wkind=W_F32_1_10, device="cuda"):
    """H x W 4-neighbour grid, weights per undirected edge, mirrored."""
    s, d, w = grid_edges(H, W, seed, wkind, device)
    return _csr(H * W, s, d, w, True, False)


def uniform_vector(n, seed=2, device="cuda"):
    """Float32 vector, element i uniform [0, 1) (gg_gen_uniform_f32)."""
    dev = torch.device(device)
    out = torch.empty(n, dtype=torch.float32, device=dev)
    L = core.lib()
    with torch.cuda.device(dev):
        check(L.gg_gen_uniform_f32(core.ctx(dev), n, seed, core.ptr(out)), L)
    return out
