"""BFS and shortest paths of GPUGraphs.jl (src/algorithms/bfs.jl,
src/algorithms/shortest_path.jl) over libgpugraphs.

All functions take A_T, the transposed adjacency matrix (row v lists the
in-neighbours of v), and 1-based vertex ids, as the reference does.  Results are
torch tensors on A_T's device: Int32 levels / parents (typemax(Int32) = unreached),
and distances of type Int32 for Bool matrices, else eltype(A_T)."""
import ctypes

import numpy as np
import torch

from . import core
from .errors import ArgumentError, check
from .storage import AbstractSparseGPUMatrix

INT32_MAX = np.iinfo(np.int32).max
PARENT_FORMAT_DEFAULT, PARENT_FIRST_IN_ROW, PARENT_MAX_INDEX = 0, 1, 2


def _check_matrix(A_T):
    if not isinstance(A_T, AbstractSparseGPUMatrix):
        raise ArgumentError("A_T must be a SparseGPUMatrixCSR or SparseGPUMatrixSELL")


def _vec_i32(t, n, name):
    core.device_vector(t, name)
    if t.dtype != torch.int32 or t.numel() != n:
        raise ArgumentError("%s must be an Int32 vector of length %d" % (name, n))
    return t


def bfs_distances_(A_T, source, dist, curr=None, next=None, to_explore=None):
    """bfs_distances!(A_T, source, dist, curr, next, to_explore) (bfs.jl:31-73):
    writes the hop level of every vertex reached from `source` into dist; other
    entries are left as they are.  The work vectors of the reference are accepted
    for signature compatibility; the library keeps its own frontier state.
    Returns the number of levels searched."""
    _check_matrix(A_T)
    n = A_T.size(1)
    _vec_i32(dist, n, "dist")
    L = core.lib()
    lv = ctypes.c_int64()
    with torch.cuda.device(A_T.device):
        check(L.gg_bfs_levels(core.ctx(A_T.device), A_T.handle, int(source), core.ptr(dist), n,
                              ctypes.byref(lv)), L)
    return lv.value


def bfs_distances(A_T, source, use_mask=True):
    """bfs_distances(A_T, source; use_mask) (bfs.jl:1-29): Int32 hop levels from
    `source` (0 at the source, typemax(Int32) when unreached).  An edge counts when
    its stored value is odd / true, like the reference's band semiring."""
    _check_matrix(A_T)
    dist = torch.full((A_T.size(1),), INT32_MAX, dtype=torch.int32, device=A_T.device)
    bfs_distances_(A_T, source, dist)
    return dist


def bfs_distances_batch(A_T, sources):
    """Batched bfs_distances: an n x S column-major Int32 matrix whose column q is
    bfs_distances(A_T, sources[q]).  Up to 256 sources share each pass over the graph
    (gg_bfs_levels_batch); the reference has no multi-source BFS."""
    _check_matrix(A_T)
    n = A_T.size(1)
    src = _sources(sources)
    dist = torch.empty((len(src), n), dtype=torch.int32, device=A_T.device).T
    L = core.lib()
    lv = ctypes.c_int64()
    with torch.cuda.device(A_T.device):
        check(L.gg_bfs_levels_batch(core.ctx(A_T.device), A_T.handle,
                                    src.ctypes.data_as(ctypes.c_void_p), len(src), core.ptr(dist),
                                    n, ctypes.byref(lv)), L)
    return dist


def bfs_parents_(A_T, source, parents, curr=None, next=None, to_explore=None, batch_size=8,
                 rule=PARENT_FORMAT_DEFAULT):
    """bfs_parents!(A_T, source, parents, curr, next, to_explore, batch_size)
    (bfs.jl:135-183): parents[source] = 0, reached vertices get a 1-based parent (the
    first frontier in-neighbour in storage order for CSR, the largest for SELL)."""
    _check_matrix(A_T)
    n = A_T.size(1)
    _vec_i32(parents, n, "parents")
    L = core.lib()
    lv = ctypes.c_int64()
    with torch.cuda.device(A_T.device):
        check(L.gg_bfs_parents(core.ctx(A_T.device), A_T.handle, int(source), core.ptr(parents), n,
                               int(rule), ctypes.byref(lv)), L)
    return lv.value


def bfs_parents(A_T, source, batch_size=8, rule=PARENT_FORMAT_DEFAULT):
    """bfs_parents(A_T, source; batch_size) (bfs.jl:113-133)."""
    _check_matrix(A_T)
    parents = torch.full((A_T.size(1),), INT32_MAX, dtype=torch.int32, device=A_T.device)
    bfs_parents_(A_T, source, parents, batch_size=batch_size, rule=rule)
    return parents


def dist_dtype(A_T):
    """T_dist = Int32 for Bool matrices, else eltype(A_T) (shortest_path.jl:18)."""
    return torch.int32 if A_T.dtype == torch.bool else A_T.dtype


def _sources(source):
    if isinstance(source, torch.Tensor):
        source = source.cpu().numpy()
    s = np.atleast_1d(np.asarray(source, dtype=np.int64))
    return np.ascontiguousarray(s)


def _sssp(A_T, sources, dist, next_, ld):
    L = core.lib()
    rounds = ctypes.c_int64()
    with torch.cuda.device(A_T.device):
        check(L.gg_sssp(core.ctx(A_T.device), A_T.handle,
                        sources.ctypes.data_as(ctypes.c_void_p), len(sources), core.ptr(dist),
                        core.ptr(next_) if next_ is not None else None,
                        core.dtype_code(dist_dtype(A_T)), ld, ctypes.byref(rounds)), L)
    return rounds.value


def _column_major(t, n, S):
    """True when t is an n x S column-major (or length-n) tensor."""
    if t.dim() == 1:
        return t.numel() == n and S == 1 and t.is_contiguous()
    return t.shape == (n, S) and t.stride() == (1, n)


def shortest_path(A_T, source):
    """shortest_path(A_T, source) / shortest_path(A_T, sources)
    (shortest_path.jl:12-32, :88-110): Bellman-Ford distances.  A vector of sources
    gives an n x S column-major matrix, column i for sources[i]."""
    _check_matrix(A_T)
    n = A_T.size(1)
    multi = not np.isscalar(source) and not (isinstance(source, torch.Tensor) and source.dim() == 0)
    src = _sources(source)
    S = len(src)
    dt = dist_dtype(A_T)
    dist = torch.empty((S, n), dtype=dt, device=A_T.device).T  # column-major n x S
    _sssp(A_T, src, dist, None, n)
    return dist if multi else dist[:, 0]


def shortest_path_(A_T, source, dist, next, updated=None, diff=None):
    """shortest_path!(A_T, source(s), dist, next, updated, diff)
    (shortest_path.jl:34-83, :112-161): starts from the caller's dist / next
    (typemax except at the sources, as shortest_path allocates them), leaves the
    distances in both.  Returns the number of relaxation rounds."""
    _check_matrix(A_T)
    n = A_T.size(1)
    src = _sources(source)
    S = len(src)
    dt = dist_dtype(A_T)
    for t, name in ((dist, "dist"), (next, "next")):
        core.device_vector(t.T if t.dim() == 2 else t, name)
        if t.dtype != dt or not _column_major(t, n, S):
            raise ArgumentError("%s must be a column-major %s array of size (%d, %d)" % (name, dt, n, S))
    return _sssp(A_T, src, dist, next, n)
