"""Many independent graphs processed by single launches (gg_multigraph_* in the C ABI).

    mg = MultiGraph([A1, A2, ...])          # square CSR graphs of one element type
    y = mg.spmv(x)                          # y_g = A_g x_g for all graphs, one launch
    d = mg.bfs([s1, s2, ...])               # one BFS per graph, one persistent launch
    D = mg.sssp([s1, s2, ...])              # one shortest-path search per graph
    parts = mg.split(d)                     # per-graph views of a concatenated vector
"""
import ctypes

import numpy as np
import torch

from . import core
from .errors import ArgumentError, check


class MultiGraph:
    def __init__(self, graphs):
        if not graphs:
            raise ArgumentError("need at least one graph")
        self.device = graphs[0].device
        self.dtype_code = graphs[0].dtype_code
        L = core.lib()
        arr = (ctypes.c_void_p * len(graphs))(*[g.handle.value for g in graphs])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(L.gg_multigraph_create(core.ctx(self.device), arr, len(graphs), ctypes.byref(h)), L)
        self._h = h
        G, n, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        off = np.zeros(len(graphs) + 1, np.int64)
        check(L.gg_multigraph_info(h, ctypes.byref(G), ctypes.byref(n), ctypes.byref(nnz),
                                   off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))), L)
        self.ngraphs, self.total_n, self.total_nnz = G.value, n.value, nnz.value
        self.offsets = off

    def spmv(self, x, y=None):
        """y_g = A_g * x_g (plus-times Float32) for every graph in one launch."""
        if y is None:
            y = torch.empty(self.total_n, dtype=torch.float32, device=self.device)
        L = core.lib()
        with torch.cuda.device(self.device):
            check(L.gg_multigraph_spmv(core.ctx(self.device), self._h, core.ptr(x), core.ptr(y)), L)
        return y

    def bfs(self, sources, dist=None):
        """BFS levels of every graph from its source (1-based within the graph)."""
        src = np.ascontiguousarray(np.asarray(sources, dtype=np.int64))
        if len(src) != self.ngraphs:
            raise ArgumentError("one source per graph")
        if dist is None:
            dist = torch.empty(self.total_n, dtype=torch.int32, device=self.device)
        L = core.lib()
        lv = ctypes.c_int64()
        with torch.cuda.device(self.device):
            check(L.gg_multigraph_bfs(core.ctx(self.device), self._h,
                                      src.ctypes.data_as(ctypes.c_void_p), core.ptr(dist),
                                      ctypes.byref(lv)), L)
        self.last_levels = lv.value
        return dist

    def sssp(self, sources, dist=None):
        """Shortest-path distances of every graph from its source (1-based within the
        graph), element type as shortest_path (Int32 for Bool graphs)."""
        src = np.ascontiguousarray(np.asarray(sources, dtype=np.int64))
        if len(src) != self.ngraphs:
            raise ArgumentError("one source per graph")
        code = core.INT32 if self.dtype_code == core.BOOL else self.dtype_code
        if dist is None:
            dist = torch.empty(self.total_n, dtype=core.CODE2TORCH[code], device=self.device)
        L = core.lib()
        r = ctypes.c_int64()
        with torch.cuda.device(self.device):
            check(L.gg_multigraph_sssp(core.ctx(self.device), self._h,
                                       src.ctypes.data_as(ctypes.c_void_p), core.ptr(dist),
                                       core.dtype_code(dist.dtype), ctypes.byref(r)), L)
        self.last_rounds = r.value
        return dist

    def split(self, v):
        return [v[self.offsets[g]:self.offsets[g + 1]] for g in range(self.ngraphs)]

    def close(self):
        if self._h is not None:
            core.lib().gg_multigraph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
