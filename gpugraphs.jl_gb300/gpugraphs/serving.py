"""Continuous-batching query server over resident graphs (gg_server_* in the C ABI).

    srv = Server()
    g = srv.add_graph(A_T)
    rid = srv.submit_bfs(g, source)        # or submit_sssp / submit_spmv_iter
    done = srv.wait(timeout=10)            # {request id: (result tensor, latency s)}

BFS results are Int32 levels (typemax(Int32) unreached), shortest-path results have
shortest_path's element type, SpMV-iteration results are Float32 `steps`-fold
products.  Each result equals the single-query function's."""
import ctypes
import time

import numpy as np
import torch

from . import core
from .algorithms import dist_dtype
from .errors import ArgumentError, check

BFS, SSSP, SPMV_ITER = 1, 2, 3


class Server:
    def __init__(self, reserve_bytes=1 << 30, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        L = core.lib()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(L.gg_server_create(core.ctx(self.device), int(reserve_bytes), ctypes.byref(h)), L)
        self._h = h
        self._graphs = []
        self._pending = {}  # id -> (out tensor, keep-alive refs)

    def add_graph(self, A_T):
        L = core.lib()
        gid = ctypes.c_int()
        check(L.gg_server_add_graph(self._h, A_T.handle, ctypes.byref(gid)), L)
        self._graphs.append(A_T)
        return gid.value

    def _submit(self, kind, graph, source, x, steps, out, keep):
        L = core.lib()
        rid = ctypes.c_int64()
        check(L.gg_server_submit(self._h, kind, graph, int(source),
                                 core.ptr(x) if x is not None else None, int(steps),
                                 core.ptr(out), ctypes.byref(rid)), L)
        self._pending[rid.value] = (out, keep)
        return rid.value

    def submit_bfs(self, graph, source):
        A = self._graphs[graph]
        out = torch.empty(A.n, dtype=torch.int32, device=self.device)
        return self._submit(BFS, graph, source, None, 0, out, None)

    def submit_sssp(self, graph, source):
        A = self._graphs[graph]
        out = torch.empty(A.n, dtype=dist_dtype(A), device=self.device)
        return self._submit(SSSP, graph, source, None, 0, out, None)

    def submit_spmv_iter(self, graph, x, steps=20):
        A = self._graphs[graph]
        if x.dtype != torch.float32 or x.numel() != A.n or not x.is_cuda:
            raise ArgumentError("x must be a Float32 CUDA vector of length n")
        x = x.contiguous()
        torch.cuda.current_stream(self.device).synchronize()  # x is read on the server stream
        out = torch.empty(A.n, dtype=torch.float32, device=self.device)
        return self._submit(SPMV_ITER, graph, 0, x, steps, out, x)

    def poll(self, max_n=4096):
        L = core.lib()
        ids = (ctypes.c_int64 * max_n)()
        lat = (ctypes.c_double * max_n)()
        nd, infl = ctypes.c_int64(), ctypes.c_int64()
        check(L.gg_server_poll(self._h, ids, lat, max_n, ctypes.byref(nd), ctypes.byref(infl)), L)
        out = {}
        for i in range(nd.value):
            t, _ = self._pending.pop(ids[i])
            out[ids[i]] = (t, lat[i])
        return out, infl.value

    def wait(self, timeout=60.0, poll_interval=0.0002):
        done = {}
        t_end = time.time() + timeout
        while True:
            d, infl = self.poll()
            done.update(d)
            if infl == 0 and not self._pending:
                return done
            if time.time() > t_end:
                raise TimeoutError("%d requests still in flight" % infl)
            time.sleep(poll_interval)

    def stats(self):
        L = core.lib()
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(L.gg_server_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), L)
        return {"ticks": a.value, "admission_waits": b.value, "executor_bytes": c.value}

    def close(self):
        if self._h is not None:
            core.lib().gg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
