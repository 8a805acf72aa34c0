"""Launch tracing of the SpMV / SpMM calls (gg_trace_begin / gg_trace_end).

    with launch_trace() as t:
        for _ in range(k):
            gpu_spmv_(y, A, x)
    t.launches      # kernel launches made by those calls
    t.timed         # calls whose main kernel was bracketed by CUDA events
    t.kernel_ms     # summed device time of those main kernels
"""
import ctypes

from . import core
from .errors import check


class launch_trace:
    def __init__(self, device=None):
        self.device = device
        self.launches = self.timed = 0
        self.kernel_ms = 0.0

    def __enter__(self):
        L = core.lib()
        check(L.gg_trace_begin(core.ctx(self.device)), L)
        return self

    def __exit__(self, *exc):
        L = core.lib()
        n, t, ms = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        check(L.gg_trace_end(core.ctx(self.device), ctypes.byref(n), ctypes.byref(t),
                             ctypes.byref(ms)), L)
        self.launches, self.timed, self.kernel_ms = n.value, t.value, ms.value
        return False
