"""Launch tracer: counts the kernels of SpMV / SpMM calls and times their main kernel
with CUDA events."""
import numpy as np
import pytest
import torch

import gpugraphs as G
from gpugraphs.tracing import launch_trace
from helpers import sprand_csr

pytestmark = pytest.mark.gpu


def test_trace_counts_and_times_spmv_spmm():
    m = 3000
    rowptr, colval, nzval, _ = sprand_csr(m, m, 0.01, seed=61)
    A = G.SparseGPUMatrixCSR(m, m, rowptr, colval, nzval)
    x = torch.rand(m, device="cuda")
    y = torch.zeros(m, device="cuda")
    G.gpu_spmv_(y, A, x)  # analysis outside the traced region
    with launch_trace() as t:
        for _ in range(5):
            G.gpu_spmv_(y, A, x)
    assert t.launches == 5 and t.timed == 5 and t.kernel_ms > 0
    B = torch.rand((m, 8), device="cuda")
    C = torch.zeros((m, 8), device="cuda")
    with launch_trace() as t:
        G.gpu_spmm_(C, A, B)
    assert t.launches >= 1 and t.timed == 1
    # outside a trace nothing is counted
    with launch_trace() as t:
        pass
    assert t.launches == 0 and t.timed == 0
