"""Argument checks of the Python host mirror that run before any device work (no GPU):
the reference's ArgumentError / DimensionMismatch cases for the sparse-vector, CSC and
e-wise entry points."""
import numpy as np
import pytest
import torch

import gpugraphs as G


def test_sparse_vector_lengths_must_agree():
    # GPUGraphsVector.jl:38-40
    with pytest.raises(G.ArgumentError):
        G.SparseGPUVector(10, [1, 2, 3], np.ones(2, np.float32))


def test_csc_constructor_checks_run_first():
    # colptr must have n + 1 entries; rowval and nzval the same length
    with pytest.raises(G.ArgumentError):
        G.SparseGPUMatrixCSC(4, 3, np.ones(3, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    with pytest.raises(G.ArgumentError):
        G.SparseGPUMatrixCSC(4, 3, np.array([1, 2, 2, 2], np.int32), np.array([1], np.int32),
                             np.zeros(2, np.float32))


def test_ewise_needs_device_vectors_of_one_length():
    x = torch.zeros(5)
    with pytest.raises(G.ArgumentError):
        G.gpu_ewise_(x, x, x, G.GPUGraphs_add)  # host tensors: "All inputs must be on the same backend"
    with pytest.raises(G.ArgumentError):
        G.gpu_apply_(x, x, 1.0, G.GPUGraphs_min)
    with pytest.raises(G.ArgumentError):
        G.gpu_reduce(x, G.GPUGraphs_add)


def test_operators_without_a_kernel_are_rejected():
    from gpugraphs.algebra import op_code
    with pytest.raises(G.ArgumentError):
        op_code(lambda a, b: a + b)
