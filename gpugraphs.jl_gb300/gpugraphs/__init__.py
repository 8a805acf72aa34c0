"""gpugraphs -- Python host mirror of GPUGraphs.jl's API over libgpugraphs.so, the
hand-written sm_103a (GB300) implementation of its semiring sparse kernels and
graph algorithms.

Julia's in-place ``f!`` functions are spelled ``f_`` here (gpu_spmv_, bfs_distances_,
...); names, arguments, 1-based indices and raised errors otherwise follow the
reference's exports (src/GPUGraphs.jl:25-51)."""
from .algebra import (GPUGraphs_add, GPUGraphs_any, GPUGraphs_band, GPUGraphs_bor,
                      GPUGraphs_bxor, GPUGraphs_first, GPUGraphs_firsti, GPUGraphs_firstj,
                      GPUGraphs_land, GPUGraphs_lor, GPUGraphs_max, GPUGraphs_min,
                      GPUGraphs_minus, GPUGraphs_mul, GPUGraphs_pair, GPUGraphs_rminus,
                      GPUGraphs_safe_add, GPUGraphs_second, GPUGraphs_secondi,
                      GPUGraphs_secondj, monoid_absorb, monoid_neutral)
from .algorithms import (bfs_distances, bfs_distances_, bfs_distances_batch, bfs_parents,
                         bfs_parents_,
                         shortest_path, shortest_path_)
from .errors import (ArgumentError, BoundsError, DimensionMismatch, GPUGraphsError,
                     SpmmAssertionError, UnsupportedError)
from .ewise import gpu_apply_, gpu_ewise_, gpu_reduce
from .fileio import RBData, read_edgelist, read_mtx, read_rb
from .ops import (gpu_spmm_, gpu_spmspv, gpu_spmspv_, gpu_spmv_, gpu_spmv_rows_, set_wait_limit,
                  synchronize)
from .storage import (AbstractSparseGPUMatrix, SparseGPUMatrixCSC, SparseGPUMatrixCSR,
                      SparseGPUMatrixSELL, sprand_gpu)
from .tuning import autotune, spmv_layout, spmv_hub_rows
from .vectors import SparseGPUVector

__all__ = [
    "AbstractSparseGPUMatrix", "SparseGPUMatrixCSR", "SparseGPUMatrixSELL", "gpu_spmv_",
    "gpu_spmm_", "SparseGPUMatrixCSC", "SparseGPUVector", "gpu_spmspv_", "gpu_spmspv", "gpu_spmv_rows_",
    "gpu_ewise_", "gpu_apply_", "gpu_reduce", "RBData", "read_rb", "read_mtx", "read_edgelist", "sprand_gpu", "autotune", "spmv_layout", "spmv_hub_rows", "bfs_distances", "bfs_distances_", "bfs_distances_batch", "bfs_parents",
    "bfs_parents_", "shortest_path", "shortest_path_", "monoid_neutral", "monoid_absorb", "synchronize",
    "set_wait_limit",
    "GPUGraphs_add", "GPUGraphs_safe_add", "GPUGraphs_mul", "GPUGraphs_second",
    "GPUGraphs_band", "GPUGraphs_bor", "GPUGraphs_any", "GPUGraphs_secondi", "GPUGraphs_max",
    "GPUGraphs_min", "GPUGraphs_first", "GPUGraphs_pair", "GPUGraphs_minus", "GPUGraphs_rminus",
    "GPUGraphs_lor", "GPUGraphs_land", "GPUGraphs_bxor", "GPUGraphs_firsti", "GPUGraphs_firstj",
    "GPUGraphs_secondj", "ArgumentError", "DimensionMismatch", "BoundsError",
    "UnsupportedError", "SpmmAssertionError", "GPUGraphsError",
]
