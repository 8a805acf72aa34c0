"""Exceptions mirroring the Julia exceptions GPUGraphs.jl throws, and the mapping
from the C ABI's status codes."""


class GPUGraphsError(RuntimeError):
    """Base class of errors returned by libgpugraphs."""


class DimensionMismatch(GPUGraphsError, ValueError):
    """Julia DimensionMismatch (src/spmv/CSR.jl:374-379)."""


class ArgumentError(GPUGraphsError, ValueError):
    """Julia ArgumentError (src/storage/CSR.jl:48-63, src/spmv/CSR.jl:381-387)."""


class BoundsError(GPUGraphsError, IndexError):
    """Julia BoundsError (src/storage/CSR.jl:155-157)."""


class UnsupportedError(GPUGraphsError, TypeError):
    """No neutral element / no method for this operator and element type (algebra.jl:10-11)."""


class OutOfMemoryError(GPUGraphsError, MemoryError):
    pass


class CudaError(GPUGraphsError):
    pass


class TimeoutError_(GPUGraphsError, TimeoutError):
    pass


class NotConvergedError(GPUGraphsError):
    pass


class SpmmAssertionError(GPUGraphsError, AssertionError):
    """Julia AssertionError from the @assert shape checks of gpu_spmm! (src/spmm/CSR.jl:131-133)."""


_BY_CODE = {1: DimensionMismatch, 2: ArgumentError, 3: ArgumentError, 4: UnsupportedError,
            5: OutOfMemoryError, 6: CudaError, 7: TimeoutError_, 8: BoundsError,
            9: SpmmAssertionError, 10: NotConvergedError}


def check(rc, lib):
    if rc != 0:
        msg = lib.gg_last_error().decode(errors="replace")
        raise _BY_CODE.get(rc, GPUGraphsError)(msg or "libgpugraphs error %d" % rc)
