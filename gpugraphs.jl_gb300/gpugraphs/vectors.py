"""SparseGPUVector (src/GPUGraphsVector.jl:12-100 of GPUGraphs.jl): a length, 1-based
strictly increasing indices and their values, all on the device."""
import numpy as np
import torch

from . import core
from .errors import ArgumentError


class SparseGPUVector:
    """``SparseGPUVector(n, nzind, nzval, device=None)``.  Host arrays (numpy, lists or
    CPU tensors) are copied to the device; indices become Int32.  Raises ArgumentError
    when ``len(nzind) != len(nzval)`` (GPUGraphsVector.jl:38-40).  Index order and range
    are checked by the calls that read them."""

    def __init__(self, n, nzind, nzval, device=None):
        if len(nzind) != len(nzval):
            raise ArgumentError("length(nzind) must be equal to length(nzval)")
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else
                           torch.device(device).index or 0)
        if not isinstance(nzind, torch.Tensor):
            nzind = torch.as_tensor(np.asarray(nzind, dtype=np.int32))
        if not isinstance(nzval, torch.Tensor):
            nzval = torch.as_tensor(np.asarray(nzval))
        self.n = int(n)
        self.nzind = nzind.to(device=dev, dtype=torch.int32).contiguous()
        self.nzval = nzval.to(device=dev).contiguous()
        core.dtype_code(self.nzval)
        self.device = dev

    @classmethod
    def from_dense(cls, v, device=None):
        """SparseGPUVector(v::Vector, backend) (GPUGraphsVector.jl:60-65): the nonzeros of v."""
        v = v.detach() if isinstance(v, torch.Tensor) else torch.as_tensor(np.asarray(v))
        ind = torch.nonzero(v != 0).flatten()
        return cls(v.numel(), (ind + 1).to(torch.int32), v[ind], device=device)

    @property
    def dtype(self):
        return self.nzval.dtype

    def nnz(self):
        return self.nzind.numel()

    def __len__(self):
        return self.n

    def to_dense(self):
        """Dense torch vector with zeros outside the stored entries."""
        out = torch.zeros(self.n, dtype=self.nzval.dtype, device=self.device)
        if self.nnz():
            out[self.nzind.long() - 1] = self.nzval
        return out
