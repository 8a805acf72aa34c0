"""Context, element-type codes and device-array plumbing shared by the API modules.

Device arrays are torch CUDA tensors (torch is used for device memory and streams
only).  Each device gets one library context; every call binds the caller's current
torch stream, so work is ordered with the caller's own kernels like the reference's
KernelAbstractions launches are ordered on the backend's stream."""
import ctypes

import numpy as np
import torch

from . import _lib
from .errors import ArgumentError, check

BOOL, INT32, INT64, FLOAT32, FLOAT64 = 1, 2, 3, 4, 5

TORCH2CODE = {torch.bool: BOOL, torch.int32: INT32, torch.int64: INT64, torch.float32: FLOAT32,
              torch.float64: FLOAT64}
CODE2TORCH = {v: k for k, v in TORCH2CODE.items()}
NP2CODE = {np.dtype(np.bool_): BOOL, np.dtype(np.int32): INT32, np.dtype(np.int64): INT64,
           np.dtype(np.float32): FLOAT32, np.dtype(np.float64): FLOAT64}
CODE2NP = {v: k for k, v in NP2CODE.items()}

_ctx = {}


def lib():
    return _lib.load()


def ctx(device=None):
    """Library context of `device` (default: torch's current device), bound to the
    current torch stream."""
    if device is None:
        device = torch.cuda.current_device()
    elif isinstance(device, torch.device):
        device = device.index if device.index is not None else torch.cuda.current_device()
    L = lib()
    c = _ctx.get(device)
    if c is None:
        h = ctypes.c_void_p()
        check(L.gg_init(device, ctypes.byref(h)), L)
        c = h
        _ctx[device] = c
    stream = torch.cuda.current_stream(device).cuda_stream
    check(L.gg_set_stream(c, ctypes.c_void_p(stream)), L)
    return c


def dtype_code(t):
    if isinstance(t, torch.Tensor):
        t = t.dtype
    if isinstance(t, torch.dtype):
        if t not in TORCH2CODE:
            raise ArgumentError("element type %s is not supported" % t)
        return TORCH2CODE[t]
    return NP2CODE[np.dtype(t)]


def promote_code(a, b):
    """Julia promote_type over Bool < Int32 < Int64 < Float32 < Float64."""
    return max(a, b)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def device_vector(t, name):
    """Check that t is a contiguous CUDA tensor usable as a device vector."""
    if not isinstance(t, torch.Tensor):
        raise ArgumentError("%s must be a CUDA tensor" % name)
    if not t.is_cuda:
        raise ArgumentError("All inputs must be on the same backend")
    if not t.is_contiguous():
        raise ArgumentError("%s must be contiguous" % name)
    dtype_code(t)
    return t


class _CudaArray:
    """__cuda_array_interface__ view of library-owned device memory; keeps its owner alive."""

    def __init__(self, owner, p, n, code):
        self.owner = owner
        dt = CODE2NP[code]
        self.__cuda_array_interface__ = {
            "shape": (int(n),), "typestr": dt.str, "data": (int(p), False), "version": 3,
            "strides": None}


def wrap_device(owner, p, n, code, device):
    """Zero-copy torch tensor over device memory owned by `owner`."""
    if n == 0 or p is None:
        return torch.empty(0, dtype=CODE2TORCH[code], device=device)
    return torch.as_tensor(_CudaArray(owner, p, n, code), device=device)
