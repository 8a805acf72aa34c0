"""Element-wise, apply and reduce over dense device vectors with the operators of
src/algebra.jl.

The reference's src/e_wise_ops.jl and src/map_and_reduce.jl are empty; its algorithms
do these steps with Julia broadcasts (bfs.jl:60-70, shortest_path.jl:72-79).  Each
call here is one kernel with Julia's scalar semantics; the computation type is
promote_type of the operands and the result vector must be able to hold it."""
import ctypes

import numpy as np
import torch

from . import core
from .algebra import op_code
from .errors import ArgumentError, DimensionMismatch, check


def _mask_args(mask, n, device):
    if mask is None:
        return None, 0
    if not isinstance(mask, torch.Tensor) or mask.dim() != 1 or mask.numel() != n:
        raise DimensionMismatch("Mask length must be equal to the length of the vectors")
    if not mask.is_cuda or mask.device != device:
        raise ArgumentError("Mask must be on the same backend")
    mask = mask.contiguous()
    return mask, core.dtype_code(mask)


def gpu_ewise_(z, x, y, op, mask=None):
    """z[i] = op(x[i], y[i]) (index operators see entry i as row i, column 1), only
    where mask[i] != 0 when a mask is given.  Asynchronous on the current stream."""
    for t, name in ((z, "z"), (x, "x"), (y, "y")):
        core.device_vector(t, name)
    if not (z.numel() == x.numel() == y.numel()):
        raise DimensionMismatch("vector lengths must agree")
    if x.device != z.device or y.device != z.device:
        raise ArgumentError("All inputs must be on the same backend")
    mask, mcode = _mask_args(mask, z.numel(), z.device)
    L = core.lib()
    with torch.cuda.device(z.device):
        c = core.ctx(z.device)
        check(L.gg_ewise(c, op_code(op), core.ptr(z), core.dtype_code(z), core.ptr(x),
                         core.dtype_code(x), core.ptr(y), core.dtype_code(y), z.numel(),
                         core.ptr(mask), mcode), L)
    return z


def _scalar(s, s_dtype, like):
    if s_dtype is None:
        if isinstance(s, (np.generic, np.ndarray)):
            s_dtype = np.asarray(s).dtype
        else:
            s_dtype = like
    code = core.dtype_code(s_dtype)
    buf = np.array([s], dtype=core.CODE2NP[code])
    return buf, code


def gpu_apply_(z, x, s, op, bind_first=False, s_dtype=None, mask=None):
    """z[i] = op(x[i], s), or op(s, x[i]) with bind_first; s is a host scalar, of
    s_dtype (a torch or numpy dtype; default: the numpy scalar's own type, else x's
    element type).  Asynchronous on the current stream."""
    core.device_vector(z, "z")
    core.device_vector(x, "x")
    if z.numel() != x.numel():
        raise DimensionMismatch("vector lengths must agree")
    if x.device != z.device:
        raise ArgumentError("All inputs must be on the same backend")
    buf, scode = _scalar(s, s_dtype, x.dtype)
    mask, mcode = _mask_args(mask, z.numel(), z.device)
    L = core.lib()
    with torch.cuda.device(z.device):
        c = core.ctx(z.device)
        check(L.gg_apply(c, op_code(op), core.ptr(z), core.dtype_code(z), core.ptr(x),
                         core.dtype_code(x), buf.ctypes.data_as(ctypes.c_void_p), scode,
                         1 if bind_first else 0, z.numel(), core.ptr(mask), mcode), L)
    return z


def gpu_reduce(x, add):
    """add over x from the monoid's neutral element, in x's element type (a numpy
    scalar).  Float sums follow one fixed order, the same on every GPU (chunks of 8192
    values folded by thread, then by xor butterflies).  Synchronous."""
    core.device_vector(x, "x")
    code = core.dtype_code(x)
    out = np.zeros(1, dtype=core.CODE2NP[code])
    L = core.lib()
    with torch.cuda.device(x.device):
        c = core.ctx(x.device)
        check(L.gg_reduce(c, op_code(add), core.ptr(x), code, x.numel(),
                          out.ctypes.data_as(ctypes.c_void_p)), L)
    return out[0]
