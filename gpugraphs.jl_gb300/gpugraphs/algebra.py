"""Semiring operators of GPUGraphs.jl (src/algebra.jl:31-111).

Each GPUGraphs_* object is callable with the reference's 6-argument signature
``op(x, y, A_i, A_j, B_i, B_j)`` on scalars and carries the operator code passed to
the CUDA kernels.  ``monoid_neutral`` / ``monoid_absorb`` mirror algebra.jl:10-100.
"""
import numpy as np

from .errors import ArgumentError

_DT = {np.dtype(np.bool_): 1, np.dtype(np.int32): 2, np.dtype(np.int64): 3,
       np.dtype(np.float32): 4, np.dtype(np.float64): 5}


class Operator:
    __slots__ = ("name", "code", "_f")

    def __init__(self, name, code, f):
        self.name, self.code, self._f = name, code, f

    def __call__(self, x, y, A_i=None, A_j=None, B_i=None, B_j=None):
        return self._f(x, y, A_i, A_j, B_i, B_j)

    def __repr__(self):
        return self.name

    def __reduce__(self):
        return (_by_name, (self.name,))


def _jl_max(x, y):
    if isinstance(x, (float, np.floating)) and (np.isnan(x) or np.isnan(y)):
        return type(x)(np.nan)
    return max(x, y)


def _jl_min(x, y):
    if isinstance(x, (float, np.floating)) and (np.isnan(x) or np.isnan(y)):
        return type(x)(np.nan)
    return min(x, y)


def _safe_add(x, y, *_):
    t = np.result_type(x, y)
    tm = np.inf if np.issubdtype(t, np.floating) else np.iinfo(t).max
    return t.type(tm) if _jl_max(x, y) == tm else (t.type(x) + t.type(y))


GPUGraphs_first = Operator("GPUGraphs_first", 1, lambda x, y, *a: x)
GPUGraphs_second = Operator("GPUGraphs_second", 2, lambda x, y, *a: y)
GPUGraphs_any = Operator("GPUGraphs_any", 3, lambda x, y, *a: _jl_max(x, y))
GPUGraphs_pair = Operator("GPUGraphs_pair", 4, lambda x, y, *a: type(x)(1) if y != 0 else type(x)(0))
GPUGraphs_add = Operator("GPUGraphs_add", 5, lambda x, y, *a: x + y)
GPUGraphs_safe_add = Operator("GPUGraphs_safe_add", 6, _safe_add)
GPUGraphs_minus = Operator("GPUGraphs_minus", 7, lambda x, y, *a: x - y)
GPUGraphs_rminus = Operator("GPUGraphs_rminus", 8, lambda x, y, *a: y - x)
GPUGraphs_mul = Operator("GPUGraphs_mul", 9, lambda x, y, *a: x * y)
GPUGraphs_min = Operator("GPUGraphs_min", 10, lambda x, y, *a: _jl_min(x, y))
GPUGraphs_max = Operator("GPUGraphs_max", 11, lambda x, y, *a: _jl_max(x, y))
GPUGraphs_lor = Operator("GPUGraphs_lor", 12, lambda x, y, *a: x | y)
GPUGraphs_land = Operator("GPUGraphs_land", 13, lambda x, y, *a: x & y)
GPUGraphs_bor = Operator("GPUGraphs_bor", 14, lambda x, y, *a: x | y)
GPUGraphs_band = Operator("GPUGraphs_band", 15, lambda x, y, *a: x & y)
GPUGraphs_bxor = Operator("GPUGraphs_bxor", 16, lambda x, y, *a: x ^ y)
GPUGraphs_firsti = Operator("GPUGraphs_firsti", 17, lambda x, y, ai, aj, bi, bj: ai)
GPUGraphs_firstj = Operator("GPUGraphs_firstj", 18, lambda x, y, ai, aj, bi, bj: aj)
GPUGraphs_secondi = Operator("GPUGraphs_secondi", 19, lambda x, y, ai, aj, bi, bj: bi * y)
GPUGraphs_secondj = Operator("GPUGraphs_secondj", 20, lambda x, y, ai, aj, bi, bj: bj)

OPERATORS = {op.name: op for op in (
    GPUGraphs_first, GPUGraphs_second, GPUGraphs_any, GPUGraphs_pair, GPUGraphs_add,
    GPUGraphs_safe_add, GPUGraphs_minus, GPUGraphs_rminus, GPUGraphs_mul, GPUGraphs_min,
    GPUGraphs_max, GPUGraphs_lor, GPUGraphs_land, GPUGraphs_bor, GPUGraphs_band,
    GPUGraphs_bxor, GPUGraphs_firsti, GPUGraphs_firstj, GPUGraphs_secondi, GPUGraphs_secondj)}


def _by_name(name):
    return OPERATORS[name]


def op_code(op):
    """Operator code for the C ABI; rejects callables without a kernel (no JIT, no
    CPU fallback)."""
    if isinstance(op, Operator):
        return op.code
    raise ArgumentError("operator %r has no sm_103a kernel; use a GPUGraphs_* operator" % (op,))


def _typemax(t):
    t = np.dtype(t)
    if t == np.bool_:
        return np.bool_(True)
    if np.issubdtype(t, np.floating):
        return t.type(np.inf)
    return t.type(np.iinfo(t).max)


def _typemin(t):
    t = np.dtype(t)
    if t == np.bool_:
        return np.bool_(False)
    if np.issubdtype(t, np.floating):
        return t.type(-np.inf)
    return t.type(np.iinfo(t).min)


def monoid_neutral(T, op):
    """monoid_neutral(T, op) (src/algebra.jl:10-99)."""
    t = np.dtype(T)
    one_bits = np.bool_(True) if t == np.bool_ else t.type(-1)
    if op is GPUGraphs_add or op is GPUGraphs_safe_add or op is GPUGraphs_any or op is GPUGraphs_bor:
        return t.type(0)
    if op is GPUGraphs_mul:
        return t.type(1)
    if op is GPUGraphs_min:
        return _typemax(t)
    if op is GPUGraphs_max:
        return _typemin(t)
    if op is GPUGraphs_band and not np.issubdtype(t, np.floating):
        return one_bits
    if op is GPUGraphs_lor and t == np.bool_:
        return np.bool_(False)
    if op is GPUGraphs_land and t == np.bool_:
        return np.bool_(True)
    raise ArgumentError("monoid_neutral not implemented for type %s and operation %s" % (t, op))


def monoid_absorb(T, op):
    """monoid_absorb(T, op) (src/algebra.jl:14-100); None when there is none."""
    t = np.dtype(T)
    if op in (GPUGraphs_add, GPUGraphs_safe_add, GPUGraphs_max):
        return _typemax(t)
    if op is GPUGraphs_mul or op is GPUGraphs_band:
        return t.type(0)
    if op is GPUGraphs_min:
        return _typemin(t)
    if op is GPUGraphs_bor:
        return np.bool_(True) if t == np.bool_ else t.type(-1)
    if op is GPUGraphs_lor and t == np.bool_:
        return np.bool_(True)
    if op is GPUGraphs_land and t == np.bool_:
        return np.bool_(False)
    return None
