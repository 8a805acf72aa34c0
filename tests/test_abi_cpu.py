"""C-ABI checks that need no GPU: the library loads, exports every entry point that
include/gpugraphs.h declares, and the Python binding and the oracle agree with the
header's constants."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpugraphs.h")


def header_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|int64_t|const char\*)\s+(gg_\w+)\s*\(", src, re.M)))


def header_enums():
    src = open(HEADER).read()
    return {k: int(v) for k, v in re.findall(r"\b(GG_\w+)\s*=\s*(-?\d+)", src)}


@pytest.fixture(scope="module")
def libpath():
    from gpugraphs import _lib
    if not os.path.exists(_lib.LIB_PATH):
        import build_lib
        build_lib.build()
    return _lib.LIB_PATH


def test_library_exports_every_declared_symbol(libpath):
    funcs = header_functions()
    assert len(funcs) >= 10
    lib = ctypes.CDLL(libpath)
    missing = [f for f in funcs if not hasattr(lib, f)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True)
    if out.returncode == 0:
        exported = set(re.findall(r"\bT (gg_\w+)", out.stdout))
        assert set(funcs) <= exported


def test_binding_covers_header(libpath):
    from gpugraphs import _lib
    assert set(_lib.declared_symbols()) == set(header_functions())
    L = _lib.load()
    assert L.gg_version().decode().startswith("gpugraphs")
    assert L.gg_last_error() is not None


def test_constants_agree():
    from gpugraphs import algebra, core
    from oracle import oracle as O
    e = header_enums()
    assert (e["GG_BOOL"], e["GG_INT32"], e["GG_INT64"], e["GG_FLOAT32"], e["GG_FLOAT64"]) == (
        O.BOOL, O.INT32, O.INT64, O.FLOAT32, O.FLOAT64)
    assert (core.BOOL, core.INT32, core.INT64, core.FLOAT32, core.FLOAT64) == (1, 2, 3, 4, 5)
    names = {"FIRST": "first", "SECOND": "second", "ANY": "any", "PAIR": "pair", "ADD": "add",
             "SAFE_ADD": "safe_add", "MINUS": "minus", "RMINUS": "rminus", "MUL": "mul",
             "MIN": "min", "MAX": "max", "LOR": "lor", "LAND": "land", "BOR": "bor",
             "BAND": "band", "BXOR": "bxor", "FIRSTI": "firsti", "FIRSTJ": "firstj",
             "SECONDI": "secondi", "SECONDJ": "secondj"}
    for k, v in names.items():
        assert e["GG_OP_" + k] == getattr(O, k) == algebra.OPERATORS["GPUGraphs_" + v].code


def test_calls_without_gpu_fail_cleanly(libpath):
    """gg_init on a machine without a usable device returns an error status (no crash)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gpugraphs import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    rc = L.gg_init(0, ctypes.byref(h))
    assert rc != 0 and L.gg_last_error()


def test_operator_scalars_match_algebra():
    import numpy as np
    import gpugraphs as G
    assert G.GPUGraphs_safe_add(np.int32(5), np.int32(2 ** 31 - 1)) == 2 ** 31 - 1
    assert G.GPUGraphs_safe_add(np.float32(1), np.float32(2)) == 3
    assert G.GPUGraphs_secondi(None, 1, 0, 0, 7, 0) == 7
    assert G.monoid_neutral(np.float32, G.GPUGraphs_min) == np.inf
    assert G.monoid_neutral(np.int32, G.GPUGraphs_band) == -1
    assert G.monoid_absorb(np.float32, G.GPUGraphs_any) is None
    with pytest.raises(G.ArgumentError):
        G.monoid_neutral(np.float32, G.GPUGraphs_lor)


def test_null_handles_are_argument_errors(libpath):
    """Every entry point checks its handles before touching a device: NULL context or
    matrix returns GG_ERR_ARGUMENT with a message (no GPU needed, no crash)."""
    from gpugraphs import _lib
    L = _lib.load()
    ARG = header_enums()["GG_ERR_ARGUMENT"]
    n64 = ctypes.c_int64(0)
    cases = [
        L.gg_spmv(None, None, 9, 5, 2, None, 4, 0, None, 4, 0, None, 0, 0, 0, 0),
        L.gg_spmv_t(None, None, 9, 5, 2, None, 4, 0, None, 4, 0, None, 0, 0, 0, 0),
        L.gg_spmspv(None, None, 9, 5, 2, None, 4, 0, None, None, 4, 0, 0, None, ctypes.byref(n64)),
        L.gg_spmv_rows(None, None, 9, 5, 2, None, 4, 0, None, 4, 0, None, 0),
        L.gg_ewise(None, 5, None, 4, None, 4, None, 4, 0, None, 0),
        L.gg_apply(None, 5, None, 4, None, 4, None, 4, 0, 0, None, 0),
        L.gg_reduce(None, 5, None, 4, 0, None),
        L.gg_read_rb(None, 1, None, None, None, None, None, None, None),
        L.gg_read_mtx(None, 1, None, None, None, None, None, None, None),
        L.gg_read_edgelist(None, 1, None, None, None, None, None, None),
        L.gg_mat_values_changed(None, None),
        L.gg_set_wait_limit(None, 5),
    ]
    for rc in cases:
        assert rc == ARG
        assert L.gg_last_error()
