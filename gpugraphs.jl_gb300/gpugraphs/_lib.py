"""ctypes binding of libgpugraphs.so (declarations in include/gpugraphs.h).

The library is loaded from gpugraphs.jl_gb300/lib/.  There is no fallback: when the
library is missing the import of the compute entry points raises."""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libgpugraphs.so")

P = ctypes.c_void_p
I = ctypes.c_int
I64 = ctypes.c_int64
U64 = ctypes.c_uint64
D = ctypes.c_double
PP = ctypes.POINTER(ctypes.c_void_p)
PI64 = ctypes.POINTER(ctypes.c_int64)
PI = ctypes.POINTER(ctypes.c_int)

# name -> argument types (all functions return int status unless listed in _RESTYPE)
SIGNATURES = {
    "gg_last_error": [],
    "gg_version": [],
    "gg_init": [I, PP],
    "gg_destroy": [P],
    "gg_set_stream": [P, P],
    "gg_stream_sync": [P],
    "gg_set_wait_limit": [P, U64],
    "gg_trace_begin": [P],
    "gg_trace_end": [P, PI64, PI64, ctypes.POINTER(ctypes.c_double)],
    "gg_csr_create": [P, I64, I64, I64, P, P, P, I, I, PP],
    "gg_sell_create": [P, P, I64, I64, PP],
    "gg_mat_destroy": [P],
    "gg_mat_info": [P, PI, PI64, PI64, PI64, PI, PI64, PI64, PI64],
    "gg_mat_arrays": [P, PP, PP, PP, PP],
    "gg_spmv": [P, P, I, I, I, P, I, I64, P, I, I64, P, I, I64, I64, I64],
    "gg_spmm": [P, P, I, I, I, P, I, I64, I64, P, I, I64, I64, I64, I, P, I, I64, I64, I64],
    "gg_mat_values_changed": [P, P],
    "gg_read_rb": [ctypes.c_char_p, I, PI64, PI64, PI64, PP, PP, PP, PI],
    "gg_read_mtx": [ctypes.c_char_p, I, PI64, PI64, PI64, PP, PP, PP, PI],
    "gg_read_edgelist": [ctypes.c_char_p, I, PI64, PI64, PP, PP, PP, PI],
    "gg_host_free": [P],
    "gg_spmv_t": [P, P, I, I, I, P, I, I64, P, I, I64, P, I, I64, I64, I64],
    "gg_spmspv": [P, P, I, I, I, P, I, I64, P, P, I, I64, I64, P, PI64],
    "gg_spmv_rows": [P, P, I, I, I, P, I, I64, P, I, I64, P, I64],
    "gg_ewise": [P, I, P, I, P, I, P, I, I64, P, I],
    "gg_apply": [P, I, P, I, P, I, P, I, I, I64, P, I],
    "gg_reduce": [P, I, P, I, I64, P],
    "gg_bfs_levels": [P, P, I64, P, I64, PI64],
    "gg_bfs_parents": [P, P, I64, P, I64, I, PI64],
    "gg_sssp": [P, P, P, I64, P, P, I, I64, PI64],
    "gg_bfs_levels_batch": [P, P, P, I64, P, I64, PI64],
    "gg_sssp_batch": [P, P, P, I64, P, I, I64, PI64],
    "gg_server_create": [P, I64, PP],
    "gg_server_add_graph": [P, P, PI],
    "gg_server_submit": [P, I, I, I64, P, I, P, PI64],
    "gg_server_poll": [P, PI64, ctypes.POINTER(ctypes.c_double), I64, PI64, PI64],
    "gg_server_stats": [P, PI64, PI64, PI64],
    "gg_server_destroy": [P],
    "gg_multigraph_create": [P, P, I64, PP],
    "gg_multigraph_destroy": [P],
    "gg_multigraph_info": [P, PI64, PI64, PI64, PI64],
    "gg_multigraph_spmv": [P, P, P, P],
    "gg_multigraph_bfs": [P, P, P, P, PI64],
    "gg_multigraph_sssp": [P, P, P, P, I, PI64],
    "gg_tune": [P, P, I64, P],
    "gg_tune_apply": [P, P, P],
    "gg_spmv_layout": [P],
    "gg_spmv_hub_rows": [P],
    "gg_bfs_levels_noalloc": [P, P, P, I, I64, I64, I64, P, P, PI64],
    "gg_gen_rmat_edges": [P, I, I64, D, D, D, U64, I, P, P, P],
    "gg_gen_er_edges": [P, I64, I64, U64, I, P, P, P],
    "gg_gen_grid_edges": [P, I64, I64, U64, I, P, P, P],
    "gg_gen_uniform_f32": [P, I64, U64, P],
}
_RESTYPE = {"gg_last_error": ctypes.c_char_p, "gg_version": ctypes.c_char_p,
            "gg_spmv_hub_rows": ctypes.c_int64}

_lock = threading.Lock()
_lib = None


def load():
    """Load libgpugraphs.so (built by gpugraphs.jl_gb300/build_lib.py)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    "libgpugraphs.so is not built (expected at %s); run "
                    "`python gpugraphs.jl_gb300/build_lib.py`" % LIB_PATH)
            lib = ctypes.CDLL(LIB_PATH)
            for name, args in SIGNATURES.items():
                f = getattr(lib, name)
                f.argtypes = args
                f.restype = _RESTYPE.get(name, ctypes.c_int)
            _lib = lib
    return _lib


def declared_symbols():
    return list(SIGNATURES)
