/*
 * gpugraphs.h — C ABI of libgpugraphs.so, the sm_103a (GB300) implementation of the
 * semiring sparse kernels and graph algorithms of GPUGraphs.jl.
 *
 * Every entry point replaces one Julia method of the reference package; the citation
 * beside each declaration is the reference interface it stands in for (paths are
 * relative to the GPUGraphs.jl repository).
 *
 * Conventions
 *  - Every call returns an int status (GG_OK == 0).  No exceptions cross the ABI.
 *    gg_last_error() returns a thread-local message for the last failing call.
 *  - Index arrays follow the reference: 1-based Int32 rowptr / colval / slice_ptr,
 *    colval == -1 for SELL padding, 1-based vertex ids in BFS/SSSP.
 *  - Vectors and dense matrices passed to compute calls are caller-owned DEVICE
 *    pointers.  Matrix handles (gg_mat) own their device storage until
 *    gg_mat_destroy().
 *  - Work is enqueued on the context's stream (gg_set_stream; default: the legacy
 *    default stream) and is asynchronous unless stated otherwise, like the
 *    reference's KernelAbstractions launches (callers synchronize before reading).
 *  - A context may be used from one host thread at a time.
 */
#ifndef GPUGRAPHS_H
#define GPUGRAPHS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (Julia exception the reference throws in brackets) ---- */
enum {
  GG_OK = 0,
  GG_ERR_DIMENSION = 1,     /* DimensionMismatch  (src/spmv/CSR.jl:374-379) */
  GG_ERR_ARGUMENT = 2,      /* ArgumentError      (src/storage/CSR.jl:48-63) */
  GG_ERR_TYPE = 3,          /* ArgumentError "Result type must be able to hold ..." (src/spmv/CSR.jl:381-387) */
  GG_ERR_UNSUPPORTED = 4,   /* no neutral element / no method for this operator and type (src/algebra.jl:10-11) */
  GG_ERR_OOM = 5,           /* device allocation failed */
  GG_ERR_CUDA = 6,          /* any other CUDA runtime error */
  GG_ERR_TIMEOUT = 7,       /* a bounded device-side wait ran out */
  GG_ERR_BOUNDS = 8,        /* BoundsError (source vertex outside 1..n) */
  GG_ERR_ASSERTION = 9,     /* AssertionError (src/spmm/CSR.jl:131-133) */
  GG_ERR_NOT_CONVERGED = 10 /* Bellman-Ford still improving after n rounds (negative cycle) */
};

/* ---- element types, numbered in Julia's promotion order (promote = max) ---- */
enum {
  GG_BOOL = 1,    /* Julia Bool, one byte holding 0 or 1 */
  GG_INT32 = 2,
  GG_INT64 = 3,
  GG_FLOAT32 = 4,
  GG_FLOAT64 = 5
};

/* ---- semiring operators: the GPUGraphs_* functions of src/algebra.jl:31-111 ---- */
enum {
  GG_OP_FIRST = 1,     /* GPUGraphs_first    x                        algebra.jl:31  */
  GG_OP_SECOND = 2,    /* GPUGraphs_second   y                        algebra.jl:32  */
  GG_OP_ANY = 3,       /* GPUGraphs_any      max(x,y), neutral 0      algebra.jl:35  */
  GG_OP_PAIR = 4,      /* GPUGraphs_pair     y != 0 ? 1 : 0           algebra.jl:40  */
  GG_OP_ADD = 5,       /* GPUGraphs_add      x + y                    algebra.jl:43  */
  GG_OP_SAFE_ADD = 6,  /* GPUGraphs_safe_add typemax-saturating +     algebra.jl:47  */
  GG_OP_MINUS = 7,     /* GPUGraphs_minus    x - y                    algebra.jl:52  */
  GG_OP_RMINUS = 8,    /* GPUGraphs_rminus   y - x                    algebra.jl:53  */
  GG_OP_MUL = 9,       /* GPUGraphs_mul      x * y                    algebra.jl:55  */
  GG_OP_MIN = 10,      /* GPUGraphs_min                               algebra.jl:65  */
  GG_OP_MAX = 11,      /* GPUGraphs_max                               algebra.jl:68  */
  GG_OP_LOR = 12,      /* GPUGraphs_lor      x | y (Bool monoid)      algebra.jl:77  */
  GG_OP_LAND = 13,     /* GPUGraphs_land     x & y (Bool monoid)      algebra.jl:80  */
  GG_OP_BOR = 14,      /* GPUGraphs_bor      x | y                    algebra.jl:95  */
  GG_OP_BAND = 15,     /* GPUGraphs_band     x & y                    algebra.jl:98  */
  GG_OP_BXOR = 16,     /* GPUGraphs_bxor     x xor y                  algebra.jl:102 */
  GG_OP_FIRSTI = 17,   /* GPUGraphs_firsti   A_i (row)                algebra.jl:106 */
  GG_OP_FIRSTJ = 18,   /* GPUGraphs_firstj   A_j (column of A)        algebra.jl:107 */
  GG_OP_SECONDI = 19,  /* GPUGraphs_secondi  B_i * y                  algebra.jl:109 */
  GG_OP_SECONDJ = 20   /* GPUGraphs_secondj  B_j (column of B)        algebra.jl:111 */
};

enum { GG_FMT_CSR = 1, GG_FMT_SELL = 2 };

/* dense layouts for gg_spmm: Julia matrices are column-major */
enum { GG_COL_MAJOR = 0, GG_ROW_MAJOR = 1 };

/* BFS parent rules (which frontier in-neighbour becomes the parent) */
enum {
  GG_PARENT_FORMAT_DEFAULT = 0, /* CSR: FIRST_IN_ROW, SELL: MAX_INDEX, as the reference */
  GG_PARENT_FIRST_IN_ROW = 1,   /* first frontier column in storage order (src/spmv/CSR.jl:147-171) */
  GG_PARENT_MAX_INDEX = 2       /* largest frontier column index (src/algebra.jl:35 via src/spmv/SELL.jl:100-133) */
};

/* query kinds served by gg_server */
enum { GG_QUERY_BFS = 1, GG_QUERY_SSSP = 2, GG_QUERY_SPMV_ITER = 3 };

typedef struct gg_ctx gg_ctx; /* device, stream, scratch arena */
typedef struct gg_mat gg_mat; /* a CSR or SELL-C-sigma matrix resident on the device */
typedef struct gg_server gg_server; /* continuous-batching query server */
typedef struct gg_multigraph gg_multigraph; /* many graphs in one block-diagonal structure */

/* ---- library / context ---------------------------------------------------- */

/* Message of the last failing call on this thread ("" if none). */
const char* gg_last_error(void);

/* Library version string. */
const char* gg_version(void);

/* Replaces KernelAbstractions backend selection (test/spmv.jl:1-8): binds device `device`. */
int gg_init(int device, gg_ctx** out);

/* Frees the context and its scratch arena (matrices must be destroyed separately). */
int gg_destroy(gg_ctx* ctx);

/* Enqueue subsequent work on `stream` (a cudaStream_t; NULL = legacy default stream). */
int gg_set_stream(gg_ctx* ctx, void* stream);

/* Replaces KernelAbstractions.synchronize(backend) (test/spmv.jl:25). */
int gg_stream_sync(gg_ctx* ctx);

/* Poll limit of the bounded device-side waits of this context's later calls (no
 * reference counterpart: the reference's host loops wait on nothing on the device).
 * It bounds the grid barriers of the persistent kernels (cooperative BFS and
 * shortest-path phases of hub-free graphs, the near-far search, the many-graph BFS /
 * shortest paths; each poll sleeps ~100 ns) and the bulk-copy waits of the staged
 * SpMV kernels.  A wait that runs out records an error; every block returns, and the
 * call (or, for asynchronous SpMV calls, the next gg_stream_sync) returns
 * GG_ERR_TIMEOUT with partial results.  The context stays usable.  polls = 0
 * restores the built-in limits (2^26 barrier polls, about 7 s; 2^22 copy polls);
 * values above 2^32 - 1 are clamped. */
int gg_set_wait_limit(gg_ctx* ctx, uint64_t polls);

/* Launch tracing (no reference counterpart).  Between gg_trace_begin and
 * gg_trace_end, the kernel launches of gg_spmv / gg_spmm calls on this context are
 * counted, and the main kernel of each call (the one that streams the matrix) is
 * bracketed by CUDA events on the context's stream (first 4096 calls).  gg_trace_end
 * synchronizes the stream and returns the launch count, the number of bracketed
 * launches and their summed device time in ms.  Any out pointer may be NULL. */
int gg_trace_begin(gg_ctx* ctx);
int gg_trace_end(gg_ctx* ctx, int64_t* launches, int64_t* timed, double* timed_ms);

/* ---- storage ------------------------------------------------------------------ */

/*
 * Replaces SparseGPUMatrixCSR(m, n, rowptr, colval, nzval, backend)
 * (src/storage/CSR.jl:34-92).  rowptr (m+1), colval (nnz) are 1-based Int32,
 * nzval (nnz) has element type `dtype`.  on_device != 0: the three pointers are
 * device pointers, else host pointers.  The arrays are copied.  Validation follows
 * src/storage/CSR.jl:48-63 (rowptr[1] == 1, rowptr[m+1] == nnz+1, 1 <= colval <= n)
 * and also requires rowptr to be non-decreasing; violations return GG_ERR_ARGUMENT.
 */
int gg_csr_create(gg_ctx* ctx, int64_t m, int64_t n, int64_t nnz, const int32_t* rowptr,
                  const int32_t* colval, const void* nzval, int dtype, int on_device,
                  gg_mat** out);

/*
 * Replaces SparseGPUMatrixSELL(transpose(A_csc), backend, slice_size)
 * (src/storage/SELL.jl:99-181), built on the device from a CSR handle.
 * slice_size C is clamped to m like the reference (SELL.jl:108).  sigma == 1 gives
 * the reference layout exactly (identity perm, test/structs.jl:188-190); sigma > 1
 * sorts rows by decreasing length inside windows of sigma rows (SELL-C-sigma) and
 * records the permutation.
 */
int gg_sell_create(gg_ctx* ctx, const gg_mat* csr, int64_t slice_size, int64_t sigma,
                   gg_mat** out);

/* Frees a matrix handle and its device storage. */
int gg_mat_destroy(gg_mat* A);

/*
 * Replaces size(A), nnz(A) and the SELL fields m, n, slice_size, nslices, n_stored
 * (src/storage/CSR.jl:142-184, src/storage/SELL.jl:9-16,193-242).  Any out pointer
 * may be NULL.
 */
int gg_mat_info(const gg_mat* A, int* format, int64_t* m, int64_t* n, int64_t* nnz,
                int* dtype, int64_t* n_stored, int64_t* slice_size, int64_t* nslices);

/*
 * Device pointers of the fields A.rowptr / A.colval / A.nzval (CSR) or
 * A.slice_ptr / A.colval / A.nzval / perm (SELL; perm is 1-based Int32, length m).
 * The memory stays owned by the handle.  Any out pointer may be NULL.
 */
int gg_mat_arrays(const gg_mat* A, void** ptr, void** colval, void** nzval, void** perm);

/*
 * Drops everything the library derived from the handle's values on first use (the
 * SELL-32 and transposed copies, graph analyses, plans); call it after writing to the
 * arrays gg_mat_arrays returns (setindex!, src/storage/CSR.jl:166-180).  Waits for the
 * context's stream first.
 */
int gg_mat_values_changed(gg_ctx* ctx, gg_mat* A);

/* ---- semiring kernels -------------------------------------------------------- */

/*
 * Replaces gpu_spmv!(C, A, B; mul, add, accum, range, mask)
 * (src/spmv/CSR.jl:2-29 and src/spmv/SELL.jl:2-29):
 *   y[r] = accum(y[r], add_k mul(A[r,k], x[k], r, k, k, 1))   for every selected row r
 * Rows are selected by the optional dense mask (mask[r] != 0; NULL = all rows) and the
 * optional 1-based inclusive row range [range_lo, range_hi] (range_lo == 0: no range).
 * Unselected rows are not written.  With add == GG_OP_ANY on CSR and a mask, the
 * first stored column (storage order) whose x is nonzero is taken, as
 * any_dense_masked_csr_spmv_kernel! does (src/spmv/CSR.jl:147-171), and rows without
 * such a column are not written.  Checks of _validate_args (src/spmv/CSR.jl:358-408)
 * return GG_ERR_DIMENSION / GG_ERR_TYPE.
 * Device memory: the first call of a kind builds its analysis on the handle, kept until
 * gg_mat_destroy or gg_mat_values_changed.  The first plus-times Float32 call on a CSR
 * handle of at least 65536 rows builds a SELL-32 copy of the matrix with rows sorted by
 * length and relabelled columns: about 12 bytes per stored entry plus 16 per row, i.e.
 * more than the CSR itself (about 1.6 GB at R-MAT scale 22, 6.5 GB at scale 24).  Other
 * first calls add row-block descriptors (16 bytes per block of up to 256 entries).
 * Later calls allocate nothing and are asynchronous.
 */
int gg_spmv(gg_ctx* ctx, const gg_mat* A, int mul, int add, int accum, void* y, int y_dtype,
            int64_t y_len, const void* x, int x_dtype, int64_t x_len, const void* mask,
            int mask_dtype, int64_t mask_len, int64_t range_lo, int64_t range_hi);

/*
 * Replaces gpu_spmm!(C, A, B; mul, add, accum, mask, range)
 * (src/spmm/CSR.jl:111-204, src/spmm/SELL.jl:84-124):
 *   C[r,j] = accum(C[r,j], add_k mul(A[r,k], B[k,j], r, k, k, j))
 * B is b_rows x k, C is c_rows x k, both in `layout` with leading dimensions ldb/ldc
 * (elements).  Mask / range select rows as in gg_spmv.  Shape checks return
 * GG_ERR_ASSERTION like the reference's @assert.
 */
int gg_spmm(gg_ctx* ctx, const gg_mat* A, int mul, int add, int accum, void* C, int c_dtype,
            int64_t c_rows, int64_t ldc, const void* B, int b_dtype, int64_t b_rows,
            int64_t ldb, int64_t k, int layout, const void* mask, int mask_dtype,
            int64_t mask_len, int64_t range_lo, int64_t range_hi);

/*
 * Semiring SpMV over a sparse input vector: replaces gpu_spmspv!(C, A, B, mul, add,
 * accum) (src/spmspv.jl:23-54, written for CSC and never finished there), over the CSR
 * storage of A (A_T of the graph) like every other entry point.  x is the sparse vector
 * (x_len, x_ind[0..x_nnz), x_val) with 1-based, strictly increasing device indices
 * (SparseGPUVector's nzind / nzval, src/GPUGraphsVector.jl:12-24).  For every row i
 * with at least one entry whose column carries an entry of x,
 *     y[i] = accum(y[i], add over those entries k, in storage order, of
 *                        mul(A[k], x[col], i, col, col, 1))
 * with the absorb early exit of src/spmv/CSR.jl:31-54; other rows of the dense y are
 * not written.  y_ind (device, capacity m, may be NULL) receives the 1-based rows
 * written, ascending; *y_nnz (may be NULL) their count.  The first call builds a column
 * index of A and its workspace, kept on the handle: 4(n+1) + 12 nnz bytes for the index
 * and the long-row products, about 12n + 13m bytes of bitmaps, staging and lists.  Errors: GG_ERR_DIMENSION as gpu_spmspv! (n != x_len,
 * m != y_len), GG_ERR_TYPE / GG_ERR_UNSUPPORTED as gg_spmv, GG_ERR_ARGUMENT for indices
 * that are not increasing or outside 1:n (nothing written), GG_ERR_UNSUPPORTED for a
 * SELL handle.  Synchronous.
 */
int gg_spmspv(gg_ctx* ctx, const gg_mat* A, int mul, int add, int accum, void* y, int y_dtype,
              int64_t y_len, const int32_t* x_ind, const void* x_val, int x_dtype,
              int64_t x_nnz, int64_t x_len, int32_t* y_ind, int64_t* y_nnz);

/*
 * Semiring SpMV with the transpose of a CSR handle: y = A' x.  Replaces the CSC method of
 * gpu_spmv! (src/spmv/CSC.jl:2-61, which adds with an atomic += whatever the semiring):
 * a CSC matrix B is the CSR storage of B' (same colptr / rowval / nzval), so B x is this
 * call on the handle made from B's arrays.  For every row j of A' selected by mask
 * (length n) and range (1-based rows of A'),
 *     y[j] = accum(y[j], add over the rows i of A holding column j, ascending, of
 *                        mul(A[i, j], x[i], j, i, i, 1))
 * with the absorb early exit, i.e. gg_spmv over the CSR storage of A', which the first
 * call builds on the handle (stable radix sort of the column ids): a second matrix of
 * 4(n+1) + 8 nnz bytes kept until gg_mat_destroy or gg_mat_values_changed, plus what
 * gg_spmv builds on it.  x_len must be m, y_len n; errors as gg_spmv;
 * GG_ERR_UNSUPPORTED for a SELL handle.  Asynchronous after the first call.
 */
int gg_spmv_t(gg_ctx* ctx, const gg_mat* A, int mul, int add, int accum, void* y, int y_dtype,
              int64_t y_len, const void* x, int x_dtype, int64_t x_len, const void* mask,
              int mask_dtype, int64_t mask_len, int64_t range_lo, int64_t range_hi);

/*
 * SpMV of the listed rows only: replaces sparse_masked_csr_spmv_kernel!
 * (src/spmv/CSR.jl:90-115), whose mask is a list of row ids.  For every 1-based row r of
 * rows[0..nrows) (device), y[r] = accum(y[r], add over row r in storage order of
 * mul(A[k], x[col], r, col, col, 1)) with the absorb early exit; other rows are not
 * written.  Rows should be distinct (a repeated row applies accum once per listing).
 * GG_ERR_BOUNDS when a listed row is outside 1:m (the other rows are written);
 * GG_ERR_UNSUPPORTED for a SELL handle.  Synchronous.
 */
int gg_spmv_rows(gg_ctx* ctx, const gg_mat* A, int mul, int add, int accum, void* y,
                 int y_dtype, int64_t y_len, const void* x, int x_dtype, int64_t x_len,
                 const int32_t* rows, int64_t nrows);

/* ---- element-wise, apply, reduce ---------------------------------------------- */
/*
 * The reference's src/e_wise_ops.jl and src/map_and_reduce.jl are empty; its
 * algorithms use Julia broadcasts for these steps (bfs.jl:60-70, shortest_path.jl:72-79).
 * Operators and element types are those of the semiring calls, with Julia's scalar
 * semantics; the computation type is promote_type of the two operands (Int32 / Int64
 * at least for the index operators, as in gg_spmv), and the result type must hold it
 * (GG_ERR_TYPE otherwise); an operator without a method for that type returns
 * GG_ERR_UNSUPPORTED.  Index operators see vector entry i as (row i, column 1).
 * Entries where mask (optional, any element type) is zero are not written.
 */
/* z[i] = op(x[i], y[i]) for i in 0..n-1.  Asynchronous on the context's stream. */
int gg_ewise(gg_ctx* ctx, int op, void* z, int z_dtype, const void* x, int x_dtype,
             const void* y, int y_dtype, int64_t n, const void* mask, int mask_dtype);
/* z[i] = op(x[i], s), or op(s, x[i]) when s_first != 0; s points to one host value of
   s_dtype.  Asynchronous on the context's stream. */
int gg_apply(gg_ctx* ctx, int op, void* z, int z_dtype, const void* x, int x_dtype,
             const void* s, int s_dtype, int s_first, int64_t n, const void* mask,
             int mask_dtype);
/* *out (host, x_dtype) = add over x[0..n) starting from add's neutral element
   (GG_ERR_UNSUPPORTED when add is not a monoid of x_dtype).  Order: chunks of 8192
   values, one 256-thread block each (thread t folds t, t+256, ... left to right, then
   xor butterflies over the lanes and over the 8 warp totals), chunk totals reduced
   again the same way; exact monoids give the same value in any order.  Synchronous. */
int gg_reduce(gg_ctx* ctx, int add, const void* x, int x_dtype, int64_t n, void* out);

/* ---- graph files (host) --------------------------------------------------------- */
/*
 * Reads an assembled Rutherford-Boeing (or Harwell-Boeing) matrix file: the files the
 * reference's benchmark loads with RutherfordBoeingData (benchmark/benchmarks.jl:262-266).
 * Returns the m x n matrix as CSC: 1-based Int32 colptr (n+1) / rowval (nnz, rows
 * ascending in each column) and Float64 values (1.0 for pattern files), all allocated
 * by the library on the host (release each with gg_host_free).  expand_symmetric != 0
 * mirrors the stored triangle of symmetric / skew-symmetric / Hermitian files.  kind
 * (may be NULL): bit 0 pattern, bit 1 integer, bit 2 symmetric, bit 3 skew, bit 4
 * Hermitian.  Fields are read by the widths of the file's Fortran formats.  Repeated
 * entries keep the first.  GG_ERR_ARGUMENT for unreadable or malformed files,
 * GG_ERR_UNSUPPORTED for complex or elemental files.
 */
int gg_read_rb(const char* path, int expand_symmetric, int64_t* m, int64_t* n, int64_t* nnz,
               int32_t** colptr, int32_t** rowval, double** values, int* kind);

/*
 * Reads a Matrix Market coordinate file (real / integer / pattern; general / symmetric /
 * skew-symmetric / Hermitian), the other format SuiteSparse matrices are published in.
 * Same result, ownership, expansion and kind flags as gg_read_rb; GG_ERR_UNSUPPORTED for
 * array (dense) or complex files.
 */
int gg_read_mtx(const char* path, int expand_symmetric, int64_t* m, int64_t* n, int64_t* nnz,
                int32_t** colptr, int32_t** rowval, double** values, int* kind);

/*
 * Reads an edge list (GraphIO.EdgeList, benchmark/benchmarks.jl:12-14): one edge
 * "u v [w]" per line (spaces, tabs or commas), '#' / '%' comment lines, vertex ids
 * starting at `base` (0 or 1).  Returns the adjacency A (A[u, v] for the edge u -> v)
 * of nv = largest id + 1 - base vertices as CSC, which is the CSR storage of A_T, the
 * form the graph calls take: colptr (nv+1), rowval, values (w, or 1.0 without a third
 * column; *weighted says which), host memory released with gg_host_free.  A repeated
 * edge keeps its first weight.
 */
int gg_read_edgelist(const char* path, int base, int64_t* nv, int64_t* nnz, int32_t** colptr,
                     int32_t** rowval, double** values, int* weighted);

/* Releases host memory returned by gg_read_rb / gg_read_edgelist. */
int gg_host_free(void* p);

/* ---- graph algorithms ------------------------------------------------------- */

/*
 * Replaces bfs_distances!(A_T, source, dist, curr, next, to_explore)
 * (src/algorithms/bfs.jl:31-73).  A_T is the transposed adjacency matrix (row v lists
 * the in-neighbours of v); an edge counts when its stored value is odd / true, as the
 * reference's band(A[v,u], curr[u]) test does.  Writes dist[v] = hop level for every
 * reached vertex (dist[source] = 0) and leaves the other entries untouched, so the
 * caller pre-fills dist with typemax(Int32) like bfs_distances (bfs.jl:16-18).
 * Synchronous (returns after the search).  levels_out (may be NULL): levels searched.
 */
int gg_bfs_levels(gg_ctx* ctx, const gg_mat* A_T, int64_t source, int32_t* dist, int64_t n,
                  int64_t* levels_out);

/*
 * Replaces bfs_parents!(A_T, source, parents, curr, next, to_explore)
 * (src/algorithms/bfs.jl:135-183).  parents[source] = 0; every reached vertex gets a
 * 1-based in-neighbour one level closer to the source, chosen by `rule`
 * (GG_PARENT_FORMAT_DEFAULT: first in storage order for CSR, largest index for SELL,
 * as the reference's kernels choose); other entries are untouched.  Every stored edge
 * counts, whatever its value (GPUGraphs_secondi ignores A's values).  Synchronous.
 */
int gg_bfs_parents(gg_ctx* ctx, const gg_mat* A_T, int64_t source, int32_t* parents, int64_t n,
                   int rule, int64_t* levels_out);

/*
 * Replaces shortest_path(A_T, source | sources) and shortest_path!(...)
 * (src/algorithms/shortest_path.jl:12-161): the fixpoint of
 *   next[v] = min(next[v], min_u safe_add(A_T[v,u], dist[u]))
 * for each of the nsources (1-based, host array) columns of dist (n x nsources,
 * column-major, leading dimension ld, element type Int32 for Bool A_T, else eltype).
 * next == NULL: dist is initialised here (typemax, 0 at the source) -- the
 * non-mutating form.  next != NULL: the caller's dist / next are the starting
 * iterates, sources are set to 0 in both, and both hold the result on return -- the
 * in-place form.  Non-negative weights use a frontier Bellman-Ford (same fixpoint);
 * negative or NaN weights run the reference's Jacobi rounds and return
 * GG_ERR_NOT_CONVERGED after n+1 rounds without convergence.  Synchronous.
 * rounds_out (may be NULL): relaxation rounds used, summed over sources.
 */
int gg_sssp(gg_ctx* ctx, const gg_mat* A_T, const int64_t* sources, int64_t nsources, void* dist,
            void* next, int dist_dtype, int64_t ld, int64_t* rounds_out);

/*
 * Batched BFS: column q of dist (n x S, column-major, leading dimension ld) receives
 * bfs_distances(A_T, sources[q]) -- levels over edges with odd / true values,
 * typemax(Int32) when unreached.  Up to 256 sources share one pass over the graph
 * per level (frontiers and visited sets packed as bits).  The reference has no
 * multi-source BFS; this is the batched form of bfs_distances (src/algorithms/
 * bfs.jl:1-29).  Synchronous.  levels_out (may be NULL): levels summed over groups.
 */
int gg_bfs_levels_batch(gg_ctx* ctx, const gg_mat* A_T, const int64_t* sources, int64_t S,
                        int32_t* dist, int64_t ld, int64_t* levels_out);

/*
 * Batched shortest paths from the standard start: column q of dist receives
 * shortest_path(A_T, sources[q]), as the reference's multi-source shortest_path
 * (src/algorithms/shortest_path.jl:88-161) computes with a min-plus SpMM per round.
 * 32 sources per pass, relaxing only from vertices that changed in the previous
 * round.  Needs non-negative weights (GG_ERR_UNSUPPORTED otherwise; gg_sssp then
 * runs the reference's Jacobi rounds).  gg_sssp routes several sources here.
 * Memory: a 32-column distance block (n x 32 elements) per group of 32 sources, up to
 * 8 groups at once; for CSR graphs of at least 65536 vertices with 4-byte distances
 * the rounds over every vertex also use the SELL-32 copy of A_T that single-source
 * gg_sssp builds (about the size of the CSR), built by the first call that needs it
 * (when it does not fit, those rounds run vertex by vertex instead).
 */
int gg_sssp_batch(gg_ctx* ctx, const gg_mat* A_T, const int64_t* sources, int64_t S, void* dist,
                  int dist_dtype, int64_t ld, int64_t* rounds_out);

/*
 * BFS levels for callers that cannot allocate device memory (no counterpart in the
 * reference).  Same result as gg_bfs_levels -- dist[v] = hop level along edges with
 * odd / true stored values (all stored edges when nzval is NULL), dist[source] = 0,
 * unreached entries untouched -- computed from plain device pointers to the 1-based
 * CSR arrays of A_T (rowptr n+1, colval nnz, nzval nnz of type dtype) on the current
 * device, on `stream` (NULL = legacy default stream).  Calls no cudaMalloc /
 * cudaFree: its working state lives in a fixed array of the library sized for at
 * most 4,194,304 vertices (1.5 MiB, held by every GPU that loads the library until
 * exit); larger n returns GG_ERR_ARGUMENT.  Every call looks up that array's device
 * address on the current device (the lookup allocates nothing); the first call on a
 * device also loads the library's device code there, so make it before any stream
 * capture.  All calls share
 * the one array: calls whose work overlaps on the GPU race and must be ordered by
 * the caller.  Bottom-up only: O(levels * (n + nnz)) work.  The CSR arrays are not
 * validated.  Synchronous.
 */
int gg_bfs_levels_noalloc(const int32_t* rowptr, const int32_t* colval, const void* nzval,
                          int dtype, int64_t n, int64_t nnz, int64_t source, int32_t* dist,
                          void* stream, int64_t* levels_out);

/* ---- serving (no reference counterpart) ------------------------------------------
 * A scheduler thread keeps per (graph, query kind) executors with fixed slots --
 * 256 BFS slots (bits of packed frontier words), 32 shortest-path columns, 32 SpMV
 * columns -- and advances every active slot one level / round / step per tick.
 * Requests arriving meanwhile join free slots at the next tick (continuous
 * batching); executors are created only when cudaMemGetInfo shows their memory plus
 * reserve_bytes free (admission by free HBM), otherwise requests wait.  Results
 * equal the single-query functions: BFS -> gg_bfs_levels semantics with unreached =
 * typemax(Int32); SSSP -> gg_sssp (non-negative weights); SPMV_ITER -> `steps` times
 * x <- A*x with the plus-times Float32 semiring. */

/* Server bound to ctx's device, with its own stream and worker thread. */
int gg_server_create(gg_ctx* ctx, int64_t reserve_bytes, gg_server** out);
/* Registers a resident graph (A_T must outlive the server); before the first submit. */
int gg_server_add_graph(gg_server* server, const gg_mat* A_T, int* graph_id);
/* Queues a query.  out: device array of n results (Int32 levels, distances of the
 * shortest_path element type, or Float32); x: device start vector for SPMV_ITER. */
int gg_server_submit(gg_server* server, int kind, int graph, int64_t source, const float* x,
                     int steps, void* out, int64_t* request_id);
/* Non-blocking: up to max completed request ids with their latencies (seconds from
 * submit to result in `out`); inflight receives the number still pending. */
int gg_server_poll(gg_server* server, int64_t* ids, double* latency_s, int64_t max,
                   int64_t* ndone, int64_t* inflight);
/* Ticks run, executor creations deferred for lack of free HBM, executor bytes held. */
int gg_server_stats(gg_server* server, int64_t* ticks, int64_t* admission_waits,
                    int64_t* exec_bytes);
/* Stops the worker and frees the executors (queued requests are dropped). */
int gg_server_destroy(gg_server* server);

/* ---- many graphs per launch (no reference counterpart) ---------------------------
 * G square CSR graphs (one element type) concatenated with 64-bit offsets: vertex v
 * of graph g has the global id row_offsets[g] + v - 1 in the concatenated vectors. */

/* Copies the graphs into one structure (the handles may be destroyed afterwards). */
int gg_multigraph_create(gg_ctx* ctx, const gg_mat* const* graphs, int64_t ngraphs,
                         gg_multigraph** out);
int gg_multigraph_destroy(gg_multigraph* mg);
/* Graph count, total vertices, total entries, and (if not NULL) the G+1 offsets. */
int gg_multigraph_info(const gg_multigraph* mg, int64_t* ngraphs, int64_t* total_n,
                       int64_t* total_nnz, int64_t* row_offsets);
/* y_g = A_g * x_g (plus-times Float32) for every graph in one kernel launch;
 * x, y: concatenated device vectors of total_n entries.  Asynchronous. */
int gg_multigraph_spmv(gg_ctx* ctx, const gg_multigraph* mg, const float* x, float* y);
/* One BFS per graph (sources[g], 1-based within graph g, host array) in one
 * persistent cooperative launch captured in a CUDA graph (re-captured when dist
 * changes).  dist: concatenated Int32 device vector, levels as bfs_distances of
 * each graph with rows of A_T used as out-edges (exact for symmetric graphs; a
 * floating-point graph is searched over its Bool pattern, every stored entry an
 * edge), typemax(Int32) when unreached.  Synchronous; GG_ERR_TIMEOUT if the grid barrier's
 * bounded wait ran out.  levels_out: levels run (deepest graph). */
int gg_multigraph_bfs(gg_ctx* ctx, gg_multigraph* mg, const int64_t* sources, int32_t* dist,
                      int64_t* levels_out);
/* One shortest-path search per graph (sources[g], 1-based within graph g, host
 * array) in one persistent cooperative launch captured in a CUDA graph: frontier
 * Bellman-Ford with atomic min, the fixpoint of shortest_path of each graph
 * (src/algorithms/shortest_path.jl:12-83) with rows of A_T used as out-edges (exact
 * for symmetric graphs).  dist: concatenated device vector of dist_dtype (Int32 for
 * Bool graphs, else the graphs' type), typemax / +Inf when unreached.  Needs
 * non-negative weights (GG_ERR_UNSUPPORTED otherwise).  Synchronous; GG_ERR_TIMEOUT
 * if the grid barrier's bounded wait ran out.  rounds_out: rounds run. */
int gg_multigraph_sssp(gg_ctx* ctx, gg_multigraph* mg, const int64_t* sources, void* dist,
                       int dist_dtype, int64_t* rounds_out);

/* ---- autotuning (no reference counterpart: the reference's layouts are fixed,
 *      src/storage/SELL.jl:99-181) -------------------------------------------------- */

typedef struct gg_tune_result {
  int spmv_kernel;         /* 1 = CSR row blocks, 2 = a SELL-C-sigma layout, 3 = column-window tiles */
  int block_rows;          /* rows per row block (spmv_kernel 1) */
  int64_t slice_size;      /* C (spmv_kernel 2) */
  int64_t sigma;           /* sigma (spmv_kernel 2) */
  double spmv_ms;          /* median time of the chosen SpMV configuration */
  double spmv_default_ms;  /* median time of the built-in choice */
  int mm_cols_per_lane;    /* SpMM column tile: 32 x this columns per warp pass */
  double spmm_ms;          /* median time of the chosen SpMM tile (spmm_k > 0) */
  int candidates;          /* configurations timed */
  int sell_variant;        /* SELL-32 plus-times kernel: 0 = register loads, 1 = matrix
                              stream staged in shared memory by bulk copies, 2 = register
                              loads with the hub rows folded from shared-memory column
                              windows where dense enough (gg_spmv_hub_rows) (-1 in
                              gg_tune_apply: leave as is) */
  int hot_cols;            /* most frequent x values staged in shared memory by the register
                              kernel (0: built-in 32768; at most 53248) */
} gg_tune_result;

/*
 * Times the Float32 plus-times SpMV of A over a grid of layouts (CSR row blocks of
 * 32..256 rows; SELL-C-sigma copies, C in {8,16,32}, sigma in {1,64,1024,m}) and,
 * when spmm_k > 0, the SpMM column tile (32, 64, 128 columns per warp pass) for a
 * row-major n x spmm_k operand; keeps the fastest on the handle for later calls.
 * Results of every configuration are identical for rows folded in storage order.
 * GG_ERR_UNSUPPORTED unless A is Float32.  Synchronous.
 */
int gg_tune(gg_ctx* ctx, gg_mat* A, int64_t spmm_k, gg_tune_result* out);
/* Applies a choice (e.g. one cached from an earlier gg_tune of the same matrix)
 * without timing: spmv_kernel 1 with block_rows, 2 with slice_size and sigma (a SELL
 * copy of a CSR handle is built), 3 column-window tiles (CSR handles; built on the
 * next call), 0 leaves SpMV as is; mm_cols_per_lane 1, 2 or 4
 * (0 leaves SpMM as is).  Synchronous. */
int gg_tune_apply(gg_ctx* ctx, gg_mat* A, const gg_tune_result* choice);
/* Layout the last plus-times Float32 gg_spmv of A ran on: 0 = none yet, 1 = CSR row
 * blocks, 2 = a SELL-C-sigma layout (the handle itself or a copy), 3 = column-window
 * tiles.  No reference counterpart (introspection of the layouts gg_tune chooses). */
int gg_spmv_layout(const gg_mat* A);
/* Rows of A whose plus-times Float32 gg_spmv is folded from shared-memory column
 * windows (sell_variant 2 of gg_tune_apply): the hub rows (more than 128 entries,
 * longest first) of the sorted SELL-32 layout, when its analysis (run by the first
 * such call) found groups of them dense enough; 0 otherwise.  Those rows are summed in a fixed order (window after window,
 * storage order inside a window), so results are identical from call to call and
 * within rounding of the storage-order fold.  The layout costs about 6 bytes per hub
 * entry of extra device memory beside the SELL-32 copy.  No reference counterpart
 * (introspection of the layouts gg_tune chooses). */
int64_t gg_spmv_hub_rows(const gg_mat* A);

/* ---- seeded synthetic inputs (no reference counterpart: the reference's benchmark
 *      draws its inputs with Julia's sprand / Graphs.jl generators,
 *      benchmark/benchmarks.jl:57-63,100-104) ------------------------------------ */

enum {
  GG_W_PATTERN = 0,   /* Bool true */
  GG_W_U01_F32 = 1,   /* Float32 uniform [0, 1) */
  GG_W_INT_1_255 = 2, /* Int32 uniform 1..255 */
  GG_W_F32_1_10 = 3   /* Float32 uniform [1, 10) */
};

/*
 * Edge lists written to device arrays (1-based vertex ids, generation order).
 * Edge e draws its random numbers from splitmix64(splitmix64(seed) + 64*e + j), so
 * any edge can be regenerated alone.  weights may be NULL.
 * R-MAT: 2^scale vertices, quadrant probabilities a, b, c, 1-a-b-c.
 * Erdos-Renyi: uniform (src, dst) pairs over n vertices.
 * Grid: H x W 4-neighbour lattice, H*(W-1) + (H-1)*W undirected edges.
 */
int gg_gen_rmat_edges(gg_ctx* ctx, int scale, int64_t nedges, double a, double b, double c,
                      uint64_t seed, int weight_kind, int32_t* src, int32_t* dst, void* weights);
int gg_gen_er_edges(gg_ctx* ctx, int64_t n, int64_t nedges, uint64_t seed, int weight_kind,
                    int32_t* src, int32_t* dst, void* weights);
int gg_gen_grid_edges(gg_ctx* ctx, int64_t H, int64_t W, uint64_t seed, int weight_kind,
                      int32_t* src, int32_t* dst, void* weights);
/* Dense Float32 vector, element i uniform [0, 1) from the same stream definition. */
int gg_gen_uniform_f32(gg_ctx* ctx, int64_t len, uint64_t seed, float* out);

#ifdef __cplusplus
}
#endif

#endif /* GPUGRAPHS_H */
