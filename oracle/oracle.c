/*
 * oracle.c -- CPU restatement of GPUGraphs.jl's semiring sparse kernels, SELL
 * builder, BFS and Bellman-Ford, written to check the CUDA library.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file; the
 * parity tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it as
 * the checker.  Each function cites the reference file:line whose behaviour it
 * restates (paths relative to the GPUGraphs.jl repository).
 *
 * Parity pins: the SELL layout golden vector of test/structs.jl:176-190, the
 * constructor error cases of test/structs.jl:79-149, and the reference's own test
 * oracles (SparseArrays A*b, Graphs.gdistances, dijkstra_shortest_paths) restated
 * through scipy / networkx in tests/test_oracle_cpu.py.
 *
 * Arithmetic follows Julia exactly: Int32/Int64 wrap, Float32 operations round once
 * each (this file is compiled with -ffp-contract=off), min/max propagate NaN and
 * order -0.0 below +0.0, Bool values are 0/1 bytes.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* element types and operators share the numbering of include/gpugraphs.h */
enum { T_BOOL = 1, T_I32 = 2, T_I64 = 3, T_F32 = 4, T_F64 = 5 };
enum {
  OP_FIRST = 1, OP_SECOND, OP_ANY, OP_PAIR, OP_ADD, OP_SAFE_ADD, OP_MINUS, OP_RMINUS,
  OP_MUL, OP_MIN, OP_MAX, OP_LOR, OP_LAND, OP_BOR, OP_BAND, OP_BXOR, OP_FIRSTI,
  OP_FIRSTJ, OP_SECONDI, OP_SECONDJ
};
enum { ORC_OK = 0, ORC_DIM = 1, ORC_ARG = 2, ORC_TYPE = 3, ORC_UNSUPPORTED = 4, ORC_ASSERT = 9 };

/* ------------------------------------------------------------------------------ */
/* scalar engine                                                                    */
/* ------------------------------------------------------------------------------ */

typedef struct {
  int t;
  int64_t i; /* BOOL / INT32 / INT64 */
  float f;   /* FLOAT32 */
  double d;  /* FLOAT64 */
} val;

static int is_float(int t) { return t == T_F32 || t == T_F64; }

static val wrap(val v) {
  if (v.t == T_I32) v.i = (int32_t)(uint32_t)(uint64_t)v.i;
  if (v.t == T_BOOL) v.i = v.i & 1;
  return v;
}

static val vi(int t, int64_t i) { val v; v.t = t; v.i = i; v.f = 0; v.d = 0; return wrap(v); }
static val vf(float f) { val v; v.t = T_F32; v.i = 0; v.f = f; v.d = 0; return v; }
static val vd(double d) { val v; v.t = T_F64; v.i = 0; v.f = 0; v.d = d; return v; }

/* Julia convert / promotion between the five element types */
static val cvt(val x, int t) {
  if (x.t == t) return x;
  if (!is_float(x.t)) {
    if (t == T_F32) return vf((float)x.i);
    if (t == T_F64) return vd((double)x.i);
    if (t == T_BOOL) return vi(t, x.i != 0);
    return vi(t, x.i);
  }
  double s = (x.t == T_F32) ? (double)x.f : x.d;
  if (t == T_F32) return vf((float)s);
  if (t == T_F64) return vd(s);
  if (t == T_BOOL) return vi(t, s != 0.0);
  return vi(t, (int64_t)s);
}

static val load(const void* p, int t, int64_t k) {
  switch (t) {
    case T_BOOL: return vi(T_BOOL, ((const uint8_t*)p)[k] != 0);
    case T_I32: return vi(T_I32, ((const int32_t*)p)[k]);
    case T_I64: return vi(T_I64, ((const int64_t*)p)[k]);
    case T_F32: return vf(((const float*)p)[k]);
    default: return vd(((const double*)p)[k]);
  }
}

static void store(void* p, int t, int64_t k, val v) {
  v = cvt(v, t);
  switch (t) {
    case T_BOOL: ((uint8_t*)p)[k] = (uint8_t)(v.i & 1); break;
    case T_I32: ((int32_t*)p)[k] = (int32_t)v.i; break;
    case T_I64: ((int64_t*)p)[k] = v.i; break;
    case T_F32: ((float*)p)[k] = v.f; break;
    default: ((double*)p)[k] = v.d; break;
  }
}

static val typemax(int t) {
  switch (t) {
    case T_BOOL: return vi(t, 1);
    case T_I32: return vi(t, INT32_MAX);
    case T_I64: return vi(t, INT64_MAX);
    case T_F32: return vf(INFINITY);
    default: return vd(INFINITY);
  }
}
static val typemin(int t) {
  switch (t) {
    case T_BOOL: return vi(t, 0);
    case T_I32: return vi(t, INT32_MIN);
    case T_I64: return vi(t, INT64_MIN);
    case T_F32: return vf(-INFINITY);
    default: return vd(-INFINITY);
  }
}

static int is_zero(val x) {
  if (x.t == T_F32) return x.f == 0.0f;
  if (x.t == T_F64) return x.d == 0.0;
  return x.i == 0;
}

/* Julia `==` (IEEE for floats) */
static int veq(val a, val b) {
  if (a.t == T_F32) return a.f == b.f;
  if (a.t == T_F64) return a.d == b.d;
  return a.i == b.i;
}

/* Julia max/min: NaN if either is NaN; -0.0 < +0.0 (base/math.jl semantics) */
static double jl_maxd(double x, double y) {
  if (isnan(x) || isnan(y)) return NAN;
  if (x == y) return signbit(x) ? y : x;
  return x > y ? x : y;
}
static double jl_mind(double x, double y) {
  if (isnan(x) || isnan(y)) return NAN;
  if (x == y) return signbit(x) ? x : y;
  return x < y ? x : y;
}

static val vmax(val x, val y) {
  if (x.t == T_F32) return vf((float)jl_maxd(x.f, y.f));
  if (x.t == T_F64) return vd(jl_maxd(x.d, y.d));
  return vi(x.t, x.i > y.i ? x.i : y.i);
}
static val vmin(val x, val y) {
  if (x.t == T_F32) return vf((float)jl_mind(x.f, y.f));
  if (x.t == T_F64) return vd(jl_mind(x.d, y.d));
  return vi(x.t, x.i < y.i ? x.i : y.i);
}

static val vadd(val x, val y) {
  if (x.t == T_F32) return vf(x.f + y.f);
  if (x.t == T_F64) return vd(x.d + y.d);
  return vi(x.t, (int64_t)((uint64_t)x.i + (uint64_t)y.i));
}
static val vsub(val x, val y) {
  if (x.t == T_F32) return vf(x.f - y.f);
  if (x.t == T_F64) return vd(x.d - y.d);
  return vi(x.t, (int64_t)((uint64_t)x.i - (uint64_t)y.i));
}
static val vmul(val x, val y) {
  if (x.t == T_F32) return vf(x.f * y.f);
  if (x.t == T_F64) return vd(x.d * y.d);
  if (x.t == T_BOOL) return vi(x.t, x.i & y.i);
  return vi(x.t, (int64_t)((uint64_t)x.i * (uint64_t)y.i));
}

/* src/algebra.jl:47-48: ifelse(max(x,y) == max(typemax(x),typemax(y)), typemax, x+y) */
static val vsafe_add(val x, val y) {
  val tm = typemax(x.t);
  val mx = vmax(x, y);
  if (veq(mx, tm)) return tm;
  return vadd(x, y);
}

static int is_index_op(int op) {
  return op == OP_FIRSTI || op == OP_FIRSTJ || op == OP_SECONDI || op == OP_SECONDJ;
}

/* element type the accumulator lives in: promote_type(Tv, Tx) widened by index
   operators (row / column ids are Int64 / Int32 in the reference kernels) */
static int compute_type(int tv, int tx, int mul) {
  int tc = tv > tx ? tv : tx;
  if ((mul == OP_FIRSTJ || mul == OP_SECONDI) && tc < T_I32) tc = T_I32;
  if ((mul == OP_FIRSTI || mul == OP_SECONDJ) && tc < T_I64) tc = T_I64;
  return tc;
}

/* does Julia define `op` on values of type t without leaving t? */
static int op_defined(int op, int t) {
  switch (op) {
    case OP_ADD: case OP_SAFE_ADD: case OP_MINUS: case OP_RMINUS:
      return t != T_BOOL; /* Bool + Bool is Int */
    case OP_LOR: case OP_LAND: case OP_BOR: case OP_BAND: case OP_BXOR:
      return !is_float(t);
    default:
      return 1;
  }
}

/* monoid_neutral / monoid_absorb, src/algebra.jl:10-100 */
static int neutral_of(int add, int t, val* out) {
  switch (add) {
    case OP_ADD: case OP_SAFE_ADD: case OP_ANY: case OP_BOR: *out = cvt(vi(T_I64, 0), t); return 1;
    case OP_MUL: *out = cvt(vi(T_I64, 1), t); return 1;
    case OP_MIN: *out = typemax(t); return 1;
    case OP_MAX: *out = typemin(t); return 1;
    case OP_BAND: *out = (t == T_BOOL) ? vi(t, 1) : cvt(vi(T_I64, -1), t); return !is_float(t);
    case OP_LOR: *out = vi(T_BOOL, 0); return t == T_BOOL;
    case OP_LAND: *out = vi(T_BOOL, 1); return t == T_BOOL;
    default: return 0;
  }
}
static int absorb_of(int add, int t, val* out) {
  switch (add) {
    case OP_ADD: case OP_SAFE_ADD: case OP_MAX: *out = typemax(t); return 1;
    case OP_MUL: *out = cvt(vi(T_I64, 0), t); return 1;
    case OP_MIN: *out = typemin(t); return 1;
    case OP_BOR: *out = (t == T_BOOL) ? vi(t, 1) : cvt(vi(T_I64, -1), t); return 1;
    case OP_BAND: *out = cvt(vi(T_I64, 0), t); return 1;
    case OP_LOR: *out = vi(T_BOOL, 1); return 1;
    case OP_LAND: *out = vi(T_BOOL, 0); return 1;
    default: return 0; /* GPUGraphs_any: absorb is the type Any, never equal to a value */
  }
}

/*
 * op(x, y, A_i, A_j, B_i, B_j) of src/algebra.jl:31-111 evaluated in type tc.
 * x, y are already converted to tc; yraw is y before conversion (GPUGraphs_secondi
 * multiplies the Int32 column by the raw y, algebra.jl:109).
 */
static val apply(int op, int tc, val x, val y, val yraw, int64_t ai, int64_t aj, int64_t bi,
                 int64_t bj) {
  switch (op) {
    case OP_FIRST: return x;
    case OP_SECOND: return y;
    case OP_ANY: return vmax(x, y);
    case OP_PAIR: return is_zero(y) ? cvt(vi(T_I64, 0), tc) : cvt(vi(T_I64, 1), tc);
    case OP_ADD: return vadd(x, y);
    case OP_SAFE_ADD: return vsafe_add(x, y);
    case OP_MINUS: return vsub(x, y);
    case OP_RMINUS: return vsub(y, x);
    case OP_MUL: return vmul(x, y);
    case OP_MIN: return vmin(x, y);
    case OP_MAX: return vmax(x, y);
    case OP_LOR: case OP_BOR: return vi(tc, x.i | y.i);
    case OP_LAND: case OP_BAND: return vi(tc, x.i & y.i);
    case OP_BXOR: return vi(tc, x.i ^ y.i);
    case OP_FIRSTI: return cvt(vi(T_I64, ai), tc);
    case OP_FIRSTJ: return cvt(vi(T_I32, aj), tc);
    case OP_SECONDJ: return cvt(vi(T_I64, bj), tc);
    case OP_SECONDI: {
      int tp = yraw.t > T_I32 ? yraw.t : T_I32; /* promote_type(Int32, typeof(y)) */
      val p = vmul(cvt(vi(T_I32, bi), tp), cvt(yraw, tp));
      return cvt(p, tc);
    }
  }
  return x;
}

/* Shared validation of the semiring for a (tv, tx, ty) call; mirrors the type rule
   of _validate_args (src/spmv/CSR.jl:381-387) with Ty >= promote_type(Tv, Tx). */
static int check_semiring(int tv, int tx, int ty, int mul, int add, int accum, int* tc_out) {
  int tc = compute_type(tv, tx, mul);
  int tp = tv > tx ? tv : tx;
  if (ty < tp || ty < tc) return ORC_TYPE;
  if (!is_index_op(mul) && !op_defined(mul, tc)) return ORC_UNSUPPORTED;
  if (!op_defined(add, tc)) return ORC_UNSUPPORTED;
  if (!is_index_op(accum) && !op_defined(accum, ty)) return ORC_UNSUPPORTED;
  val nv;
  if (!neutral_of(add, tc, &nv)) return ORC_UNSUPPORTED;
  *tc_out = tc;
  return ORC_OK;
}

static int row_selected(int64_t r /*1-based*/, const void* mask, int tmask, int64_t lo,
                        int64_t hi) {
  if (lo > 0 && (r < lo || r > hi)) return 0;
  if (mask && is_zero(load(mask, tmask, r - 1))) return 0;
  return 1;
}

/* ------------------------------------------------------------------------------ */
/* CSR SpMV: src/spmv/CSR.jl:31-54 (plain), :117-144 (dense mask), :147-171 (any),  */
/* :224-248 (range), :285-313 (range + mask)                                         */
/* ------------------------------------------------------------------------------ */

int orc_csr_spmv(int64_t m, int64_t n, const int32_t* rowptr, const int32_t* colval,
                 const void* nzval, int tv, void* y, int ty, const void* x, int tx,
                 const void* mask, int tmask, int64_t range_lo, int64_t range_hi, int mul,
                 int add, int accum) {
  (void)n;
  int tc;
  int rc = check_semiring(tv, tx, ty, mul, add, accum, &tc);
  if (rc) return rc;
  val neutral, absorb;
  neutral_of(add, tc, &neutral);
  int has_absorb = absorb_of(add, tc, &absorb);
  /* any_dense_masked_csr_spmv_kernel! is chosen for add == any with a mask and no
     range (src/spmv/CSR.jl:191-204) */
  int first_hit = (add == OP_ANY && mask != NULL && range_lo == 0);
  for (int64_t r = 1; r <= m; ++r) {
    if (!row_selected(r, mask, tmask, range_lo, range_hi)) continue;
    if (first_hit) {
      for (int64_t i = rowptr[r - 1]; i <= rowptr[r] - 1; ++i) {
        int64_t col = colval[i - 1];
        val b = load(x, tx, col - 1);
        if (!is_zero(b)) {
          val a = cvt(load(nzval, tv, i - 1), tc);
          val mres = apply(mul, tc, a, cvt(b, tc), b, r, col, col, 1);
          val yo = load(y, ty, r - 1);
          val acc = cvt(mres, ty);
          store(y, ty, r - 1, apply(accum, ty, yo, acc, acc, r, 1, r, 1));
          break;
        }
      }
      continue;
    }
    val acc = neutral;
    for (int64_t i = rowptr[r - 1]; i <= rowptr[r] - 1; ++i) {
      int64_t col = colval[i - 1];
      val b = load(x, tx, col - 1);
      val a = cvt(load(nzval, tv, i - 1), tc);
      val mres = apply(mul, tc, a, cvt(b, tc), b, r, col, col, 1);
      acc = apply(add, tc, acc, mres, mres, r, col, col, 1);
      if (has_absorb && veq(acc, absorb)) break;
    }
    val yo = load(y, ty, r - 1);
    val a2 = cvt(acc, ty);
    store(y, ty, r - 1, apply(accum, ty, yo, a2, a2, r, 1, r, 1));
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------------ */
/* SELL-C storage builder: src/storage/SELL.jl:99-181                               */
/* ------------------------------------------------------------------------------ */

/*
 * Sizes of the SELL layout: slice_size is clamped to m (SELL.jl:108), nslices =
 * ceil(m / C) (:109), n_stored = sum over slices of C * max row length (:119-125).
 * With sigma > 1 rows are sorted by decreasing length (stable) inside windows of
 * sigma rows before slicing (SELL-C-sigma; the reference's perm is the identity,
 * :113-116, which is sigma == 1).  perm[s] = 1-based original row of stored row s.
 */
int orc_sell_sizes(int64_t m, const int32_t* rowptr, int64_t slice_size, int64_t sigma,
                   int64_t* C_out, int64_t* nslices_out, int64_t* n_stored_out, int32_t* perm) {
  int64_t C = slice_size < m ? slice_size : m;
  if (C <= 0) { *C_out = C; *nslices_out = 0; *n_stored_out = 0; return ORC_OK; }
  int64_t ns = (m + C - 1) / C;
  for (int64_t r = 0; r < m; ++r) perm[r] = (int32_t)(r + 1);
  if (sigma > 1) {
    for (int64_t w0 = 0; w0 < m; w0 += sigma) {
      int64_t w1 = w0 + sigma < m ? w0 + sigma : m;
      /* stable insertion-merge by decreasing length: simple stable sort */
      for (int64_t i = w0 + 1; i < w1; ++i) {
        int32_t p = perm[i];
        int64_t len = rowptr[p] - rowptr[p - 1];
        int64_t j = i - 1;
        while (j >= w0 && (rowptr[perm[j]] - rowptr[perm[j] - 1]) < len) {
          perm[j + 1] = perm[j];
          --j;
        }
        perm[j + 1] = p;
      }
    }
  }
  int64_t nst = 0;
  for (int64_t s = 0; s < ns; ++s) {
    int64_t mx = 0;
    for (int64_t r = s * C; r < (s + 1) * C && r < m; ++r) {
      int64_t len = rowptr[perm[r]] - rowptr[perm[r] - 1];
      if (len > mx) mx = len;
    }
    nst += mx * C;
  }
  *C_out = C;
  *nslices_out = ns;
  *n_stored_out = nst;
  return ORC_OK;
}

/* Fill slice_ptr (1-based, nslices+1), colval (-1 padded) and nzval (0 padded) in the
   slice-column-major order of SELL.jl:134-165 (element j of slice row o sits at
   slice_ptr[s] + j*C + o). */
int orc_sell_fill(int64_t m, const int32_t* rowptr, const int32_t* colval, const void* nzval,
                  int tv, int64_t C, int64_t nslices, const int32_t* perm, int32_t* slice_ptr,
                  int32_t* s_colval, void* s_nzval) {
  slice_ptr[0] = 1;
  for (int64_t s = 0; s < nslices; ++s) {
    int64_t mx = 0;
    for (int64_t r = s * C; r < (s + 1) * C && r < m; ++r) {
      int64_t len = rowptr[perm[r]] - rowptr[perm[r] - 1];
      if (len > mx) mx = len;
    }
    slice_ptr[s + 1] = (int32_t)(slice_ptr[s] + mx * C);
    int64_t base = slice_ptr[s] - 1;
    for (int64_t j = 0; j < mx; ++j) {
      for (int64_t o = 0; o < C; ++o) {
        int64_t dst = base + j * C + o;
        int64_t r = s * C + o;
        int64_t len = 0, start = 0;
        if (r < m) {
          start = rowptr[perm[r] - 1] - 1;
          len = rowptr[perm[r]] - rowptr[perm[r] - 1];
        }
        if (j < len) {
          s_colval[dst] = colval[start + j];
          store(s_nzval, tv, dst, load(nzval, tv, start + j));
        } else {
          s_colval[dst] = -1;
          store(s_nzval, tv, dst, vi(T_I64, 0));
        }
      }
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------------ */
/* SELL SpMV: src/spmv/SELL.jl:31-63 (plain), :100-133 (mask), :176-209 (range),   */
/* :249-283 (range + mask).  Stops at the first padding column (-1), no absorb exit. */
/* ------------------------------------------------------------------------------ */

int orc_sell_spmv(int64_t m, int64_t n, int64_t C, int64_t nslices, const int32_t* slice_ptr,
                  const int32_t* s_colval, const void* s_nzval, int tv, const int32_t* perm,
                  void* y, int ty, const void* x, int tx, const void* mask, int tmask,
                  int64_t range_lo, int64_t range_hi, int mul, int add, int accum) {
  (void)n;
  int tc;
  int rc = check_semiring(tv, tx, ty, mul, add, accum, &tc);
  if (rc) return rc;
  val neutral;
  neutral_of(add, tc, &neutral);
  for (int64_t s = 0; s < nslices; ++s) {
    for (int64_t o = 0; o < C; ++o) {
      int64_t sr = s * C + o;
      if (sr >= m) break;
      int64_t r = perm[sr];
      if (!row_selected(r, mask, tmask, range_lo, range_hi)) continue;
      val acc = neutral;
      for (int64_t i = slice_ptr[s] + o; i <= slice_ptr[s + 1] - 1; i += C) {
        int64_t col = s_colval[i - 1];
        if (col == -1) break;
        val b = load(x, tx, col - 1);
        val a = cvt(load(s_nzval, tv, i - 1), tc);
        val mres = apply(mul, tc, a, cvt(b, tc), b, r, col, col, 1);
        acc = apply(add, tc, acc, mres, mres, r, col, col, 1);
      }
      val yo = load(y, ty, r - 1);
      val a2 = cvt(acc, ty);
      store(y, ty, r - 1, apply(accum, ty, yo, a2, a2, r, 1, r, 1));
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------------ */
/* SpMM: src/spmm/CSR.jl:3-35,37-71,73-109 and src/spmm/SELL.jl:2-39,41-82.         */
/* B is nb x k, C is m x k; layout 0 = column-major (Julia), 1 = row-major.          */
/* The accumulator starts at monoid_neutral(promote_type(Tv, Tx), add) for both      */
/* formats (the SELL rule, src/spmm/SELL.jl:115).                                    */
/* ------------------------------------------------------------------------------ */

static int64_t dense_idx(int64_t r, int64_t j, int64_t ld, int layout) {
  return layout == 0 ? r + j * ld : r * ld + j;
}

int orc_csr_spmm(int64_t m, const int32_t* rowptr, const int32_t* colval, const void* nzval,
                 int tv, void* Cm, int tcm, int64_t ldc, const void* B, int tb, int64_t ldb,
                 int64_t k, int layout, const void* mask, int tmask, int64_t range_lo,
                 int64_t range_hi, int mul, int add, int accum) {
  int tc;
  int rc = check_semiring(tv, tb, tcm, mul, add, accum, &tc);
  if (rc) return rc;
  val neutral, absorb;
  neutral_of(add, tc, &neutral);
  int has_absorb = absorb_of(add, tc, &absorb);
  for (int64_t r = 1; r <= m; ++r) {
    if (!row_selected(r, mask, tmask, range_lo, range_hi)) continue;
    for (int64_t j = 1; j <= k; ++j) {
      val acc = neutral;
      for (int64_t i = rowptr[r - 1]; i <= rowptr[r] - 1; ++i) {
        int64_t col = colval[i - 1];
        val b = load(B, tb, dense_idx(col - 1, j - 1, ldb, layout));
        val a = cvt(load(nzval, tv, i - 1), tc);
        val mres = apply(mul, tc, a, cvt(b, tc), b, r, col, col, j);
        acc = apply(add, tc, acc, mres, mres, r, col, col, j);
        if (has_absorb && veq(acc, absorb)) break;
      }
      int64_t ci = dense_idx(r - 1, j - 1, ldc, layout);
      val yo = load(Cm, tcm, ci);
      val a2 = cvt(acc, tcm);
      store(Cm, tcm, ci, apply(accum, tcm, yo, a2, a2, r, j, r, j));
    }
  }
  return ORC_OK;
}

int orc_sell_spmm(int64_t m, int64_t C, int64_t nslices, const int32_t* slice_ptr,
                  const int32_t* s_colval, const void* s_nzval, int tv, const int32_t* perm,
                  void* Cm, int tcm, int64_t ldc, const void* B, int tb, int64_t ldb, int64_t k,
                  int layout, const void* mask, int tmask, int64_t range_lo, int64_t range_hi,
                  int mul, int add, int accum) {
  int tc;
  int rc = check_semiring(tv, tb, tcm, mul, add, accum, &tc);
  if (rc) return rc;
  val neutral, absorb;
  neutral_of(add, tc, &neutral);
  int has_absorb = absorb_of(add, tc, &absorb);
  for (int64_t s = 0; s < nslices; ++s) {
    for (int64_t o = 0; o < C; ++o) {
      int64_t sr = s * C + o;
      if (sr >= m) break;
      int64_t r = perm[sr];
      if (!row_selected(r, mask, tmask, range_lo, range_hi)) continue;
      for (int64_t j = 1; j <= k; ++j) {
        val acc = neutral;
        for (int64_t i = slice_ptr[s] + o; i <= slice_ptr[s + 1] - 1; i += C) {
          int64_t col = s_colval[i - 1];
          if (col == -1 || (has_absorb && veq(acc, absorb))) break;
          val b = load(B, tb, dense_idx(col - 1, j - 1, ldb, layout));
          val a = cvt(load(s_nzval, tv, i - 1), tc);
          val mres = apply(mul, tc, a, cvt(b, tc), b, r, col, col, j);
          acc = apply(add, tc, acc, mres, mres, r, col, col, j);
        }
        int64_t ci = dense_idx(r - 1, j - 1, ldc, layout);
        val yo = load(Cm, tcm, ci);
        val a2 = cvt(acc, tcm);
        store(Cm, tcm, ci, apply(accum, tcm, yo, a2, a2, r, j, r, j));
      }
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------------ */
/* Graph algorithms.  A_T is given as CSR (rows = vertices, columns = in-neighbours) */
/* with values of type tv (Bool / Int32 / Int64 / Float32 / Float64).                */
/* ------------------------------------------------------------------------------ */

/* bit 0 of a stored value: GPUGraphs_band(a, 1) != 0 (the edge is active in the
   levels BFS, src/algorithms/bfs.jl:52-59 with algebra.jl:98) */
static int edge_odd(const void* nzval, int tv, int64_t k) {
  switch (tv) {
    case T_BOOL: return ((const uint8_t*)nzval)[k] & 1;
    case T_I32: return ((const int32_t*)nzval)[k] & 1;
    case T_I64: return (int)(((const int64_t*)nzval)[k] & 1);
    default: return 0;
  }
}

/*
 * bfs_distances(A_T, source) of src/algorithms/bfs.jl:1-73: level-synchronous,
 * masked (band, bor) SpMV per level over unvisited rows; a row joins level `iter`
 * when an in-neighbour in the current frontier has an odd (true) stored value.
 * dist is filled with typemax(Int32) first (bfs.jl:16-18).  Returns the number of
 * levels run (iterations of bfs.jl:50-71), or minus that number when max_levels > 0
 * stopped the search early (bounded CPU samples).  Parallel over rows.
 */
int64_t orc_bfs_levels(int64_t n, const int32_t* rowptr, const int32_t* colval,
                       const void* nzval, int tv, int64_t source, int32_t* dist,
                       int64_t max_levels) {
  uint8_t* curr = (uint8_t*)calloc((size_t)n, 1);
  uint8_t* next = (uint8_t*)calloc((size_t)n, 1);
  uint8_t* to_explore = (uint8_t*)malloc((size_t)n);
  memset(to_explore, 1, (size_t)n);
  for (int64_t v = 0; v < n; ++v) dist[v] = INT32_MAX;
  curr[source - 1] = 1;
  dist[source - 1] = 0;
  to_explore[source - 1] = 0;
  int32_t iter = 0;
  int64_t levels = 0;
  for (;;) {
    if (max_levels > 0 && levels >= max_levels) { levels = -levels; break; }
    ++iter;
    ++levels;
    int any = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : any)
    for (int64_t r = 0; r < n; ++r) {
      if (!to_explore[r]) continue;
      uint8_t acc = 0;
      for (int64_t i = rowptr[r] - 1; i < rowptr[r + 1] - 1; ++i) {
        int64_t c = colval[i] - 1;
        if (curr[c] && edge_odd(nzval, tv, i)) { acc = 1; break; } /* bor absorb: true */
      }
      next[r] = acc;
      any |= acc;
    }
    if (!any) break;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; ++r) {
      if (next[r] == 1) dist[r] = iter;
      to_explore[r] = to_explore[r] & (next[r] == 0);
      curr[r] = next[r];
      next[r] = 0;
    }
  }
  free(curr);
  free(next);
  free(to_explore);
  return levels;
}

/*
 * bfs_parents(A_T, source) of src/algorithms/bfs.jl:113-183: per level the masked
 * (secondi, any) SpMV gives, for every unvisited row, a frontier in-neighbour
 * column; stored values are ignored.  rule 1 (CSR, src/spmv/CSR.jl:147-171): the
 * first frontier column in storage order; rule 2 (SELL, algebra.jl:35 with
 * src/spmv/SELL.jl:100-133): the largest frontier column.  parents is filled with
 * typemax(Int32), the source gets 0 (bfs.jl:129,151).
 */
int64_t orc_bfs_parents(int64_t n, const int32_t* rowptr, const int32_t* colval,
                        int64_t source, int rule, int32_t* parents) {
  uint8_t* curr = (uint8_t*)calloc((size_t)n, 1);
  int32_t* next = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  uint8_t* to_explore = (uint8_t*)malloc((size_t)n);
  memset(to_explore, 1, (size_t)n);
  for (int64_t v = 0; v < n; ++v) parents[v] = INT32_MAX;
  curr[source - 1] = 1;
  parents[source - 1] = 0;
  to_explore[source - 1] = 0;
  int64_t levels = 0;
  for (;;) {
    ++levels;
    int any = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : any)
    for (int64_t r = 0; r < n; ++r) {
      if (!to_explore[r]) continue;
      int32_t p = 0;
      for (int64_t i = rowptr[r] - 1; i < rowptr[r + 1] - 1; ++i) {
        int32_t c = colval[i];
        if (curr[c - 1]) {
          if (rule == 1) { p = c; break; }
          if (c > p) p = c;
        }
      }
      next[r] = p;
      any |= (p != 0);
    }
    /* the reference tests `any(curr)` only every batch_size levels (bfs.jl:169-174);
       levels without a frontier change nothing, so testing every level is equal */
    if (!any) break;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; ++r) {
      curr[r] = next[r] != 0;
      if (curr[r]) parents[r] = next[r];
      to_explore[r] = to_explore[r] & (curr[r] == 0);
      next[r] = 0;
    }
  }
  free(curr);
  free(next);
  free(to_explore);
  return levels;
}

/*
 * shortest_path(A_T, source) of src/algorithms/shortest_path.jl:12-83 (single
 * source) and :88-161 (S sources, dist column-major n x S): Jacobi Bellman-Ford,
 *   next[r] = min(next[r], min_k safe_add(A[r,k], dist[k]));  dist .= next
 * until a round changes nothing.  dist type td = Int32 for Bool A, else tv
 * (shortest_path.jl:18).  dist and next start at typemax, sources at 0.  The single
 * source loop tests for progress every 8 rounds, the multi-source loop every round;
 * extra rounds after the fixpoint change nothing.  Returns the number of rounds, or
 * -1 if max_rounds was reached first.
 */
int64_t orc_sssp(int64_t n, const int32_t* rowptr, const int32_t* colval, const void* nzval,
                 int tv, const int64_t* sources, int64_t S, void* dist, int td,
                 int64_t max_rounds) {
  size_t esz = (td == T_I64 || td == T_F64) ? 8 : 4;
  void* next = malloc((size_t)n * (size_t)S * esz);
  for (int64_t q = 0; q < S; ++q) {
    for (int64_t v = 0; v < n; ++v) {
      store(dist, td, v + q * n, typemax(td));
      store(next, td, v + q * n, typemax(td));
    }
    store(dist, td, sources[q] - 1 + q * n, vi(T_I64, 0));
    store(next, td, sources[q] - 1 + q * n, vi(T_I64, 0));
  }
  int tc = td > tv ? td : tv;
  int64_t rounds = 0;
  int changed = 1;
  while (changed) {
    if (max_rounds > 0 && rounds >= max_rounds) { rounds = -1; break; }
    ++rounds;
    changed = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : changed)
    for (int64_t r = 0; r < n; ++r) {
      for (int64_t q = 0; q < S; ++q) {
        val acc = typemax(tc);
        for (int64_t i = rowptr[r] - 1; i < rowptr[r + 1] - 1; ++i) {
          val w = cvt(load(nzval, tv, i), tc);
          val d = cvt(load(dist, td, colval[i] - 1 + q * n), tc);
          acc = vmin(acc, vsafe_add(w, d));
        }
        val old = cvt(load(next, td, r + q * n), tc);
        val nv = vmin(old, acc);
        store(next, td, r + q * n, nv);
      }
    }
    for (int64_t idx = 0; idx < n * S; ++idx) {
      val a = load(next, td, idx), b = load(dist, td, idx);
      int lt = (td == T_F32) ? (a.f < b.f) : (td == T_F64) ? (a.d < b.d) : (a.i < b.i);
      if (lt) changed = 1;
    }
    memcpy(dist, next, (size_t)n * (size_t)S * esz);
  }
  free(next);
  return rounds;
}

/* ------------------------------------------------------------------------------ */
/* Cross-checks for full-size graphs.  The restatements above follow the           */
/* reference's level-synchronous BFS and Jacobi Bellman-Ford loops, which cost      */
/* O(levels x nnz) and O(rounds x nnz) -- hours on a 4096 x 4096 grid.  The         */
/* functions below reach the same results by other algorithms (frontier BFS,        */
/* Dijkstra) in O(nnz) / O(nnz log n); tests/test_oracle_cpu.py checks them against */
/* the restatements on graphs of every kind the tests use.                          */
/* ------------------------------------------------------------------------------ */

/* Out-edges of A_T (row v of A_T lists the in-neighbours u of v): for every column
   u the rows v of its entries, with the entry's value widened to the distance type
   when weights != 0.  pattern = 1 takes every stored entry, 0 only those with an
   odd (true) stored value, the edges bfs_distances! follows (edge_odd).  Rows of one
   column come in no particular order.  sym = 1 (with pattern = 1) states that A_T is
   symmetric with mirrored values: its rows are then its own out-edge lists. */
typedef struct {
  int64_t* ptr;  /* n + 1 */
  int32_t* row;  /* 0-based v */
  int32_t* wi;   /* integer weights (or NULL) */
  float* wf;     /* Float32 weights (or NULL) */
} outedges;

static void outedges_free(outedges* T) {
  free(T->ptr);
  free(T->row);
  free(T->wi);
  free(T->wf);
}

static int outedges_build(int64_t n, const int32_t* rowptr, const int32_t* colval,
                          const void* nzval, int tv, int pattern, int weights, int sym,
                          outedges* T) {
  memset(T, 0, sizeof(*T));
  int64_t nnz = rowptr[n] - 1;
  if (sym && pattern) {
    /* A_T == A (the caller says so): row u of A_T lists the out-neighbours of u */
    T->ptr = (int64_t*)malloc(((size_t)n + 1) * sizeof(int64_t));
    T->row = (int32_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int32_t));
    if (weights && tv == T_F32) T->wf = (float*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(float));
    if (weights && tv != T_F32) T->wi = (int32_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int32_t));
    if (!T->ptr || !T->row || (weights && !T->wf && !T->wi)) { outedges_free(T); return ORC_ARG; }
    for (int64_t u = 0; u <= n; ++u) T->ptr[u] = rowptr[u] - 1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nnz; ++i) {
      T->row[i] = colval[i] - 1;
      if (T->wf) T->wf[i] = ((const float*)nzval)[i];
      if (T->wi) T->wi[i] = (int32_t)load(nzval, tv, i).i;
    }
    return ORC_OK;
  }
  T->ptr = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  int64_t* fill = (int64_t*)malloc(((size_t)n + 1) * sizeof(int64_t));
  if (!T->ptr || !fill) { free(fill); outedges_free(T); return ORC_ARG; }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < n; ++v)
    for (int64_t i = rowptr[v] - 1; i < rowptr[v + 1] - 1; ++i)
      if (pattern || edge_odd(nzval, tv, i)) __atomic_fetch_add(&T->ptr[colval[i]], 1, __ATOMIC_RELAXED);
  for (int64_t u = 0; u < n; ++u) T->ptr[u + 1] += T->ptr[u];
  int64_t ne = T->ptr[n];
  memcpy(fill, T->ptr, ((size_t)n + 1) * sizeof(int64_t));
  T->row = (int32_t*)malloc((size_t)(ne > 0 ? ne : 1) * sizeof(int32_t));
  if (weights && tv == T_F32) T->wf = (float*)malloc((size_t)(ne > 0 ? ne : 1) * sizeof(float));
  if (weights && tv != T_F32) T->wi = (int32_t*)malloc((size_t)(ne > 0 ? ne : 1) * sizeof(int32_t));
  if (!T->row || (weights && !T->wf && !T->wi)) { free(fill); outedges_free(T); return ORC_ARG; }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < n; ++v)
    for (int64_t i = rowptr[v] - 1; i < rowptr[v + 1] - 1; ++i) {
      if (!pattern && !edge_odd(nzval, tv, i)) continue;
      int64_t at = __atomic_fetch_add(&fill[colval[i] - 1], 1, __ATOMIC_RELAXED);
      T->row[at] = (int32_t)v;
      if (T->wf) T->wf[at] = ((const float*)nzval)[i];
      if (T->wi) T->wi[at] = (int32_t)load(nzval, tv, i).i;
    }
  free(fill);
  (void)nnz;
  return ORC_OK;
}

/* Hop distances from the source along out-edges, one frontier at a time; a vertex
   is claimed by the first thread that moves its distance off typemax (every
   claimant writes the same level).  Equals bfs_distances(A_T, source) of
   src/algorithms/bfs.jl:1-73: a row joins level L exactly when an in-neighbour of
   level L-1 reaches it over an active entry. */
static int64_t frontier_bfs(int64_t n, const outedges* T, int64_t source, int32_t* dist) {
  int32_t* F = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
  int32_t* N = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
  if (!F || !N) { free(F); free(N); return -1; }
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < n; ++v) dist[v] = INT32_MAX;
  dist[source - 1] = 0;
  F[0] = (int32_t)(source - 1);
  int64_t nf = 1, level = 0;
  while (nf > 0) {
    int64_t nn = 0;
    const int32_t L = (int32_t)level + 1;
#pragma omp parallel
    {
      int32_t buf[256];
      int nb = 0;
#pragma omp for schedule(dynamic, 64)
      for (int64_t i = 0; i < nf; ++i) {
        const int32_t u = F[i];
        for (int64_t e = T->ptr[u]; e < T->ptr[u + 1]; ++e) {
          int32_t v = T->row[e];
          int32_t expect = INT32_MAX;
          if (__atomic_load_n(&dist[v], __ATOMIC_RELAXED) == INT32_MAX &&
              __atomic_compare_exchange_n(&dist[v], &expect, L, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
            buf[nb++] = v;
            if (nb == 256) {
              int64_t at = __atomic_fetch_add(&nn, nb, __ATOMIC_RELAXED);
              memcpy(N + at, buf, (size_t)nb * sizeof(int32_t));
              nb = 0;
            }
          }
        }
      }
      if (nb > 0) {
        int64_t at = __atomic_fetch_add(&nn, nb, __ATOMIC_RELAXED);
        memcpy(N + at, buf, (size_t)nb * sizeof(int32_t));
      }
    }
    int32_t* t = F;
    F = N;
    N = t;
    nf = nn;
    if (nf > 0) ++level;
  }
  free(F);
  free(N);
  return level;
}

/* bfs_distances(A_T, source) by frontier BFS; returns the largest level, or -1. */
int64_t orc_bfs_levels_fast(int64_t n, const int32_t* rowptr, const int32_t* colval,
                            const void* nzval, int tv, int64_t source, int32_t* dist, int sym) {
  outedges T;
  if (outedges_build(n, rowptr, colval, nzval, tv, nzval == NULL, 0, sym, &T) != ORC_OK) return -1;
  int64_t lv = frontier_bfs(n, &T, source, dist);
  outedges_free(&T);
  return lv;
}

/* bfs_parents(A_T, source) of src/algorithms/bfs.jl:113-183 from the pattern's hop
   distances: the frontier of the level that reaches row v is every vertex at
   distance dist[v] - 1, so v's parent is its first (rule 1, CSR) or largest (rule 2,
   SELL) in-neighbour column at that distance.  dist: hop distances over every
   stored entry (bfs_parents ignores stored values). */
void orc_bfs_parents_from_levels(int64_t n, const int32_t* rowptr, const int32_t* colval,
                                 const int32_t* dist, int64_t source, int rule,
                                 int32_t* parents) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < n; ++v) {
    if (v == source - 1) { parents[v] = 0; continue; }
    if (dist[v] == INT32_MAX) { parents[v] = INT32_MAX; continue; }
    const int32_t want = dist[v] - 1;
    int32_t p = 0;
    for (int64_t i = rowptr[v] - 1; i < rowptr[v + 1] - 1; ++i) {
      int32_t c = colval[i];
      if (dist[c - 1] == want) {
        if (rule == 1) { p = c; break; }
        if (c > p) p = c;
      }
    }
    parents[v] = p;
  }
}

/* Hop distances of S sources over every stored entry -- shortest_path(A_T,
   sources) with a Bool A_T (src/algorithms/shortest_path.jl:88-161) -- kept for the
   listed rows only: out[r + q * nrows] = distance of rows[r] (0-based) from source
   q (1-based sources[q]).  Sources run in parallel, a serial queue BFS each. */
int orc_bfs_levels_multi(int64_t n, const int32_t* rowptr, const int32_t* colval,
                         const int64_t* sources, int64_t S, const int64_t* rows,
                         int64_t nrows, int32_t* out, int sym) {
  outedges T;
  if (outedges_build(n, rowptr, colval, NULL, T_BOOL, 1, 0, sym, &T) != ORC_OK) return ORC_ARG;
  int fail = 0;
#pragma omp parallel reduction(| : fail)
  {
    int32_t* dist = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    int32_t* Q = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    if (!dist || !Q) fail = 1;
#pragma omp for schedule(dynamic, 1)
    for (int64_t q = 0; q < S; ++q) {
      if (!dist || !Q) continue;
      for (int64_t v = 0; v < n; ++v) dist[v] = INT32_MAX;
      int64_t head = 0, tail = 0;
      dist[sources[q] - 1] = 0;
      Q[tail++] = (int32_t)(sources[q] - 1);
      while (head < tail) {
        int32_t u = Q[head++];
        int32_t du = dist[u] + 1;
        for (int64_t e = T.ptr[u]; e < T.ptr[u + 1]; ++e) {
          int32_t v = T.row[e];
          if (dist[v] == INT32_MAX) { dist[v] = du; Q[tail++] = v; }
        }
      }
      for (int64_t r = 0; r < nrows; ++r) out[r + q * nrows] = dist[rows[r]];
    }
    free(dist);
    free(Q);
  }
  outedges_free(&T);
  return fail ? ORC_ARG : ORC_OK;
}

/* binary min-heap of (key << 32 | vertex); keys are the distance's order-preserving
   32-bit pattern (non-negative Int32, or the bits of a non-negative Float32) */
typedef struct { uint64_t* a; int64_t n, cap; } heap64;
static int heap_push(heap64* h, uint64_t x) {
  if (h->n == h->cap) {
    int64_t nc = h->cap ? h->cap * 2 : 1024;
    uint64_t* na = (uint64_t*)realloc(h->a, (size_t)nc * sizeof(uint64_t));
    if (!na) return 0;
    h->a = na;
    h->cap = nc;
  }
  int64_t i = h->n++;
  while (i > 0) {
    int64_t p = (i - 1) >> 1;
    if (h->a[p] <= x) break;
    h->a[i] = h->a[p];
    i = p;
  }
  h->a[i] = x;
  return 1;
}
static uint64_t heap_pop(heap64* h) {
  uint64_t top = h->a[0], x = h->a[--h->n];
  int64_t i = 0;
  for (;;) {
    int64_t c = 2 * i + 1;
    if (c >= h->n) break;
    if (c + 1 < h->n && h->a[c + 1] < h->a[c]) ++c;
    if (x <= h->a[c]) break;
    h->a[i] = h->a[c];
    i = c;
  }
  if (h->n > 0) h->a[i] = x;
  return top;
}

/*
 * shortest_path(A_T, source) of src/algorithms/shortest_path.jl:12-83 by Dijkstra.
 * The Jacobi rounds reach, for every row, the minimum over paths from the source of
 * the left fold safe_add(w_k, ... safe_add(w_1, 0)) in the distance type (Int32 for
 * Bool / Int32 values, Float32 for Float32 values, shortest_path.jl:18).  For
 * non-negative weights each step x -> fl(w + x) is non-decreasing in x and never
 * below x, so settling vertices in order of distance reaches the same minimum bit
 * for bit (Float32 included).  Negative or NaN weights return ORC_ARG, as do Int32
 * lengths beyond typemax (the reference would wrap).
 */
int orc_sssp_dijkstra(int64_t n, const int32_t* rowptr, const int32_t* colval,
                      const void* nzval, int tv, int64_t source, void* dist, int sym) {
  if (tv != T_BOOL && tv != T_I32 && tv != T_F32) return ORC_TYPE;
  const int64_t nnz = rowptr[n] - 1;
  for (int64_t i = 0; i < nnz; ++i) {
    if (tv == T_F32) {
      float w = ((const float*)nzval)[i];
      if (!(w >= 0.0f)) return ORC_ARG;
    } else if (tv == T_I32 && ((const int32_t*)nzval)[i] < 0) {
      return ORC_ARG;
    }
  }
  outedges T;
  if (outedges_build(n, rowptr, colval, nzval, tv, 1, 1, sym, &T) != ORC_OK) return ORC_ARG;
  float* df = tv == T_F32 ? (float*)dist : NULL;
  int32_t* di = tv == T_F32 ? NULL : (int32_t*)dist;
  for (int64_t v = 0; v < n; ++v) {
    if (df) df[v] = INFINITY;
    else di[v] = INT32_MAX;
  }
  heap64 h = {NULL, 0, 0};
  int rc = ORC_OK;
  if (df) df[source - 1] = 0.0f;
  else di[source - 1] = 0;
  if (!heap_push(&h, (uint64_t)(source - 1))) rc = ORC_ARG;
  while (rc == ORC_OK && h.n > 0) {
    uint64_t top = heap_pop(&h);
    const int32_t u = (int32_t)(top & 0xffffffffu);
    const uint32_t key = (uint32_t)(top >> 32);
    uint32_t cur;
    if (df) memcpy(&cur, &df[u], 4);
    else cur = (uint32_t)di[u];
    if (key != cur) continue; /* stale entry */
    for (int64_t e = T.ptr[u]; e < T.ptr[u + 1]; ++e) {
      const int32_t v = T.row[e];
      uint32_t nk;
      if (df) {
        volatile float s = T.wf[e] + df[u]; /* safe_add: +Inf stays +Inf */
        float nd = s;
        if (!(nd < df[v])) continue;
        df[v] = nd;
        memcpy(&nk, &nd, 4);
      } else {
        int64_t nd = (int64_t)T.wi[e] + (int64_t)di[u];
        if (nd >= INT32_MAX) { rc = ORC_ARG; break; }
        if (nd >= di[v]) continue;
        di[v] = (int32_t)nd;
        nk = (uint32_t)nd;
      }
      if (!heap_push(&h, ((uint64_t)nk << 32) | (uint32_t)v)) { rc = ORC_ARG; break; }
    }
  }
  free(h.a);
  outedges_free(&T);
  return rc;
}

/* ------------------------------------------------------------------------------ */
/* Fast typed paths timed as the CPU baseline (same algorithms, no interpreter).     */
/* ------------------------------------------------------------------------------ */

/* csr_spmv_kernel! with (GPUGraphs_mul, GPUGraphs_add, GPUGraphs_second) on Float32,
   src/spmv/CSR.jl:31-54, including the early exit when the sum reaches +Inf
   (monoid_absorb(Float32, GPUGraphs_add) == typemax, algebra.jl:45). */
void orc_csr_spmv_plus_times_f32(int64_t m, const int32_t* rowptr, const int32_t* colval,
                                 const float* nzval, const float* x, float* y) {
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t r = 0; r < m; ++r) {
    float acc = 0.0f;
    for (int64_t i = rowptr[r] - 1; i < rowptr[r + 1] - 1; ++i) {
      float p = nzval[i] * x[colval[i] - 1];
      acc = acc + p;
      if (acc == INFINITY) break;
    }
    y[r] = acc;
  }
}

/* Same loop over a row window [r0, r1) (0-based) -- bounded CPU samples. */
void orc_csr_spmv_plus_times_f32_rows(int64_t r0, int64_t r1, const int32_t* rowptr,
                                      const int32_t* colval, const float* nzval,
                                      const float* x, float* y) {
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t r = r0; r < r1; ++r) {
    float acc = 0.0f;
    for (int64_t i = rowptr[r] - 1; i < rowptr[r + 1] - 1; ++i) {
      float p = nzval[i] * x[colval[i] - 1];
      acc = acc + p;
      if (acc == INFINITY) break;
    }
    y[r] = acc;
  }
}

/* ------------------------------------------------------------------------------ */
/* SpMSpV: the operation of csc_spmspv_kernel! / gpu_spmspv! (src/spmspv.jl:1-54,   */
/* unfinished there) over the CSR storage of A, with the per-row loop of              */
/* src/spmv/CSR.jl:31-54 restricted to the columns that carry an entry of x.          */
/* x: 1-based strictly increasing x_ind[0..x_nnz), values x_val of type tx.           */
/* Rows with at least one such entry are written and listed in out_ind (1-based,      */
/* ascending); returns ORC_ARG for bad indices (nothing written).                     */
/* ------------------------------------------------------------------------------ */
int orc_csr_spmspv(int64_t m, int64_t n, const int32_t* rowptr, const int32_t* colval,
                   const void* nzval, int tv, void* y, int ty, const int32_t* x_ind,
                   const void* x_val, int tx, int64_t x_nnz, int mul, int add, int accum,
                   int32_t* out_ind, int64_t* out_nnz) {
  int tc;
  int rc = check_semiring(tv, tx, ty, mul, add, accum, &tc);
  if (rc) return rc;
  for (int64_t t = 0; t < x_nnz; ++t)
    if (x_ind[t] < 1 || x_ind[t] > n || (t > 0 && x_ind[t - 1] >= x_ind[t])) return ORC_ARG;
  int64_t* pos = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t j = 0; j < n; ++j) pos[j] = -1;
  for (int64_t t = 0; t < x_nnz; ++t) pos[x_ind[t] - 1] = t;
  val neutral, absorb;
  neutral_of(add, tc, &neutral);
  int has_absorb = absorb_of(add, tc, &absorb);
  int64_t cnt = 0;
  for (int64_t r = 1; r <= m; ++r) {
    val acc = neutral;
    int hit = 0;
    for (int64_t i = rowptr[r - 1]; i <= rowptr[r] - 1; ++i) {
      int64_t col = colval[i - 1];
      int64_t t = pos[col - 1];
      if (t < 0) continue;
      hit = 1;
      val b = load(x_val, tx, t);
      val a = cvt(load(nzval, tv, i - 1), tc);
      val mres = apply(mul, tc, a, cvt(b, tc), b, r, col, col, 1);
      acc = apply(add, tc, acc, mres, mres, r, col, col, 1);
      if (has_absorb && veq(acc, absorb)) break;
    }
    if (!hit) continue;
    val yo = load(y, ty, r - 1);
    val a2 = cvt(acc, ty);
    store(y, ty, r - 1, apply(accum, ty, yo, a2, a2, r, 1, r, 1));
    if (out_ind) out_ind[cnt] = (int32_t)r;
    ++cnt;
  }
  free(pos);
  if (out_nnz) *out_nnz = cnt;
  return ORC_OK;
}

/* ------------------------------------------------------------------------------ */
/* SpMV of listed rows: sparse_masked_csr_spmv_kernel! (src/spmv/CSR.jl:90-115),    */
/* whose mask holds 1-based row ids.  ORC_ARG for a row outside 1:m (other rows are  */
/* still written, in list order).                                                    */
/* ------------------------------------------------------------------------------ */
int orc_csr_spmv_rows(int64_t m, const int32_t* rowptr, const int32_t* colval,
                      const void* nzval, int tv, void* y, int ty, const void* x, int tx,
                      const int32_t* rows, int64_t nrows, int mul, int add, int accum) {
  int tc;
  int rc = check_semiring(tv, tx, ty, mul, add, accum, &tc);
  if (rc) return rc;
  val neutral, absorb;
  neutral_of(add, tc, &neutral);
  int has_absorb = absorb_of(add, tc, &absorb);
  int bad = 0;
  for (int64_t e = 0; e < nrows; ++e) {
    int64_t r = rows[e];
    if (r < 1 || r > m) {
      bad = 1;
      continue;
    }
    val acc = neutral;
    for (int64_t i = rowptr[r - 1]; i <= rowptr[r] - 1; ++i) {
      int64_t col = colval[i - 1];
      val b = load(x, tx, col - 1);
      val a = cvt(load(nzval, tv, i - 1), tc);
      val mres = apply(mul, tc, a, cvt(b, tc), b, r, col, col, 1);
      acc = apply(add, tc, acc, mres, mres, r, col, col, 1);
      if (has_absorb && veq(acc, absorb)) break;
    }
    val yo = load(y, ty, r - 1);
    val a2 = cvt(acc, ty);
    store(y, ty, r - 1, apply(accum, ty, yo, a2, a2, r, 1, r, 1));
  }
  return bad ? ORC_ARG : ORC_OK;
}

/* ------------------------------------------------------------------------------ */
/* Element-wise / apply / reduce with the operators of src/algebra.jl (the          */
/* reference's e_wise_ops.jl and map_and_reduce.jl are empty; its algorithms use    */
/* broadcasts, bfs.jl:60-70, shortest_path.jl:72-79).                               */
/* ------------------------------------------------------------------------------ */
static int ewise_type(int op, int ta, int tb, int tz, int* tc_out) {
  int tc = compute_type(ta, tb, op);
  int tp = ta > tb ? ta : tb;
  if (tz < tc || tz < tp) return ORC_TYPE;
  if (!is_index_op(op) && !op_defined(op, tc)) return ORC_UNSUPPORTED;
  *tc_out = tc;
  return ORC_OK;
}

/* z[i] = op(x[i], y[i], i, 1, i, 1) where mask[i] != 0 (or everywhere) */
int orc_ewise(int op, void* z, int tz, const void* x, int tx, const void* y, int ty, int64_t n,
              const void* mask, int tmask) {
  int tc;
  int rc = ewise_type(op, tx, ty, tz, &tc);
  if (rc) return rc;
  for (int64_t i = 0; i < n; ++i) {
    if (mask && is_zero(load(mask, tmask, i))) continue;
    val a = load(x, tx, i), b = load(y, ty, i);
    val v = apply(op, tc, cvt(a, tc), cvt(b, tc), b, i + 1, 1, i + 1, 1);
    store(z, tz, i, cvt(v, tz));
  }
  return ORC_OK;
}

/* z[i] = op(x[i], s) or op(s, x[i]); s is one value of type ts */
int orc_apply(int op, void* z, int tz, const void* x, int tx, const void* s, int ts,
              int s_first, int64_t n, const void* mask, int tmask) {
  int tc;
  int rc = s_first ? ewise_type(op, ts, tx, tz, &tc) : ewise_type(op, tx, ts, tz, &tc);
  if (rc) return rc;
  val sv = load(s, ts, 0);
  for (int64_t i = 0; i < n; ++i) {
    if (mask && is_zero(load(mask, tmask, i))) continue;
    val a = load(x, tx, i);
    val v = s_first ? apply(op, tc, cvt(sv, tc), cvt(a, tc), a, i + 1, 1, i + 1, 1)
                    : apply(op, tc, cvt(a, tc), cvt(sv, tc), sv, i + 1, 1, i + 1, 1);
    store(z, tz, i, cvt(v, tz));
  }
  return ORC_OK;
}

/* One chunk of up to 8192 values in the library's order: 256 threads fold values t,
   t + 256, ... left to right; each warp's 32 lanes combine by xor butterfly (lane l
   takes add(v[l], v[l ^ o]), o = 16, 8, 4, 2, 1); lane 0 of warp 0 then combines the 8
   warp totals (lanes 8..31 neutral) the same way. */
static val reduce_chunk(int add, int t, const void* x, int tx, int64_t c0, int64_t n, val neutral) {
  val th[256], w[32], tot[8];
  for (int k = 0; k < 256; ++k) {
    val acc = neutral;
    for (int u = 0; u < 32; ++u) {
      int64_t i = c0 + k + (int64_t)u * 256;
      if (i < n) {
        val v = cvt(load(x, tx, i), t);
        acc = apply(add, t, acc, v, v, 0, 0, 0, 0);
      }
    }
    th[k] = acc;
  }
  for (int wid = 0; wid < 8; ++wid) {
    for (int l = 0; l < 32; ++l) w[l] = th[wid * 32 + l];
    for (int o = 16; o > 0; o >>= 1) {
      val nw[32];
      for (int l = 0; l < 32; ++l) nw[l] = apply(add, t, w[l], w[l ^ o], w[l ^ o], 0, 0, 0, 0);
      memcpy(w, nw, sizeof(w));
    }
    tot[wid] = w[0];
  }
  for (int l = 0; l < 32; ++l) w[l] = l < 8 ? tot[l] : neutral;
  for (int o = 16; o > 0; o >>= 1) {
    val nw[32];
    for (int l = 0; l < 32; ++l) nw[l] = apply(add, t, w[l], w[l ^ o], w[l ^ o], 0, 0, 0, 0);
    memcpy(w, nw, sizeof(w));
  }
  return w[0];
}

/* *out = add over x[0..n) from the neutral element, in the library's fixed order:
   chunks of 8192, chunk totals reduced again until one value is left. */
int orc_reduce(int add, const void* x, int tx, int64_t n, void* out) {
  int tc;
  int rc = check_semiring(tx, tx, tx, OP_FIRST, add, OP_SECOND, &tc);
  if (rc) return rc;
  val neutral;
  neutral_of(add, tx, &neutral);
  if (n == 0) {
    store(out, tx, 0, neutral);
    return ORC_OK;
  }
  size_t esz = (tx == T_BOOL) ? 1 : (tx == T_I32 || tx == T_F32) ? 4 : 8;
  int64_t cnt = n;
  const void* in = x;
  void* buf = NULL;
  for (;;) {
    int64_t chunks = (cnt + 8191) / 8192;
    void* nb = malloc((size_t)chunks * esz);
    for (int64_t c = 0; c < chunks; ++c)
      store(nb, tx, c, reduce_chunk(add, tx, in, tx, c * 8192, cnt, neutral));
    free(buf);
    buf = nb;
    in = buf;
    cnt = chunks;
    if (cnt == 1) break;
  }
  store(out, tx, 0, load(buf, tx, 0));
  free(buf);
  return ORC_OK;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}
