// gg_common.cuh -- shared definitions of libgpugraphs: handles, error reporting,
// element types and the device-side semantics of the GPUGraphs.jl operators
// (src/algebra.jl), evaluated exactly as Julia does: Int32/Int64 wrap around,
// Float32 operations round once each (no FMA contraction), min/max propagate NaN
// and order -0.0 below +0.0, Bool is a 0/1 byte.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gpugraphs.h"

// ---------------------------------------------------------------------------------
// error reporting (thread-local message behind gg_last_error)
// ---------------------------------------------------------------------------------
namespace gg {

int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

#define GG_CUDA(call)                                   \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return gg::cuda_error(_e, #call); \
  } while (0)

#define GG_CHECK(call)           \
  do {                           \
    int _rc = (call);            \
    if (_rc != GG_OK) return _rc; \
  } while (0)

// ---------------------------------------------------------------------------------
// element types
// ---------------------------------------------------------------------------------
template <int TC> struct CType;
template <> struct CType<GG_BOOL> { typedef uint8_t T; };
template <> struct CType<GG_INT32> { typedef int32_t T; };
template <> struct CType<GG_INT64> { typedef int64_t T; };
template <> struct CType<GG_FLOAT32> { typedef float T; };
template <> struct CType<GG_FLOAT64> { typedef double T; };

inline int dtype_size(int t) {
  switch (t) {
    case GG_BOOL: return 1;
    case GG_INT32: return 4;
    case GG_FLOAT32: return 4;
    case GG_INT64: return 8;
    case GG_FLOAT64: return 8;
  }
  return 0;
}
inline bool dtype_valid(int t) { return t >= GG_BOOL && t <= GG_FLOAT64; }
__host__ __device__ inline bool dtype_is_float(int t) { return t == GG_FLOAT32 || t == GG_FLOAT64; }

// A value read in its own element type: integers (and Bool) in i, floats in d
// (every Float32 is exact in a double).
struct Raw {
  int64_t i;
  double d;
};

__device__ __forceinline__ Raw load_raw(const void* p, int t, int64_t k) {
  Raw r;
  r.i = 0;
  r.d = 0.0;
  switch (t) {
    case GG_BOOL: r.i = static_cast<const uint8_t*>(p)[k] != 0; break;
    case GG_INT32: r.i = static_cast<const int32_t*>(p)[k]; break;
    case GG_INT64: r.i = static_cast<const int64_t*>(p)[k]; break;
    case GG_FLOAT32: r.d = static_cast<const float*>(p)[k]; break;
    default: r.d = static_cast<const double*>(p)[k]; break;
  }
  return r;
}

__device__ __forceinline__ bool raw_is_zero(const Raw& r, int t) {
  return dtype_is_float(t) ? (r.d == 0.0) : (r.i == 0);
}

// Julia convert from a raw value of type t into compute type TC.
template <int TC>
__device__ __forceinline__ typename CType<TC>::T raw_to(const Raw& r, int t) {
  typedef typename CType<TC>::T T;
  if (!dtype_is_float(t)) {
    if (TC == GG_BOOL) return static_cast<T>(r.i != 0);
    if (TC == GG_INT32) return static_cast<T>(static_cast<int32_t>(static_cast<uint32_t>(r.i)));
    return static_cast<T>(r.i);
  }
  if (TC == GG_FLOAT32) return static_cast<T>(static_cast<float>(r.d));
  if (TC == GG_BOOL) return static_cast<T>(r.d != 0.0);
  return static_cast<T>(r.d);
}

// Store v (compute type TC) into an array of element type t.  Float -> integer
// conversion truncates (Julia would throw InexactError for non-integral values).
template <int TC>
__device__ __forceinline__ void store_as(void* p, int t, int64_t k, typename CType<TC>::T v) {
  switch (t) {
    case GG_BOOL: static_cast<uint8_t*>(p)[k] = (v != 0) ? 1 : 0; break;
    case GG_INT32:
      static_cast<int32_t*>(p)[k] =
          dtype_is_float(TC) ? static_cast<int32_t>(v)
                             : static_cast<int32_t>(static_cast<uint32_t>(static_cast<int64_t>(v)));
      break;
    case GG_INT64: static_cast<int64_t*>(p)[k] = static_cast<int64_t>(v); break;
    case GG_FLOAT32: static_cast<float*>(p)[k] = static_cast<float>(v); break;
    default: static_cast<double*>(p)[k] = static_cast<double>(v); break;
  }
}

// ---------------------------------------------------------------------------------
// scalar semantics of src/algebra.jl
// ---------------------------------------------------------------------------------
template <typename T> struct Lim;
template <> struct Lim<uint8_t> {
  __host__ __device__ static uint8_t max() { return 1; }
  __host__ __device__ static uint8_t min() { return 0; }
};
template <> struct Lim<int32_t> {
  __host__ __device__ static int32_t max() { return INT32_MAX; }
  __host__ __device__ static int32_t min() { return INT32_MIN; }
};
template <> struct Lim<int64_t> {
  __host__ __device__ static int64_t max() { return INT64_MAX; }
  __host__ __device__ static int64_t min() { return INT64_MIN; }
};
template <> struct Lim<float> {
  __host__ __device__ static float max() { return __builtin_huge_valf(); }
  __host__ __device__ static float min() { return -__builtin_huge_valf(); }
};
template <> struct Lim<double> {
  __host__ __device__ static double max() { return __builtin_huge_val(); }
  __host__ __device__ static double min() { return -__builtin_huge_val(); }
};

// Julia max / min (base/math.jl): NaN if either is NaN, -0.0 < +0.0
template <typename T> __device__ __forceinline__ T jl_max(T x, T y) { return x > y ? x : y; }
template <typename T> __device__ __forceinline__ T jl_min(T x, T y) { return x < y ? x : y; }
template <> __device__ __forceinline__ float jl_max<float>(float x, float y) {
  if (x != x || y != y) return __int_as_float(0x7fc00000);
  if (x == y) return signbit(x) ? y : x;
  return x > y ? x : y;
}
template <> __device__ __forceinline__ float jl_min<float>(float x, float y) {
  if (x != x || y != y) return __int_as_float(0x7fc00000);
  if (x == y) return signbit(x) ? x : y;
  return x < y ? x : y;
}
template <> __device__ __forceinline__ double jl_max<double>(double x, double y) {
  if (x != x || y != y) return __longlong_as_double(0x7ff8000000000000LL);
  if (x == y) return signbit(x) ? y : x;
  return x > y ? x : y;
}
template <> __device__ __forceinline__ double jl_min<double>(double x, double y) {
  if (x != x || y != y) return __longlong_as_double(0x7ff8000000000000LL);
  if (x == y) return signbit(x) ? x : y;
  return x < y ? x : y;
}

// wrapping integer arithmetic; floats round once per operation
__device__ __forceinline__ uint8_t w_add(uint8_t x, uint8_t y) { return (x + y) & 1; }
__device__ __forceinline__ int32_t w_add(int32_t x, int32_t y) {
  return static_cast<int32_t>(static_cast<uint32_t>(x) + static_cast<uint32_t>(y));
}
__device__ __forceinline__ int64_t w_add(int64_t x, int64_t y) {
  return static_cast<int64_t>(static_cast<uint64_t>(x) + static_cast<uint64_t>(y));
}
__device__ __forceinline__ float w_add(float x, float y) { return __fadd_rn(x, y); }
__device__ __forceinline__ double w_add(double x, double y) { return __dadd_rn(x, y); }

__device__ __forceinline__ uint8_t w_sub(uint8_t x, uint8_t y) { return (x - y) & 1; }
__device__ __forceinline__ int32_t w_sub(int32_t x, int32_t y) {
  return static_cast<int32_t>(static_cast<uint32_t>(x) - static_cast<uint32_t>(y));
}
__device__ __forceinline__ int64_t w_sub(int64_t x, int64_t y) {
  return static_cast<int64_t>(static_cast<uint64_t>(x) - static_cast<uint64_t>(y));
}
__device__ __forceinline__ float w_sub(float x, float y) { return __fsub_rn(x, y); }
__device__ __forceinline__ double w_sub(double x, double y) { return __dsub_rn(x, y); }

__device__ __forceinline__ uint8_t w_mul(uint8_t x, uint8_t y) { return x & y; }
__device__ __forceinline__ int32_t w_mul(int32_t x, int32_t y) {
  return static_cast<int32_t>(static_cast<uint32_t>(x) * static_cast<uint32_t>(y));
}
__device__ __forceinline__ int64_t w_mul(int64_t x, int64_t y) {
  return static_cast<int64_t>(static_cast<uint64_t>(x) * static_cast<uint64_t>(y));
}
__device__ __forceinline__ float w_mul(float x, float y) { return __fmul_rn(x, y); }
__device__ __forceinline__ double w_mul(double x, double y) { return __dmul_rn(x, y); }

template <typename T> __device__ __forceinline__ T bit_or(T x, T y) { return x | y; }
template <typename T> __device__ __forceinline__ T bit_and(T x, T y) { return x & y; }
template <typename T> __device__ __forceinline__ T bit_xor(T x, T y) { return x ^ y; }
template <> __device__ __forceinline__ float bit_or<float>(float x, float) { return x; }
template <> __device__ __forceinline__ float bit_and<float>(float x, float) { return x; }
template <> __device__ __forceinline__ float bit_xor<float>(float x, float) { return x; }
template <> __device__ __forceinline__ double bit_or<double>(double x, double) { return x; }
template <> __device__ __forceinline__ double bit_and<double>(double x, double) { return x; }
template <> __device__ __forceinline__ double bit_xor<double>(double x, double) { return x; }

// GPUGraphs_safe_add (src/algebra.jl:47-48) in one type
template <typename T> __device__ __forceinline__ T safe_add(T x, T y) {
  T mx = jl_max<T>(x, y);
  if (mx == Lim<T>::max()) return Lim<T>::max();
  return w_add(x, y);
}

// Evaluate operator `op` on (x, y) already in compute type TC.  Index operators
// receive the row / column ids of the reference kernels: A_i = row (Int64), A_j =
// column of A (Int32), B_i = column of A (Int32), B_j = column of B (Int64).
// For GPUGraphs_secondi the product B_i * y is taken in promote_type(Int32, typeof(y))
// before conversion, so it needs the raw y and its type.
template <int TC>
__device__ __forceinline__ typename CType<TC>::T apply_op(int op, typename CType<TC>::T x,
                                                          typename CType<TC>::T y, const Raw& yraw,
                                                          int ty_raw, int64_t ai, int64_t aj,
                                                          int64_t bi, int64_t bj) {
  typedef typename CType<TC>::T T;
  switch (op) {
    case GG_OP_FIRST: return x;
    case GG_OP_SECOND: return y;
    case GG_OP_ANY: return jl_max<T>(x, y);
    case GG_OP_PAIR: return (y != T(0)) ? T(1) : T(0);
    case GG_OP_ADD: return w_add(x, y);
    case GG_OP_SAFE_ADD: return safe_add<T>(x, y);
    case GG_OP_MINUS: return w_sub(x, y);
    case GG_OP_RMINUS: return w_sub(y, x);
    case GG_OP_MUL: return w_mul(x, y);
    case GG_OP_MIN: return jl_min<T>(x, y);
    case GG_OP_MAX: return jl_max<T>(x, y);
    case GG_OP_LOR:
    case GG_OP_BOR: return bit_or<T>(x, y);
    case GG_OP_LAND:
    case GG_OP_BAND: return bit_and<T>(x, y);
    case GG_OP_BXOR: return bit_xor<T>(x, y);
    case GG_OP_FIRSTI: { Raw r; r.i = ai; r.d = 0; return raw_to<TC>(r, GG_INT64); }
    case GG_OP_FIRSTJ: { Raw r; r.i = aj; r.d = 0; return raw_to<TC>(r, GG_INT32); }
    case GG_OP_SECONDJ: { Raw r; r.i = bj; r.d = 0; return raw_to<TC>(r, GG_INT64); }
    case GG_OP_SECONDI: {
      Raw p;
      p.i = 0;
      p.d = 0;
      if (ty_raw == GG_FLOAT32) {
        p.d = __fmul_rn(static_cast<float>(static_cast<int32_t>(bi)), static_cast<float>(yraw.d));
        return raw_to<TC>(p, GG_FLOAT32);
      }
      if (ty_raw == GG_FLOAT64) {
        p.d = __dmul_rn(static_cast<double>(static_cast<int32_t>(bi)), yraw.d);
        return raw_to<TC>(p, GG_FLOAT64);
      }
      if (ty_raw == GG_INT64) {
        p.i = w_mul(static_cast<int64_t>(static_cast<int32_t>(bi)), yraw.i);
        return raw_to<TC>(p, GG_INT64);
      }
      p.i = w_mul(static_cast<int32_t>(bi), static_cast<int32_t>(yraw.i));
      return raw_to<TC>(p, GG_INT32);
    }
  }
  return x;
}

// monoid_neutral / monoid_absorb (src/algebra.jl:10-100) for the add operator
template <typename T> __host__ __device__ inline T all_ones() { return static_cast<T>(-1); }
template <> __host__ __device__ inline uint8_t all_ones<uint8_t>() { return 1; }

template <typename T> __host__ __device__ inline T neutral_of(int add) {
  switch (add) {
    case GG_OP_MUL: return T(1);
    case GG_OP_MIN: return Lim<T>::max();
    case GG_OP_MAX: return Lim<T>::min();
    case GG_OP_BAND:
    case GG_OP_LAND: return all_ones<T>();
    default: return T(0);  // add, safe_add, any, bor, lor
  }
}

// returns false when the monoid has no absorbing value (GPUGraphs_any)
template <typename T> __host__ __device__ inline bool absorb_of(int add, T* out) {
  switch (add) {
    case GG_OP_ADD:
    case GG_OP_SAFE_ADD:
    case GG_OP_MAX: *out = Lim<T>::max(); return true;
    case GG_OP_MUL: *out = T(0); return true;
    case GG_OP_MIN: *out = Lim<T>::min(); return true;
    case GG_OP_BOR:
    case GG_OP_LOR: *out = all_ones<T>(); return true;
    case GG_OP_BAND:
    case GG_OP_LAND: *out = T(0); return true;
  }
  return false;
}

// warp shuffle that also handles the one-byte Bool type
template <typename T> __device__ __forceinline__ T shfl_xor(T v, int off, int width) {
  return __shfl_xor_sync(0xffffffffu, v, off, width);
}
template <> __device__ __forceinline__ uint8_t shfl_xor<uint8_t>(uint8_t v, int off, int width) {
  return static_cast<uint8_t>(__shfl_xor_sync(0xffffffffu, static_cast<int>(v), off, width));
}

// ---------------------------------------------------------------------------------
// handles
// ---------------------------------------------------------------------------------

// Row-block partition of a CSR matrix for the SpMV / SpMM row-block kernels.
// Regular blocks: contiguous short rows (at most kShortRow entries each) [first,
// last) holding at most kBlockNnz stored entries and kBlockRows rows.  Longer rows
// are handled one warp per segment; rows of more than kSegNnz entries are cut into
// segments of kSegNnz entries; the warp that finishes a row's last segment combines
// the partials in segment order.
struct RowBlocks {
  int64_t nblocks = 0;      // regular blocks
  int64_t nsegs = 0;        // long-row segments
  int64_t nlong = 0;        // long rows
  int4* blocks = nullptr;   // [nblocks] (first row, end row, first entry, end entry) 0-based
  int4* segs = nullptr;     // [nsegs] (row, k_begin, k_end, long-row index) 0-based
  int32_t* long_first_seg = nullptr;  // [nlong + 1] first segment of each long row
  int32_t* long_rows = nullptr;       // [nlong] row id
  unsigned int* long_count = nullptr; // [nlong] arrival counters (self-resetting)
  void* partials = nullptr;           // [nsegs * partial_stride] bytes
  int64_t partial_bytes = 0;
};

struct GraphAux;  // graph-algorithm analysis (gg_graph.cu)
struct SpvPlan;   // column index and workspace of SpMSpV (gg_spmspv.cu)

// Work list of a SELL matrix: slices cut into chunks of at most kSellChunk stored
// columns.  items: (slice, first column, end column, partial index or -1 when the
// slice is a single chunk); multi: (slice, first partial index, number of chunks).
struct SellPlan {
  int64_t nitems = 0, nmulti = 0;
  int4* items = nullptr;
  int4* multi = nullptr;
  void* partials = nullptr;  // [npartials * C] accumulators (8 bytes each)
  // work items of the SELL-32 warp kernel: a chunk of a slice wider than
  // kNarrowCols as (first entry position, first stored row, columns, partial index
  // or -1), or a group of up to 8 consecutive narrow slices holding at most
  // kNarrowCols columns in total as (first entry position, first stored row,
  // -(slices), widths packed 4 bits per slice)
  int4* pitems = nullptr;
  int64_t npitems = 0;
  // the chunked slices (multi) split by width for the plus-times Float32 combine:
  // at most kNarrowChunks chunks (a thread per row) and wider (a warp per row)
  int4* narrow = nullptr;
  int4* wide = nullptr;
  int64_t nnarrow = 0, nwide = 0;
  // the same warp items with chunks of kSegMM columns (the pieces of the SpMM fold)
  // for the one-column plus-times SpMM; multi256: (first stored row, first partial,
  // chunks) of the slices cut into several chunks; built on first use
  int4* pitems256 = nullptr;
  int4* multi256 = nullptr;
  int64_t npitems256 = -1, nmulti256 = 0, npart256 = 0;
};
static const int kNarrowChunks = 8;
static const int kNarrowCols = 8;
static const int kSellChunk = 128;

// SpMM long-row segments.  Rows (CSR) or slices (SELL) longer than kSegMM entries
// are cut into pieces of kSegMM; one warp folds one piece for all dense columns into
// partials[slot * k + j] and a second pass folds a row's pieces in order.
// segs: (row, first entry, end entry, slot) for CSR -- entries 0-based positions in
// colval; (stored row, first slice column, end slice column, slot) for SELL.
// first[li] .. first[li + 1] are the slots of long row li = rows[li].
struct MMPlan {
  int64_t nseg = 0, nlong = 0;
  int4* segs = nullptr;
  int32_t* first = nullptr;
  int32_t* rows = nullptr;
  // CSR: the work of the Float32 item kernel -- every piece (as in segs) and every row
  // of 33..kSegMM entries as (row, first entry, end entry, -1), longest first
  int4* items = nullptr;
  int64_t nitems = 0;
  // CSR: the rows of at most 32 entries (the short-row kernel's), longest first, so
  // the four rows a warp takes have about the same length
  int32_t* short_rows = nullptr;
  int64_t nshort = 0;
};
static const int kSegMM = 256;

// Hub vertices of a graph's CSR view for the batched searches: rows longer than
// kHubDegB entries, cut into pieces of kHubPieceB entries (0-based positions in
// colval).  pieces: (hub index, first entry, end entry, 0); hubs: vertex (0-based).
struct HubPlan {
  int64_t nhub = 0, npiece = 0;
  int32_t* hubs = nullptr;
  int4* pieces = nullptr;
  void* acc = nullptr;  // per-hub accumulators of the batched BFS (8 words per hub)
  // rows of 33..kHubDegB entries (0-based), longest first: a warp each in pull rounds
  int32_t* mid = nullptr;
  int64_t nmid = 0;
  // every non-hub row, the mid rows first (longest first), then the others ascending:
  // the visiting order of full batched rounds (round-robin over warps balances them)
  int32_t* order = nullptr;
  unsigned long long* d_norder = nullptr;  // device copy of the order's length
  int64_t norder = 0;
};
static const int kHubDegB = 2048;
static const int kHubPieceB = 2048;

// Frequency-ordered column labels for the plus-times SpMV kernels: relabelling the
// columns of A by decreasing number of stored entries puts the most-gathered part of
// x in a few contiguous cache lines, so L1 keeps it.  colval_r mirrors the matrix's
// colval (same positions; -1 padding kept for SELL) with new 1-based labels; inv maps
// a new label (0-based) to the original column; xr holds x in the new order.
struct ColPerm {
  bool enabled = false;
  int32_t* colval_r = nullptr;
  int32_t* inv = nullptr;
  float* xr = nullptr;
};

// Column-window tiles of a large CSR for the plus-times Float32 SpMV (gg_spmv_win.cu).
// Rows sorted by length (longest first) are cut into tiles (at most kTileRows rows,
// fewer where the rows are long); columns are relabelled by decreasing frequency
// (rank).  Every row of a tile is one or more pieces (long rows are cut so the 32
// warps of a CTA get even shares); each piece belongs to one warp.  A tile's entries
// inside the tile's staged windows (kWinCols consecutive ranks, whose x values the CTA
// copies into shared memory with a bulk copy) are grouped per warp, then per window,
// then by (piece, original column); an entry is one word (piece << 19 | rank offset
// inside its window) plus its value.  The other entries form a tail CSR.
// Work units are segment ranges of one tile, balanced over the CTAs; a tile split
// into several units leaves one partial row vector per unit (combined in unit order).
struct WinTile {
  int32_t row0, rows;  // sorted row range
  int32_t nv;          // pieces (accumulator slots)
  int32_t nseg;        // segments
  int32_t seg0;        // first word of the tile's segment bases in segbase[]
  int32_t wbase;       // first word of the tile's [32][nseg + 1] entry offsets in wseg[]
  int32_t vbase;       // first word of the tile's rows + 1 piece offsets in vptr[]
  int32_t pad;
};
struct WinPlan {
  bool enabled = false;
  int64_t ntiles = 0, nseg = 0, nunits = 0, nslots = 0, nsplit = 0, nwin = 0, npieces = 0;
  int grid = 0;
  int32_t* rowperm = nullptr;  // sorted position -> original row (0-based)
  int32_t* inv = nullptr;      // rank -> original column (0-based)
  float* xr = nullptr;         // x in rank order, padded to whole windows
  uint32_t* idx = nullptr;
  float* val = nullptr;
  WinTile* tiles = nullptr;
  int32_t* segbase = nullptr;  // first rank of every segment | kSegWindow for windows
  int32_t* wseg = nullptr;     // entry offsets per (tile, warp, segment)
  int32_t* vptr = nullptr;     // per tile: first piece of every row (rows + 1 words)
  int4* units = nullptr;       // (tile, first segment, end segment, slot), grouped by CTA
  int32_t* cta_ptr = nullptr;  // grid + 1
  int32_t* cta_wptr = nullptr; // grid + 1: each CTA's windows in cta_win
  int32_t* cta_win = nullptr;  // first rank of every window a CTA stages, in order
  int4* split = nullptr;       // (tile, first slot, slots, rows)
  float* partials = nullptr;   // nslots * kWinRows
  // entries outside every staged window: a CSR over the sorted rows with rank labels
  // (row-block kernel), its row sums yt (sorted order) added at the end
  gg_mat* tail = nullptr;
  float* yt = nullptr;
};
static const int kWinRows = 8192;   // pieces per tile (13 bits of the entry word)
static const int kTileRows = 6144;  // rows per tile
static const int kWinCols = 16384;
static const int kWinShift = 19;
static const int32_t kSegWindow = 1 << 30;

// Hub rows of a sorted SELL-32 copy folded from shared-memory column windows
// (gg_spmv_hub.cu).  The first np stored rows (the longest, all above kSellChunk
// entries) are cut into groups of at most pg rows; row i of a group is accumulator
// slot i and belongs to warp i mod 32 of the CTA that runs the group.  Columns are
// the frequency ranks of ColPerm, cut into windows of kHwCols ranks whose x values a
// CTA stages in shared memory with bulk copies.  For every (group, warp, window) the
// warp's rows with entries in that window form SELL-32 slices (lane = row, rows
// sorted by their entry count in the window, padded with the zero slot kHwCols),
// entries in storage order: col = rank - window * kHwCols (16 bits), val, and a
// 16-bit accumulator slot per slice lane (0xffff = no row).  items: (first entry,
// first slice lane, width | -(slices), widths packed 4 bits per slice) per warp in
// (group, warp, window) order; itemptr[(group * 32 + warp) * nwin + w] is the first
// item of window w.  A unit (group and group-warp range, first window, end window,
// partial slot) is run by one CTA; a row's value is its slots' partials added in
// window order.
struct HubWinPlan {
  bool enabled = false;
  int64_t np = 0, nwin = 0, nunits = 0, nitems = 0, nslices = 0, nentries = 0;
  int pg = 0, ngroups = 0;
  uint16_t* col = nullptr;
  float* val = nullptr;
  uint16_t* rowid = nullptr;
  int4* items = nullptr;
  int32_t* itemptr = nullptr;
  int4* units = nullptr;         // grouped by CTA: CTA b runs units[cptr[b] .. cptr[b + 1])
  int32_t* cptr = nullptr;
  int grid = 0;
  int32_t* gptr = nullptr;       // partial slots of group g: gptr[g] .. gptr[g + 1] - 1
  float* partials = nullptr;     // nunits x pg
  SellPlan* rest = nullptr;      // SELL-32 work items of the stored rows >= np
};
static const int kHwCols = 8192;

static const int kBlockNnz = 256;
static const int kShortRow = 32;
static const int kBlockRows = 256;
static const int kSegNnz = 4096;

}  // namespace gg

struct gg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  // scratch arena, grown on demand, freed by gg_destroy
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  unsigned int* d_flags = nullptr;  // small device word array for status flags
  unsigned int* h_flags = nullptr;  // pinned mirror
  unsigned int* d_err = nullptr;    // set by kernels whose bounded waits ran out
  unsigned long long wait_polls = 0;  // gg_set_wait_limit; 0 = the built-in limits
  // launch tracing (gg_trace_begin / gg_trace_end): kernel launches of the SpMV /
  // SpMM paths are counted and their main kernel bracketed by events from a pool
  bool trace_on = false;
  int64_t trace_launches = 0;
  int trace_used = 0;
  cudaEvent_t* trace_ev = nullptr;  // 2 * kTraceMax events
};

namespace gg {
// poll limits of the bounded device-side waits: grid barriers of the persistent
// kernels (each poll sleeps ~100 ns) and bulk-copy completions of the staged SpMV
// kernels (mbarrier try_wait polls); gg_set_wait_limit replaces both
static const unsigned kBarrierPolls = 1u << 26;
static const unsigned kCopyPolls = 1u << 22;
inline unsigned barrier_polls(const gg_ctx* c) {
  return c->wait_polls ? (unsigned)(c->wait_polls < 0xffffffffull ? c->wait_polls : 0xffffffffull)
                       : kBarrierPolls;
}
inline unsigned copy_polls(const gg_ctx* c) {
  return c->wait_polls ? (unsigned)(c->wait_polls < 0xffffffffull ? c->wait_polls : 0xffffffffull)
                       : kCopyPolls;
}
static const int kTraceMax = 4096;
// count n kernel launches of the current call
inline void trace_count(gg_ctx* c, int n) {
  if (c->trace_on) c->trace_launches += n;
}
// bracket the main kernel of a call: returns the event pair index or -1
inline int trace_main_begin(gg_ctx* c) {
  if (!c->trace_on || c->trace_used >= kTraceMax) return -1;
  const int i = c->trace_used++;
  cudaEventRecord(c->trace_ev[2 * i], c->stream);
  return i;
}
inline void trace_main_end(gg_ctx* c, int i) {
  if (i >= 0) cudaEventRecord(c->trace_ev[2 * i + 1], c->stream);
}
}  // namespace gg

struct gg_mat {
  int format = GG_FMT_CSR;
  int64_t m = 0, n = 0, nnz = 0;
  int dtype = GG_FLOAT32;
  int device = 0;
  // CSR (1-based)
  int32_t* rowptr = nullptr;
  int32_t* colval = nullptr;
  void* nzval = nullptr;
  // SELL (1-based slice_ptr / perm; colval -1 padded)
  int64_t slice_size = 0, nslices = 0, n_stored = 0, sigma = 1;
  int32_t* slice_ptr = nullptr;
  int32_t* perm = nullptr;   // stored row -> original row (1-based)
  int32_t* iperm = nullptr;  // original row (0-based) -> stored row (0-based)
  // lazily built analysis
  gg::RowBlocks* blocks = nullptr;
  gg::GraphAux* aux = nullptr;
  gg::SellPlan* sellplan = nullptr;
  gg::ColPerm* colperm = nullptr;
  gg::MMPlan* mmplan = nullptr;
  gg::HubPlan* hubplan = nullptr;
  gg::WinPlan* winplan = nullptr;
  gg::HubWinPlan* hubwin = nullptr;  // SELL-32 copies: hub rows from column windows
  gg::SpvPlan* spv = nullptr;
  gg_mat* sell_copy = nullptr;  // CSR handles: SELL-32 copy (rows sorted by length) for plus-times
  gg_mat* tr_copy = nullptr;    // CSR handles: CSR storage of the transpose (gg_spmv_t)
  int64_t max_row_len = -1;
  // tuned choices (gg_tune): plus-times SpMV kernel (0 = built-in rule, 1 = CSR row
  // blocks, 2 = the SELL copy, 3 = column-window tiles), rows per row block, SpMM
  // columns per lane (0 = 1)
  int tuned_spmv = 0;
  int block_rows = 0;
  int mm_cpl = 0;
  // SELL-32 plus-times kernel: 0 = register loads (k_sell_hot32), 1 = matrix stream
  // staged by bulk copies (k_sell_tma32), 2 = register loads with the hub rows folded
  // from shared-memory column windows where the hub groups are dense enough
  // (gg_spmv_hub.cu)
  int sell_variant = 0;
  int hot_cols = 0;  // x values staged in shared memory by the register kernels (0: 32768)
  int last_layout = 0;  // layout of the last plus-times Float32 SpMV (gg_spmv_layout)
};

namespace gg {
int ensure_scratch(gg_ctx* ctx, size_t bytes);
void free_graph_aux(gg_mat* A);
int compute_type(int tv, int tx, int mul);
int check_semiring(int tv, int tx, int ty, int mul, int add, int accum, int* tc_out);
int spmv_dispatch(gg_ctx* ctx, gg_mat* A, int tc, int mul, int add, int accum, void* y, int ty,
                  const void* x, int tx, const void* mask, int tmask, int64_t lo, int64_t hi);
int build_row_blocks(gg_ctx* ctx, gg_mat* A);
int build_sell_plan(gg_ctx* ctx, gg_mat* A);
int launch_col1_sell(gg_ctx* ctx, gg_mat* A, const float* x, float* y);  // gg_spmv.cu
int build_hub_plan(gg_ctx* ctx, gg_mat* A, const int32_t* rowptr, int64_t n);  // gg_batch.cu
int launch_sell_tma(gg_ctx* ctx, gg_mat* A, const float* nzv, const float* xr, float* y,
                    const int32_t* colval);  // gg_spmv_tma.cu
int launch_pipe_f32(gg_ctx* ctx, gg_mat* A, const float* nz, const float* x, float* y,
                    const int32_t* colval, bool trace_main);  // gg_spmv.cu
int build_win_plan(gg_ctx* ctx, gg_mat* A);  // gg_spmv_win.cu
int launch_spmv_win(gg_ctx* ctx, gg_mat* A, const float* x, float* y);
int build_sell_plan_from(gg_ctx* ctx, const gg_mat* A, int64_t s0, SellPlan** out);  // gg_spmv.cu
void free_sell_plan(SellPlan* P);
int build_hubwin_plan(gg_ctx* ctx, gg_mat* S);  // gg_spmv_hub.cu
int launch_hubwin(gg_ctx* ctx, gg_mat* S, const float* xr, float* y);
void free_hubwin_plan(gg_mat* A);
void free_win_plan(gg_mat* A);
void free_spv_plan(gg_mat* A);  // gg_spmspv.cu
// out[0..n] = base + exclusive prefix sums of cnt (gg_graph.cu; synchronises the stream)
int scan_counts(gg_ctx* ctx, const int32_t* cnt, int64_t n, int32_t* out, int32_t base);
int row_stats(gg_ctx* ctx, gg_mat* A);
}  // namespace gg
