// gg_spmm.cu -- semiring SpMM over CSR and SELL (gpu_spmm!, src/spmm/CSR.jl and
// src/spmm/SELL.jl of GPUGraphs.jl).
//
// One warp per row; lane j owns output column j (32 columns per pass).  The warp
// loads 32 (column, value) pairs of the row with one coalesced access each, then
// broadcasts them by shuffle; every lane folds its (row, j) sequentially in storage
// order -- the order of csr_spmm_kernel! (src/spmm/CSR.jl:3-35), so results equal
// the reference's bit for bit, including its early exit on the absorbing value.
// Rows longer than kSegMM entries (hubs of power-law graphs) are cut into pieces
// folded by separate warps and combined in order by a second pass: exact for every
// associative monoid, within rounding for Float32/Float64 sums.
// With a row-major dense operand (the batched-query layout) each gathered B row is
// one contiguous 128-byte read.
#include <algorithm>
#include <vector>

#include "gg_semiring.cuh"

namespace gg {

static const unsigned kFullMM = 0xffffffffu;

// (mul, add, second) on Float32 with row-major B / C
struct SRPlusTimesF32MM {
  typedef float T;
  const float* __restrict__ nz;
  const float* __restrict__ x;
  float* __restrict__ y;
  int64_t ldb, ldc;
  __device__ __forceinline__ T neutral() const { return 0.0f; }
  __device__ __forceinline__ bool is_absorb(T a) const { return a == __int_as_float(0x7f800000); }
  // the matrix stream evicts first, the gathered rows of B stay in L2
  __device__ __forceinline__ T mulk(int64_t k, int32_t col1, int64_t, int64_t j) const {
    return __fmul_rn(ld_stream_p(nz + k, l2_evict_first()),
                     ld_keep(x + (int64_t)(col1 - 1) * ldb + j, l2_evict_last()));
  }
  __device__ __forceinline__ T addv(T acc, T v) const { return __fadd_rn(acc, v); }
  __device__ __forceinline__ void write_mm(int64_t row0, int64_t j, T acc) const {
    y[row0 * ldc + j] = acc;
  }
};

// Fold entries [k0, k1) of row r1 (1-based) for dense columns j0 + 32 c (c < CPL) in
// storage order, stopping at the absorbing value like csr_spmm_kernel!
// (src/spmm/CSR.jl:3-35).  The warp loads 32 column indices at a time and broadcasts
// them; each lane keeps 8 x CPL gathers in flight.
template <class SR, int CPL>
__device__ __forceinline__ void fold_csr(const SR& sr, const int32_t* __restrict__ colval,
                                         int32_t k0, int32_t k1, int64_t r1, int64_t j0,
                                         int64_t jn_abs, int lane, typename SR::T (&acc)[CPL]) {
  typedef typename SR::T T;
  bool done[CPL];
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    acc[c] = sr.neutral();
    done[c] = j0 + 32 * c >= jn_abs;
  }
  for (int32_t base = k0; base < k1; base += 32) {
    const int32_t kk = base + lane;
    const int32_t col_l = kk < k1 ? __ldg(colval + kk) : 1;
    const int n = (k1 - base) < 32 ? (k1 - base) : 32;
    int i = 0;
    for (; i + 8 <= n; i += 8) {
      int32_t cidx[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) cidx[u] = __shfl_sync(kFullMM, col_l, i + u);
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        if (done[c]) continue;
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = sr.mulk(base + i + u, cidx[u], r1, j0 + 32 * c);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (!done[c]) {
            acc[c] = sr.addv(acc[c], v[u]);
            if (sr.is_absorb(acc[c])) done[c] = true;
          }
        }
      }
    }
    for (; i < n; ++i) {
      const int32_t cc = __shfl_sync(kFullMM, col_l, i);
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        if (!done[c]) {
          acc[c] = sr.addv(acc[c], sr.mulk(base + i, cc, r1, j0 + 32 * c));
          if (sr.is_absorb(acc[c])) done[c] = true;
        }
      }
    }
  }
}

// CSR: items [0, nseg) are pieces of rows longer than kSegMM (their partials go to
// partials[slot * jn + j - jlo]); items [nseg, nseg + nrows) are the rows of
// [row_lo, row_lo + nrows), one warp per row, lane per dense column (CPL columns per
// lane and pass), rows longer than kSegMM skipped.  Columns [jlo, jlo + jn).
template <class SR, int CPL>
__global__ void __launch_bounds__(256)
    k_csr_spmm(SR sr, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
               int64_t row_lo, int64_t nrows, int64_t jlo, int64_t jn, const void* mask, int tmask,
               const int4* __restrict__ segs, int64_t nseg, typename SR::T* partials,
               int32_t skip_le) {
  typedef typename SR::T T;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = w0; t < nseg + nrows; t += nw) {
    int64_t r;
    int32_t k0, k1, slot = -1;
    if (t < nseg) {
      const int4 sg = segs[t];
      r = sg.x;
      if (r < row_lo || r >= row_lo + nrows) continue;
      k0 = sg.y;
      k1 = sg.z;
      slot = sg.w;
    } else {
      r = row_lo + (t - nseg);
      k0 = __ldg(rowptr + r) - 1;
      k1 = __ldg(rowptr + r + 1) - 1;
      if (k1 - k0 > kSegMM || k1 - k0 <= skip_le) continue;
    }
    if (mask && raw_is_zero(load_raw(mask, tmask, r), tmask)) continue;
    for (int64_t jb = 0; jb < jn; jb += 32 * CPL) {
      T acc[CPL];
      fold_csr<SR, CPL>(sr, colval, k0, k1, r + 1, jlo + jb + lane, jlo + jn, lane, acc);
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int64_t jj = jb + lane + 32 * c;
        if (jj >= jn) continue;
        if (slot >= 0) partials[(int64_t)slot * jn + jj] = acc[c];
        else sr.write_mm(r, jlo + jj, acc[c]);
      }
    }
  }
}

// SELL: fold stored row t over slice columns [c0, c1) with stride C, stopping at the
// first -1 padding column or the absorbing value
template <class SR>
__device__ __forceinline__ typename SR::T fold_sell(const SR& sr, const int32_t* __restrict__ colval,
                                                    int64_t i0, int64_t i1, int64_t C, int64_t r1,
                                                    int64_t j) {
  typename SR::T acc = sr.neutral();
  for (int64_t i = i0; i < i1; i += C) {
    const int32_t col = __ldg(colval + i);
    if (col == -1 || sr.is_absorb(acc)) break;
    acc = sr.addv(acc, sr.mulk(i, col, r1, j));
  }
  return acc;
}

// SELL: items [0, nseg) are pieces of the rows of slices wider than kSegMM, items
// [nseg, nseg + s_hi - s_lo) one warp per stored row (rows of wide slices skipped)
template <class SR>
__global__ void __launch_bounds__(256)
    k_sell_spmm(SR sr, const int32_t* __restrict__ slice_ptr, const int32_t* __restrict__ colval,
                const int32_t* __restrict__ perm, int64_t C, int64_t s_lo, int64_t s_hi,
                int64_t jlo, int64_t jn, int64_t range_lo, int64_t range_hi, const void* mask,
                int tmask, const int4* __restrict__ segs, int64_t nseg, typename SR::T* partials) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t it = w0; it < nseg + (s_hi - s_lo); it += nw) {
    int64_t t, cb, ce;
    int slot = -1;
    if (it < nseg) {
      const int4 sg = segs[it];
      t = sg.x;
      cb = sg.y;
      ce = sg.z;
      slot = sg.w;
      if (t < s_lo || t >= s_hi) continue;
    } else {
      t = s_lo + (it - nseg);
      const int64_t s = t / C;
      ce = ((int64_t)slice_ptr[s + 1] - slice_ptr[s]) / C;
      if (ce > kSegMM) continue;
      cb = 0;
    }
    const int64_t s = t / C, o = t - s * C;
    const int64_t r1 = perm ? (int64_t)perm[t] : t + 1;
    if (range_lo > 0 && (r1 < range_lo || r1 > range_hi)) continue;
    if (mask && raw_is_zero(load_raw(mask, tmask, r1 - 1), tmask)) continue;
    const int64_t base = (int64_t)slice_ptr[s] - 1 + o;
    for (int64_t jb = 0; jb < jn; jb += 32) {
      const int64_t jj = jb + lane;
      if (jj >= jn) continue;
      const typename SR::T acc = fold_sell(sr, colval, base + cb * C, base + ce * C, C, r1, jlo + jj);
      if (slot >= 0) partials[(int64_t)slot * jn + jj] = acc;
      else sr.write_mm(r1 - 1, jlo + jj, acc);
    }
  }
}

// second pass over long rows: fold each row's piece partials in order
template <class SR>
__global__ void __launch_bounds__(256)
    k_spmm_combine(SR sr, const int32_t* __restrict__ rows, const int32_t* __restrict__ first,
                   int64_t nlong, const int32_t* __restrict__ perm, bool sell, int64_t row_lo,
                   int64_t row_hi, int64_t jlo, int64_t jn, const void* mask, int tmask,
                   const typename SR::T* __restrict__ partials) {
  typedef typename SR::T T;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t li = w0; li < nlong; li += nw) {
    const int64_t t = rows[li];
    const int64_t r0 = sell ? (perm ? (int64_t)perm[t] - 1 : t) : t;  // original row, 0-based
    if (r0 < row_lo || r0 >= row_hi) continue;
    if (mask && raw_is_zero(load_raw(mask, tmask, r0), tmask)) continue;
    const int32_t q0 = first[li], q1 = first[li + 1];
    for (int64_t jb = 0; jb < jn; jb += 32) {
      const int64_t jj = jb + lane;
      if (jj >= jn) continue;
      // the pieces' partials 8 at a time (a hub row has hundreds of pieces; one load
      // at a time left its warp long after the others), folded in order up to the stop
      T acc = sr.neutral();
      bool stop = false;
      for (int32_t q = q0; q < q1 && !stop; q += 8) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          v[u] = q + u < q1 ? partials[(int64_t)(q + u) * jn + jj] : sr.neutral();
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (q + u < q1 && !stop) {
            acc = sr.addv(acc, v[u]);
            stop = sr.is_absorb(acc);
          }
        }
      }
      sr.write_mm(r0, jlo + jj, acc);
    }
  }
}

// Rows of at most kShortMM entries, plus-times Float32, row-major B and C with
// 16-byte aligned rows: four rows per warp, 8 lanes per row, each lane owning 4
// consecutive columns (one float4 of B per entry), so a warp keeps four rows' gathers
// in flight instead of one.  Each column is still folded in storage order.
static const int kShortMM = 32;

// A column of a float4 accumulator whose sum ended NaN is folded again with the
// reference's stop at +Inf (CSR.jl:49-51), so results equal the sequential fold.
__device__ __noinline__ float4 spmm_refold4(float4 acc, const int32_t* __restrict__ colval,
                                           const float* __restrict__ nz, const float* Bj,
                                           int64_t ldb, int32_t k0, int32_t k1) {
  float r[4] = {acc.x, acc.y, acc.z, acc.w};
  for (int q = 0; q < 4; ++q) {
    if (r[q] == r[q]) continue;
    float s = 0.0f;
    for (int32_t k = k0; k < k1; ++k) {
      s = __fadd_rn(s, __fmul_rn(__ldg(nz + k), __ldg(Bj + (int64_t)(__ldg(colval + k) - 1) * ldb + q)));
      if (s == __int_as_float(0x7f800000)) break;
    }
    r[q] = s;
  }
  return make_float4(r[0], r[1], r[2], r[3]);
}

__device__ __forceinline__ void fold4(float4& acc, float a, const float4& b) {
  acc.x = __fadd_rn(acc.x, __fmul_rn(a, b.x));
  acc.y = __fadd_rn(acc.y, __fmul_rn(a, b.y));
  acc.z = __fadd_rn(acc.z, __fmul_rn(a, b.z));
  acc.w = __fadd_rn(acc.w, __fmul_rn(a, b.w));
}

#ifndef GG_MM_SHORT_STEP
#define GG_MM_SHORT_STEP 4
#endif
static const int kMMShortStep = GG_MM_SHORT_STEP;  // entries of a short row per step

__global__ void __launch_bounds__(256)
    k_spmm_short_f32x4(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
                       const float* __restrict__ nz, const float* __restrict__ B, int64_t ldb,
                       float* __restrict__ C, int64_t ldc, int64_t row_lo, int64_t nrows,
                       int64_t jlo, int64_t jn, const int32_t* __restrict__ rows) {
  const int lane = threadIdx.x & 31;
  const int grp = lane >> 3, sub = lane & 7;
  const uint64_t pol_s = l2_evict_first(), pol_b = l2_evict_last();
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = gw * 4; base < nrows; base += nw * 4) {
    const int64_t t = base + grp;
    if (t >= nrows) continue;
    const int64_t r = rows ? (int64_t)__ldg(rows + t) : row_lo + t;
    const int32_t k0 = __ldg(rowptr + r) - 1, k1 = __ldg(rowptr + r + 1) - 1;
    if (k1 - k0 > kShortMM) continue;
    for (int64_t jb = 0; jb < jn; jb += 32) {
      const int64_t j = jlo + jb + 4 * sub;
      if (jb + 4 * sub >= jn) continue;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      // kMMShortStep entries per step in storage order, the next step's words loaded ahead
      int32_t c[kMMShortStep], cn[kMMShortStep];
      float a[kMMShortStep], an[kMMShortStep];
#pragma unroll
      for (int u = 0; u < kMMShortStep; ++u) {
        const bool in = k0 + u < k1;
        c[u] = in ? ld_stream_p(colval + k0 + u, pol_s) - 1 : 0;
        a[u] = in ? ld_stream_p(nz + k0 + u, pol_s) : 0.0f;
      }
      for (int32_t k = k0; k < k1; k += kMMShortStep) {
#pragma unroll
        for (int u = 0; u < kMMShortStep; ++u) {
          const bool in = k + kMMShortStep + u < k1;
          cn[u] = in ? ld_stream_p(colval + k + kMMShortStep + u, pol_s) - 1 : 0;
          an[u] = in ? ld_stream_p(nz + k + kMMShortStep + u, pol_s) : 0.0f;
        }
        float4 b[kMMShortStep];
#pragma unroll
        for (int u = 0; u < kMMShortStep; ++u)
          b[u] = k + u < k1 ? ld_keep4(B + (int64_t)c[u] * ldb + j, pol_b) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kMMShortStep; ++u)
          if (k + u < k1) fold4(acc, a[u], b[u]);
#pragma unroll
        for (int u = 0; u < kMMShortStep; ++u) {
          c[u] = cn[u];
          a[u] = an[u];
        }
      }
      if (acc.x != acc.x || acc.y != acc.y || acc.z != acc.z || acc.w != acc.w)
        acc = spmm_refold4(acc, colval, nz, B + j, ldb, k0, k1);
      st_hint4(C + r * ldc + j, acc, pol_s);
    }
  }
}

// Rows of 33..kSegMM entries and the pieces of longer rows, plus-times Float32 on
// 16-byte aligned row-major operands: four items per warp (longest first, so the four
// have about the same length), 8 lanes per item, each lane 4 dense columns with float4
// loads of B; every item is folded in storage order (kMMStep entries per step, the
// next step's column / value words loaded while the current B rows are in flight;
// 4 / 8 / 16 entries per step measured 3.67 / 3.23 / 3.98 ms at R-MAT scale 22, k = 32).
#ifndef GG_MM_STEP
#define GG_MM_STEP 8
#endif
static const int kMMStep = GG_MM_STEP;  // entries of an item folded per step

__global__ void __launch_bounds__(256)
    k_spmm_items_f32x4(const int32_t* __restrict__ colval, const float* __restrict__ nz,
                       const float* __restrict__ B, int64_t ldb, float* __restrict__ C, int64_t ldc,
                       const int4* __restrict__ items, int64_t nitems, int64_t row_lo,
                       int64_t row_hi, int64_t jlo, int64_t jn, float* partials) {
  const int lane = threadIdx.x & 31;
  const int grp = lane >> 3, sub = lane & 7;
  const uint64_t pol_s = l2_evict_first(), pol_b = l2_evict_last();
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = gw * 4; base < nitems; base += nw * 4) {
    const int64_t t = base + grp;
    if (t >= nitems) continue;
    const int4 d = items[t];  // row, first entry, end entry, partial slot or -1
    if (d.x < row_lo || d.x >= row_hi) continue;
    for (int64_t jb = 0; jb < jn; jb += 32) {
      const int64_t jj = jb + 4 * sub;
      if (jj >= jn) continue;
      const float* Bj = B + jlo + jj;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      int32_t c[kMMStep], cn[kMMStep];
      float a[kMMStep], an[kMMStep];
#pragma unroll
      for (int u = 0; u < kMMStep; ++u) {
        const bool in = d.y + u < d.z;
        c[u] = in ? ld_stream_p(colval + d.y + u, pol_s) - 1 : 0;
        a[u] = in ? ld_stream_p(nz + d.y + u, pol_s) : 0.0f;
      }
      for (int32_t k = d.y; k < d.z; k += kMMStep) {
#pragma unroll
        for (int u = 0; u < kMMStep; ++u) {
          const bool in = k + kMMStep + u < d.z;
          cn[u] = in ? ld_stream_p(colval + k + kMMStep + u, pol_s) - 1 : 0;
          an[u] = in ? ld_stream_p(nz + k + kMMStep + u, pol_s) : 0.0f;
        }
        float4 b[kMMStep];
#pragma unroll
        for (int u = 0; u < kMMStep; ++u)
          b[u] = k + u < d.z ? ld_keep4(Bj + (int64_t)c[u] * ldb, pol_b) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kMMStep; ++u)
          if (k + u < d.z) fold4(acc, a[u], b[u]);
#pragma unroll
        for (int u = 0; u < kMMStep; ++u) {
          c[u] = cn[u];
          a[u] = an[u];
        }
      }
      if (acc.x != acc.x || acc.y != acc.y || acc.z != acc.z || acc.w != acc.w)
        acc = spmm_refold4(acc, colval, nz, Bj, ldb, d.y, d.z);
      float* out = d.w < 0 ? C + (int64_t)d.x * ldc + jlo + jj : partials + (int64_t)d.w * jn + jj;
      if (d.w < 0) st_hint4(out, acc, pol_s);
      else *reinterpret_cast<float4*>(out) = acc;
    }
  }
}

// One dense column (a served SpMV iteration runs as an n x 1 SpMM so that it folds
// exactly like a column of the 32-column executor): a thread per row of <= 32 entries
// and a thread per item (rows of 33..kSegMM entries, pieces of longer rows), each
// folded in storage order 8 entries per load group, NaN sums folded again with the
// stop at +Inf.  The warp-per-row kernel leaves 31 of 32 lanes idle on one column.
__device__ __forceinline__ float col1_fold(const int32_t* __restrict__ colval,
                                           const float* __restrict__ nz, const float* B, int64_t ldb,
                                           int32_t k0, int32_t k1, uint64_t pol_s, uint64_t pol_b) {
  float acc = 0.0f;
  for (int32_t kb = k0; kb < k1; kb += 8) {
    int32_t c[8];
    float a[8], b[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const bool in = kb + t < k1;
      c[t] = in ? ld_stream_p(colval + kb + t, pol_s) - 1 : 0;
      a[t] = in ? ld_stream_p(nz + kb + t, pol_s) : 0.0f;
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) b[t] = kb + t < k1 ? ld_keep(B + (int64_t)c[t] * ldb, pol_b) : 0.0f;
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (kb + t < k1) acc = __fadd_rn(acc, __fmul_rn(a[t], b[t]));
  }
  if (acc != acc) {
    acc = 0.0f;
    for (int32_t k = k0; k < k1; ++k) {
      acc = __fadd_rn(acc, __fmul_rn(__ldg(nz + k), __ldg(B + (int64_t)(__ldg(colval + k) - 1) * ldb)));
      if (acc == __int_as_float(0x7f800000)) break;
    }
  }
  return acc;
}

__global__ void __launch_bounds__(256)
    k_spmm_col1_short(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
                      const float* __restrict__ nz, const float* __restrict__ B, int64_t ldb,
                      float* __restrict__ C, int64_t ldc, int64_t row_lo, int64_t nrows) {
  const uint64_t pol_s = l2_evict_first(), pol_b = l2_evict_last();
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nrows;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = row_lo + t;
    const int32_t k0 = __ldg(rowptr + r) - 1, k1 = __ldg(rowptr + r + 1) - 1;
    if (k1 - k0 > kShortMM) continue;
    C[r * ldc] = col1_fold(colval, nz, B, ldb, k0, k1, pol_s, pol_b);
  }
}

__global__ void __launch_bounds__(256)
    k_spmm_col1_items(const int32_t* __restrict__ colval, const float* __restrict__ nz,
                      const float* __restrict__ B, int64_t ldb, float* __restrict__ C, int64_t ldc,
                      const int4* __restrict__ items, int64_t nitems, int64_t row_lo, int64_t row_hi,
                      float* partials) {
  const uint64_t pol_s = l2_evict_first(), pol_b = l2_evict_last();
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nitems;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int4 d = items[t];  // row, first entry, end entry, partial slot or -1
    if (d.x < row_lo || d.x >= row_hi) continue;
    const float v = col1_fold(colval, nz, B, ldb, d.y, d.z, pol_s, pol_b);
    if (d.w < 0) C[(int64_t)d.x * ldc] = v;
    else partials[d.w] = v;
  }
}

static int grid_mm(gg_ctx* ctx, int64_t warps);

// which semirings / operands take the short-row kernel
template <class SR>
struct ShortRowsMM {
  static bool ok(const SR&, int64_t, int64_t, const void*) { return false; }
  static void launch(gg_ctx*, const SR&, const int32_t*, const int32_t*, int64_t, int64_t, int64_t,
                     int64_t, const int32_t*) {}
  static void launch_items(gg_ctx*, const SR&, const int32_t*, const MMPlan*, int64_t, int64_t,
                           int64_t, int64_t, typename SR::T*) {}
  static bool ok1(const SR&, int64_t, const void*) { return false; }
  static void launch1(gg_ctx*, const SR&, const int32_t*, const int32_t*, const MMPlan*, int64_t,
                      int64_t, int64_t, typename SR::T*) {}
};
template <>
struct ShortRowsMM<SRPlusTimesF32MM> {
  static bool ok(const SRPlusTimesF32MM& sr, int64_t jlo, int64_t jn, const void* mask) {
    const bool aligned = ((uintptr_t)sr.x % 16 == 0) && ((uintptr_t)sr.y % 16 == 0) &&
                         sr.ldb % 4 == 0 && sr.ldc % 4 == 0;
    return !mask && aligned && jlo % 4 == 0 && jn % 4 == 0;
  }
  // rows: the plan's short rows longest first (every row of the matrix), or nullptr
  // for the rows row_lo .. row_lo + nrows - 1 in order
  static void launch(gg_ctx* ctx, const SRPlusTimesF32MM& sr, const int32_t* rowptr,
                     const int32_t* colval, int64_t row_lo, int64_t nrows, int64_t jlo, int64_t jn,
                     const int32_t* rows) {
    k_spmm_short_f32x4<<<grid_mm(ctx, (nrows + 3) / 4), 256, 0, ctx->stream>>>(
        rowptr, colval, sr.nz, sr.x, sr.ldb, sr.y, sr.ldc, row_lo, nrows, jlo, jn, rows);
  }
  // one dense column, no mask: the thread-per-row kernels
  static bool ok1(const SRPlusTimesF32MM&, int64_t jn, const void* mask) { return !mask && jn == 1; }
  static void launch1(gg_ctx* ctx, const SRPlusTimesF32MM& sr, const int32_t* rowptr,
                      const int32_t* colval, const MMPlan* P, int64_t row_lo, int64_t row_hi,
                      int64_t jlo, float* partials) {
    const int64_t nrows = row_hi - row_lo;
    k_spmm_col1_short<<<grid_mm(ctx, (nrows + 31) / 32), 256, 0, ctx->stream>>>(
        rowptr, colval, sr.nz, sr.x + jlo, sr.ldb, sr.y + jlo, sr.ldc, row_lo, nrows);
    if (P->nitems > 0)
      k_spmm_col1_items<<<grid_mm(ctx, (P->nitems + 31) / 32), 256, 0, ctx->stream>>>(
          colval, sr.nz, sr.x + jlo, sr.ldb, sr.y + jlo, sr.ldc, P->items, P->nitems, row_lo, row_hi,
          partials);
  }
  static void launch_items(gg_ctx* ctx, const SRPlusTimesF32MM& sr, const int32_t* colval,
                           const MMPlan* P, int64_t row_lo, int64_t row_hi, int64_t jlo, int64_t jn,
                           float* partials) {
    k_spmm_items_f32x4<<<grid_mm(ctx, (P->nitems + 3) / 4), 256, 0, ctx->stream>>>(
        colval, sr.nz, sr.x, sr.ldb, sr.y, sr.ldc, P->items, P->nitems, row_lo, row_hi, jlo, jn,
        partials);
  }
};

static int grid_mm(gg_ctx* ctx, int64_t warps) {
  int64_t g = (warps * 32 + 255) / 256;
  int64_t cap = (int64_t)ctx->num_sms * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// long-row pieces, built once per matrix from rowptr (CSR) or slice_ptr (SELL)
static int build_mm_plan(gg_ctx* ctx, gg_mat* A) {
  if (A->mmplan) return GG_OK;
  std::vector<int4> segs, items;
  std::vector<int32_t> first, rows, short_rows;
  if (A->format == GG_FMT_CSR) {
    const int64_t m = A->m;
    std::vector<int32_t> rp(m + 1);
    GG_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr, (m + 1) * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    {
      std::vector<int64_t> cnt(kShortMM + 2, 0);  // rows per length, longest first
      for (int64_t r = 0; r < m; ++r) {
        const int64_t L = rp[r + 1] - rp[r];
        if (L <= kShortMM) ++cnt[kShortMM - L + 1];
      }
      for (int i = 1; i <= kShortMM + 1; ++i) cnt[i] += cnt[i - 1];
      short_rows.resize(cnt[kShortMM + 1]);
      for (int64_t r = 0; r < m; ++r) {
        const int64_t L = rp[r + 1] - rp[r];
        if (L <= kShortMM) short_rows[cnt[kShortMM - L]++] = (int32_t)r;
      }
    }
    for (int64_t r = 0; r < m; ++r) {
      const int64_t k0 = rp[r] - 1, k1 = rp[r + 1] - 1;
      if (k1 - k0 > kShortMM && k1 - k0 <= kSegMM) items.push_back(make_int4((int)r, (int)k0, (int)k1, -1));
      if (k1 - k0 <= kSegMM) continue;
      rows.push_back((int32_t)r);
      first.push_back((int32_t)segs.size());
      for (int64_t kb = k0; kb < k1; kb += kSegMM) {
        const int64_t ke = kb + kSegMM < k1 ? kb + kSegMM : k1;
        segs.push_back(make_int4((int)r, (int)kb, (int)ke, (int)segs.size()));
      }
    }
  } else {
    const int64_t ns = A->nslices, C = A->slice_size;
    std::vector<int32_t> sp(ns + 1);
    GG_CUDA(cudaMemcpyAsync(sp.data(), A->slice_ptr, (ns + 1) * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int64_t s = 0; s < ns; ++s) {
      const int64_t L = C > 0 ? ((int64_t)sp[s + 1] - sp[s]) / C : 0;
      if (L <= kSegMM) continue;
      for (int64_t o = 0; o < C && s * C + o < A->m; ++o) {
        const int64_t t = s * C + o;
        rows.push_back((int32_t)t);
        first.push_back((int32_t)segs.size());
        for (int64_t cb = 0; cb < L; cb += kSegMM) {
          const int64_t ce = cb + kSegMM < L ? cb + kSegMM : L;
          segs.push_back(make_int4((int)t, (int)cb, (int)ce, (int)segs.size()));
        }
      }
    }
  }
  first.push_back((int32_t)segs.size());
  items.insert(items.end(), segs.begin(), segs.end());
  std::stable_sort(items.begin(), items.end(),
                   [](const int4& a, const int4& b) { return (a.z - a.y) > (b.z - b.y); });
  MMPlan* P = new MMPlan();
  P->nitems = A->format == GG_FMT_CSR ? (int64_t)items.size() : 0;
  P->nseg = (int64_t)segs.size();
  P->nlong = (int64_t)rows.size();
  cudaError_t e = cudaSuccess;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(dst, bytes > 0 ? bytes : 16);
    if (e == cudaSuccess && bytes > 0)
      e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  };
  up((void**)&P->segs, segs.data(), segs.size() * sizeof(int4));
  up((void**)&P->first, first.data(), first.size() * sizeof(int32_t));
  up((void**)&P->rows, rows.data(), rows.size() * sizeof(int32_t));
  up((void**)&P->items, items.data(), (size_t)P->nitems * sizeof(int4));
  P->nshort = (int64_t)short_rows.size();
  up((void**)&P->short_rows, short_rows.data(), short_rows.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(P->segs);
    cudaFree(P->first);
    cudaFree(P->rows);
    cudaFree(P->items);
    cudaFree(P->short_rows);
    delete P;
    return cuda_error(e, "SpMM long-row analysis");
  }
  A->mmplan = P;
  return GG_OK;
}

// partial buffers are bounded: wide dense operands run in column windows
static const int64_t kMMPartialBytes = (int64_t)256 << 20;

// one dense column of plus-times Float32 over a large CSR handle: the SELL-32 copy's
// kernel with the SpMM's fold order (launch_col1_sell, gg_spmv.cu); other semirings
// and operands keep the kernels below
template <class SR>
static bool col1_sell_ok(const gg_mat*, const SR&, int64_t, const void*, int64_t) { return false; }
static bool col1_sell_ok(const gg_mat* A, const SRPlusTimesF32MM& sr, int64_t k, const void* mask,
                         int64_t lo) {
  return A->format == GG_FMT_CSR && A->m >= (1 << 16) && k == 1 && !mask && lo == 0 &&
         sr.ldb == 1 && sr.ldc == 1;
}
template <class SR>
static int col1_sell(gg_ctx*, gg_mat*, const SR&) { return GG_ERR_UNSUPPORTED; }
static int col1_sell(gg_ctx* ctx, gg_mat* A, const SRPlusTimesF32MM& sr) {
  return launch_col1_sell(ctx, A, sr.x, sr.y);
}

template <class SR>
static int launch_mm(gg_ctx* ctx, gg_mat* A, const SR& sr, int64_t k, const void* mask, int tmask,
                     int64_t lo, int64_t hi) {
  typedef typename SR::T T;
  const int64_t m = A->m;
  if (col1_sell_ok(A, sr, k, mask, lo)) return col1_sell(ctx, A, sr);
  GG_CHECK(build_mm_plan(ctx, A));
  const MMPlan* P = A->mmplan;
  int64_t jwin = k;
  if (P->nseg > 0) {
    const int64_t per_col = P->nseg * (int64_t)sizeof(T);
    const int64_t cap = kMMPartialBytes / per_col;
    if (jwin > cap) jwin = cap < 32 ? 32 : (cap / 32) * 32;
    GG_CHECK(ensure_scratch(ctx, (size_t)(per_col * jwin)));
  }
  T* partials = static_cast<T*>(ctx->scratch);
  const int64_t row_lo = lo > 0 ? lo - 1 : 0;
  const int64_t row_hi = lo > 0 ? hi : m;
  for (int64_t jlo = 0; jlo < k; jlo += jwin) {
    const int64_t jn = k - jlo < jwin ? k - jlo : jwin;
    int tr = -1;
    if (A->format == GG_FMT_CSR) {
      const int64_t nrows = row_hi - row_lo;
      const int cpl = A->mm_cpl == 4 && jn >= 128 ? 4 : (A->mm_cpl >= 2 && jn >= 64 ? 2 : 1);
      // plus-times Float32 on 16-byte aligned row-major operands: rows of <= 32 entries
      // go to the four-rows-per-warp float4 kernel
      int32_t skip = -1;  // rows of at most `skip` entries are left to the short-row kernel
      if (ShortRowsMM<SR>::ok1(sr, jn, mask)) {
        tr = trace_main_begin(ctx);
        ShortRowsMM<SR>::launch1(ctx, sr, A->rowptr, A->colval, P, row_lo, row_hi, jlo, partials);
        if (P->nitems > 0) trace_count(ctx, 1);  // the second of the two kernels
      } else if (ShortRowsMM<SR>::ok(sr, jlo, jn, mask)) {
        // Float32 fast path: short rows four per warp, the rest (medium rows and the
        // pieces of long rows) by the item kernel
        // every row (no range): the short rows longest first, four of a length per warp
        const bool all = row_lo == 0 && nrows == m;
        ShortRowsMM<SR>::launch(ctx, sr, A->rowptr, A->colval, row_lo, all ? P->nshort : nrows, jlo,
                                jn, all ? P->short_rows : nullptr);
        trace_count(ctx, 1);
        tr = trace_main_begin(ctx);
        if (P->nitems > 0)
          ShortRowsMM<SR>::launch_items(ctx, sr, A->colval, P, row_lo, row_hi, jlo, jn, partials);
      } else {
      tr = trace_main_begin(ctx);
      if (cpl == 4)
        k_csr_spmm<SR, 4><<<grid_mm(ctx, P->nseg + nrows), 256, 0, ctx->stream>>>(
            sr, A->rowptr, A->colval, row_lo, nrows, jlo, jn, mask, tmask, P->segs, P->nseg, partials,
            skip);
      else if (cpl == 2)
        k_csr_spmm<SR, 2><<<grid_mm(ctx, P->nseg + nrows), 256, 0, ctx->stream>>>(
            sr, A->rowptr, A->colval, row_lo, nrows, jlo, jn, mask, tmask, P->segs, P->nseg, partials,
            skip);
      else
        k_csr_spmm<SR, 1><<<grid_mm(ctx, P->nseg + nrows), 256, 0, ctx->stream>>>(
            sr, A->rowptr, A->colval, row_lo, nrows, jlo, jn, mask, tmask, P->segs, P->nseg, partials,
            skip);
      }
    } else {
      int64_t s_lo = 0, s_hi = m;
      if (lo > 0) {
        const int64_t w = A->sigma > 1 ? A->sigma : 1;
        s_lo = ((lo - 1) / w) * w;
        s_hi = ((hi + w - 1) / w) * w;
        if (s_hi > m) s_hi = m;
      }
      tr = trace_main_begin(ctx);
      k_sell_spmm<SR><<<grid_mm(ctx, P->nseg + s_hi - s_lo), 256, 0, ctx->stream>>>(
          sr, A->slice_ptr, A->colval, A->sigma > 1 ? A->perm : nullptr, A->slice_size, s_lo, s_hi,
          jlo, jn, lo, hi, mask, tmask, P->segs, P->nseg, partials);
    }
    trace_main_end(ctx, tr);
    trace_count(ctx, 1);
    GG_CUDA(cudaGetLastError());
    if (P->nlong > 0) {
      trace_count(ctx, 1);
      k_spmm_combine<SR><<<grid_mm(ctx, P->nlong), 256, 0, ctx->stream>>>(
          sr, P->rows, P->first, P->nlong, A->sigma > 1 ? A->perm : nullptr,
          A->format != GG_FMT_CSR, row_lo, row_hi, jlo, jn, mask, tmask, partials);
      GG_CUDA(cudaGetLastError());
    }
  }
  return GG_OK;
}

template <int TC>
static int spmm_generic(gg_ctx* ctx, gg_mat* A, int mul, int add, int accum, void* Cm, int tcm,
                        int64_t ldc, const void* B, int tb, int64_t ldb, int64_t k, int layout,
                        const void* mask, int tmask, int64_t lo, int64_t hi) {
  typedef typename CType<TC>::T T;
  SRGen<TC> sr;
  sr.mul = mul;
  sr.add = add;
  sr.accum = accum;
  sr.tv = A->dtype;
  sr.tx = tb;
  sr.ty = tcm;
  sr.neutral_v = neutral_of<T>(add);
  sr.has_absorb = absorb_of<T>(add, &sr.absorb_v);
  sr.nz = A->nzval;
  sr.x = B;
  sr.y = Cm;
  sr.ldb = ldb;
  sr.ldc = ldc;
  sr.layout = layout;
  return launch_mm(ctx, A, sr, k, mask, tmask, lo, hi);
}

int spmm_dispatch(gg_ctx* ctx, gg_mat* A, int tc, int mul, int add, int accum, void* Cm, int tcm,
                  int64_t ldc, const void* B, int tb, int64_t ldb, int64_t k, int layout,
                  const void* mask, int tmask, int64_t lo, int64_t hi) {
  if (k == 1 && layout == GG_COL_MAJOR) {
    // one column-major dense column is the same memory as a row-major one with
    // leading dimension 1, so the row-major one-column kernels serve it
    layout = GG_ROW_MAJOR;
    ldb = 1;
    ldc = 1;
  }
  if (layout == GG_ROW_MAJOR && A->dtype == GG_FLOAT32 && tb == GG_FLOAT32 && tcm == GG_FLOAT32 &&
      mul == GG_OP_MUL && add == GG_OP_ADD && accum == GG_OP_SECOND) {
    SRPlusTimesF32MM sr;
    sr.nz = static_cast<const float*>(A->nzval);
    sr.x = static_cast<const float*>(B);
    sr.y = static_cast<float*>(Cm);
    sr.ldb = ldb;
    sr.ldc = ldc;
    return launch_mm(ctx, A, sr, k, mask, tmask, lo, hi);
  }
  switch (tc) {
    case GG_BOOL: return spmm_generic<GG_BOOL>(ctx, A, mul, add, accum, Cm, tcm, ldc, B, tb, ldb, k, layout, mask, tmask, lo, hi);
    case GG_INT32: return spmm_generic<GG_INT32>(ctx, A, mul, add, accum, Cm, tcm, ldc, B, tb, ldb, k, layout, mask, tmask, lo, hi);
    case GG_INT64: return spmm_generic<GG_INT64>(ctx, A, mul, add, accum, Cm, tcm, ldc, B, tb, ldb, k, layout, mask, tmask, lo, hi);
    case GG_FLOAT32: return spmm_generic<GG_FLOAT32>(ctx, A, mul, add, accum, Cm, tcm, ldc, B, tb, ldb, k, layout, mask, tmask, lo, hi);
    default: return spmm_generic<GG_FLOAT64>(ctx, A, mul, add, accum, Cm, tcm, ldc, B, tb, ldb, k, layout, mask, tmask, lo, hi);
  }
}

}  // namespace gg
