// gg_spmm.cu -- semiring SpMM over CSR and SELL (gpu_spmm!, src/spmm/CSR.jl and
// src/spmm/SELL.jl of GPUGraphs.jl).
//
// One warp per row; lane j owns output column j (32 columns per pass).  The warp
// loads 32 (column, value) pairs of the row with one coalesced access each, then
// broadcasts them by shuffle; every lane folds its (row, j) sequentially in storage
// order -- the order of csr_spmm_kernel! (src/spmm/CSR.jl:3-35), so results equal
// the reference's bit for bit, including its early exit on the absorbing value.
// With a row-major dense operand (the batched-query layout) each gathered B row is
// one contiguous 128-byte read.
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
  __device__ __forceinline__ T mulk(int64_t k, int32_t col1, int64_t, int64_t j) const {
    return __fmul_rn(__ldg(nz + k), __ldg(x + (int64_t)(col1 - 1) * ldb + j));
  }
  __device__ __forceinline__ T addv(T acc, T v) const { return __fadd_rn(acc, v); }
  __device__ __forceinline__ void write_mm(int64_t row0, int64_t j, T acc) const {
    y[row0 * ldc + j] = acc;
  }
};

// CSR: one warp per row of [row_lo, row_lo + nrows)
template <class SR>
__global__ void __launch_bounds__(256)
    k_csr_spmm(SR sr, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
               int64_t row_lo, int64_t nrows, int64_t kcols, const void* mask, int tmask) {
  typedef typename SR::T T;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = w0; t < nrows; t += nw) {
    const int64_t r = row_lo + t;
    if (mask && raw_is_zero(load_raw(mask, tmask, r), tmask)) continue;
    const int32_t k0 = __ldg(rowptr + r) - 1, k1 = __ldg(rowptr + r + 1) - 1;
    for (int64_t jb = 0; jb < kcols; jb += 32) {
      const int64_t j = jb + lane;
      const bool active = j < kcols;
      T acc = sr.neutral();
      bool done = !active;
      for (int32_t base = k0; base < k1; base += 32) {
        const int32_t kk = base + lane;
        const int32_t col_l = kk < k1 ? __ldg(colval + kk) : 1;
        const int n = (k1 - base) < 32 ? (k1 - base) : 32;
        int i = 0;
        for (; i + 4 <= n; i += 4) {
          const int32_t c0 = __shfl_sync(kFullMM, col_l, i);
          const int32_t c1 = __shfl_sync(kFullMM, col_l, i + 1);
          const int32_t c2 = __shfl_sync(kFullMM, col_l, i + 2);
          const int32_t c3 = __shfl_sync(kFullMM, col_l, i + 3);
          if (!done) {
            const T v0 = sr.mulk(base + i, c0, r + 1, j);
            const T v1 = sr.mulk(base + i + 1, c1, r + 1, j);
            const T v2 = sr.mulk(base + i + 2, c2, r + 1, j);
            const T v3 = sr.mulk(base + i + 3, c3, r + 1, j);
            acc = sr.addv(acc, v0);
            if (sr.is_absorb(acc)) done = true;
            if (!done) { acc = sr.addv(acc, v1); if (sr.is_absorb(acc)) done = true; }
            if (!done) { acc = sr.addv(acc, v2); if (sr.is_absorb(acc)) done = true; }
            if (!done) { acc = sr.addv(acc, v3); if (sr.is_absorb(acc)) done = true; }
          }
        }
        for (; i < n; ++i) {
          const int32_t c = __shfl_sync(kFullMM, col_l, i);
          if (!done) {
            acc = sr.addv(acc, sr.mulk(base + i, c, r + 1, j));
            if (sr.is_absorb(acc)) done = true;
          }
        }
      }
      if (active) sr.write_mm(r, j, acc);
    }
  }
}

// SELL: one warp per stored row, walking its slice with stride C
template <class SR>
__global__ void __launch_bounds__(256)
    k_sell_spmm(SR sr, const int32_t* __restrict__ slice_ptr, const int32_t* __restrict__ colval,
                const int32_t* __restrict__ perm, int64_t C, int64_t s_lo, int64_t s_hi,
                int64_t kcols, int64_t range_lo, int64_t range_hi, const void* mask, int tmask) {
  typedef typename SR::T T;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = s_lo + w0; t < s_hi; t += nw) {
    const int64_t s = t / C, o = t - s * C;
    const int64_t r1 = perm ? (int64_t)perm[t] : t + 1;
    if (range_lo > 0 && (r1 < range_lo || r1 > range_hi)) continue;
    if (mask && raw_is_zero(load_raw(mask, tmask, r1 - 1), tmask)) continue;
    const int64_t i0 = (int64_t)slice_ptr[s] - 1 + o, i1 = (int64_t)slice_ptr[s + 1] - 1;
    for (int64_t jb = 0; jb < kcols; jb += 32) {
      const int64_t j = jb + lane;
      if (j >= kcols) continue;
      T acc = sr.neutral();
      for (int64_t i = i0; i < i1; i += C) {
        const int32_t col = __ldg(colval + i);
        if (col == -1 || sr.is_absorb(acc)) break;
        acc = sr.addv(acc, sr.mulk(i, col, r1, j));
      }
      sr.write_mm(r1 - 1, j, acc);
    }
  }
}

static int grid_mm(gg_ctx* ctx, int64_t warps) {
  int64_t g = (warps * 32 + 255) / 256;
  int64_t cap = (int64_t)ctx->num_sms * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

template <class SR>
static int launch_mm(gg_ctx* ctx, gg_mat* A, const SR& sr, int64_t k, const void* mask, int tmask,
                     int64_t lo, int64_t hi) {
  const int64_t m = A->m;
  if (A->format == GG_FMT_CSR) {
    const int64_t row_lo = lo > 0 ? lo - 1 : 0;
    const int64_t nrows = lo > 0 ? hi - lo + 1 : m;
    k_csr_spmm<SR><<<grid_mm(ctx, nrows), 256, 0, ctx->stream>>>(sr, A->rowptr, A->colval, row_lo,
                                                                 nrows, k, mask, tmask);
  } else {
    int64_t s_lo = 0, s_hi = m;
    if (lo > 0) {
      const int64_t w = A->sigma > 1 ? A->sigma : 1;
      s_lo = ((lo - 1) / w) * w;
      s_hi = ((hi + w - 1) / w) * w;
      if (s_hi > m) s_hi = m;
    }
    k_sell_spmm<SR><<<grid_mm(ctx, s_hi - s_lo), 256, 0, ctx->stream>>>(
        sr, A->slice_ptr, A->colval, A->sigma > 1 ? A->perm : nullptr, A->slice_size, s_lo, s_hi, k,
        lo, hi, mask, tmask);
  }
  GG_CUDA(cudaGetLastError());
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
