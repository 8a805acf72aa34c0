// gg_semiring.cuh -- semiring policies used by the sparse kernels.
//
// A policy supplies the accumulator type T and the four steps every reference
// kernel performs (src/spmv/CSR.jl:31-54, src/spmm/CSR.jl:3-35):
//   acc = neutral();  acc = add(acc, mul(A[k], B[col[k], j], row, col, col, j));
//   stop early when acc == absorb;  C[row, j] = accum(C[row, j], acc, ...)
// SRGen evaluates runtime operator codes and element types (any supported
// combination); the fixed policies are compile-time specialisations for the hot
// semirings.
#pragma once

#include "gg_common.cuh"

namespace gg {

// y[idx] = accum(y[idx], acc) evaluated in y's element type ty (>= TC).
template <int TY, int TC>
__device__ __forceinline__ void accum_store_t(void* y, int64_t idx, typename CType<TC>::T acc,
                                              int accum, int64_t ai, int64_t aj, int64_t bi,
                                              int64_t bj) {
  typedef typename CType<TY>::T Y;
  Raw r;
  r.i = 0;
  r.d = 0;
  if (dtype_is_float(TC)) r.d = static_cast<double>(acc);
  else r.i = static_cast<int64_t>(acc);
  Y a = raw_to<TY>(r, TC);
  Y* yp = static_cast<Y*>(y);
  Y old = yp[idx];
  Raw ar;
  ar.i = 0;
  ar.d = 0;
  if (dtype_is_float(TY)) ar.d = static_cast<double>(a);
  else ar.i = static_cast<int64_t>(a);
  Y v = (accum == GG_OP_SECOND) ? a : apply_op<TY>(accum, old, a, ar, TY, ai, aj, bi, bj);
  if (TY == GG_BOOL) v = (v != Y(0)) ? Y(1) : Y(0);
  yp[idx] = v;
}

template <int TC>
__device__ __forceinline__ void accum_store(void* y, int ty, int64_t idx,
                                            typename CType<TC>::T acc, int accum, int64_t ai,
                                            int64_t aj, int64_t bi, int64_t bj) {
  switch (ty) {
    case GG_BOOL: accum_store_t<GG_BOOL, TC>(y, idx, acc, accum, ai, aj, bi, bj); break;
    case GG_INT32: accum_store_t<GG_INT32, TC>(y, idx, acc, accum, ai, aj, bi, bj); break;
    case GG_INT64: accum_store_t<GG_INT64, TC>(y, idx, acc, accum, ai, aj, bi, bj); break;
    case GG_FLOAT32: accum_store_t<GG_FLOAT32, TC>(y, idx, acc, accum, ai, aj, bi, bj); break;
    default: accum_store_t<GG_FLOAT64, TC>(y, idx, acc, accum, ai, aj, bi, bj); break;
  }
}

// ---------------------------------------------------------------------------------
// generic policy: runtime operators and element types; B is a vector (ldb == 0) or a
// dense matrix (column-major or row-major with leading dimension ldb)
// ---------------------------------------------------------------------------------
template <int TC>
struct SRGen {
  typedef typename CType<TC>::T T;
  static const bool kHasAbsorbCheck = true;
  int mul, add, accum;
  int tv, tx, ty;
  T neutral_v, absorb_v;
  bool has_absorb;
  const void* nz;
  const void* x;
  void* y;
  int64_t ldb, ldc;
  int layout;

  __device__ __forceinline__ T neutral() const { return neutral_v; }
  __device__ __forceinline__ bool is_absorb(T a) const { return has_absorb && a == absorb_v; }
  __device__ __forceinline__ int64_t bidx(int32_t col1, int64_t j) const {
    return layout == GG_COL_MAJOR ? (int64_t)(col1 - 1) + j * ldb : (int64_t)(col1 - 1) * ldb + j;
  }
  __device__ __forceinline__ int64_t cidx(int64_t row0, int64_t j) const {
    return layout == GG_COL_MAJOR ? row0 + j * ldc : row0 * ldc + j;
  }
  // mul(A[k], B[col, j], row, col, col, j+1); row1 is the 1-based row
  __device__ __forceinline__ T mulk(int64_t k, int32_t col1, int64_t row1, int64_t j = 0) const {
    Raw a = load_raw(nz, tv, k);
    Raw b = load_raw(x, tx, bidx(col1, j));
    return apply_op<TC>(mul, raw_to<TC>(a, tv), raw_to<TC>(b, tx), b, tx, row1, col1, col1, j + 1);
  }
  __device__ __forceinline__ T addv(T acc, T v) const {
    Raw z;
    z.i = 0;
    z.d = 0;
    return apply_op<TC>(add, acc, v, z, TC, 0, 0, 0, 0);
  }
  // SpMV epilogue: accum(c[row], acc, row, 1, row, 1)
  __device__ __forceinline__ void write(int64_t row0, T acc) const {
    accum_store<TC>(y, ty, row0, acc, accum, row0 + 1, 1, row0 + 1, 1);
  }
  // SpMM epilogue: accum(C[row, j], acc, row, j, row, j)
  __device__ __forceinline__ void write_mm(int64_t row0, int64_t j, T acc) const {
    accum_store<TC>(y, ty, cidx(row0, j), acc, accum, row0 + 1, j + 1, row0 + 1, j + 1);
  }
};

// ---------------------------------------------------------------------------------
// streaming loads: read-once matrix data bypasses L1 (keeps L1 for the gathered
// dense operand) and asks L2 for 256-byte prefetch
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int32_t ld_stream(const int32_t* p) {
  int32_t r;
  asm("ld.global.nc.L1::no_allocate.L2::256B.s32 %0, [%1];" : "=r"(r) : "l"(p));
  return r;
}
__device__ __forceinline__ float ld_stream(const float* p) {
  float r;
  asm("ld.global.nc.L1::no_allocate.L2::256B.f32 %0, [%1];" : "=f"(r) : "l"(p));
  return r;
}
__device__ __forceinline__ int4 ld_stream4(const int32_t* p) {
  int4 r;
  asm("ld.global.nc.L1::no_allocate.L2::256B.v4.s32 {%0,%1,%2,%3}, [%4];"
      : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
      : "l"(p));
  return r;
}
__device__ __forceinline__ float4 ld_stream4(const float* p) {
  float4 r;
  asm("ld.global.nc.L1::no_allocate.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4];"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
      : "l"(p));
  return r;
}

// L2 residency hints (createpolicy + .L2::cache_hint): the matrix stream is marked
// evict-first and the gathered dense operand evict-last, so the operand stays in L2
// while gigabytes of matrix data flow through it
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_evict_last() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ int32_t ld_stream_p(const int32_t* p, uint64_t pol) {
  int32_t r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.s32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ float ld_stream_p(const float* p, uint64_t pol) {
  float r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.f32 %0, [%1], %2;" : "=f"(r) : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ int4 ld_stream4_p(const int32_t* p, uint64_t pol) {
  int4 r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.v4.s32 {%0,%1,%2,%3}, [%4], %5;"
      : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
      : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ float4 ld_stream4_p(const float* p, uint64_t pol) {
  float4 r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
      : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ float ld_keep(const float* p, uint64_t pol) {
  float r;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(r) : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ float4 ld_keep4(const float* p, uint64_t pol) {
  float4 r;
  asm("ld.global.nc.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
      : "l"(p), "l"(pol));
  return r;
}

__device__ __forceinline__ void st_hint4(float* p, const float4& v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1,%2,%3,%4}, %5;" ::"l"(p), "f"(v.x),
               "f"(v.y), "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}

// ---------------------------------------------------------------------------------
// (GPUGraphs_mul, GPUGraphs_add, GPUGraphs_second) on Float32: the headline SpMV.
// The early exit at +Inf follows monoid_absorb(Float32, GPUGraphs_add) (algebra.jl:45).
// ---------------------------------------------------------------------------------
struct SRPlusTimesF32 {
  typedef float T;
  static const bool kHasAbsorbCheck = true;
  const float* __restrict__ nz;
  const float* __restrict__ x;
  float* __restrict__ y;
  __device__ __forceinline__ T neutral() const { return 0.0f; }
  __device__ __forceinline__ bool is_absorb(T a) const { return a == __int_as_float(0x7f800000); }
  __device__ __forceinline__ T mulk(int64_t k, int32_t col1, int64_t, int64_t = 0) const {
    return __fmul_rn(ld_stream(nz + k), __ldg(x + (col1 - 1)));
  }
  __device__ __forceinline__ T addv(T acc, T v) const { return __fadd_rn(acc, v); }
  __device__ __forceinline__ void write(int64_t row0, T acc) const { __stcs(y + row0, acc); }
  // split steps for the pipelined kernel: stream A, gather x, multiply
  __device__ __forceinline__ float a(int64_t k) const { return ld_stream(nz + k); }
  __device__ __forceinline__ float4 a4(int64_t k) const { return ld_stream4(nz + k); }
  __device__ __forceinline__ float xg(int32_t col1) const { return __ldg(x + (col1 - 1)); }
  __device__ __forceinline__ T mul(float av, float xv) const { return __fmul_rn(av, xv); }
};

}  // namespace gg
