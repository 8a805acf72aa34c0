// gg_ewise.cu -- element-wise, apply and reduce over dense device vectors with the
// operators of src/algebra.jl.
//
// The reference's e-wise and map/reduce files (src/e_wise_ops.jl, src/map_and_reduce.jl)
// are empty; its algorithms do this work with Julia broadcasts between SpMV calls
// (bfs.jl:60-70, shortest_path.jl:72-79).  These entry points give those steps one
// kernel each, with Julia's scalar semantics (wrapping integers, Float32 rounded once
// per operation, NaN-propagating min / max):
//   ewise:  z[i] = op(x[i], y[i], i, 1, i, 1)   computed in promote_type(x, y)
//   apply:  z[i] = op(x[i], s, i, 1, i, 1)      or op(s, x[i], ...) with s bound first
//   reduce: add over x with the monoid's neutral element as the initial value
// ewise / apply skip the entries where a mask is zero.  reduce folds in one fixed
// order, independent of the GPU: chunks of kRedChunk consecutive values, each chunk
// folded by one 256-thread block (thread t adds values t, t + 256, ... left to right,
// then the 32 lanes of each warp combine by an xor butterfly, lane l taking
// add(v[l], v[l ^ o]) for o = 16, 8, 4, 2, 1, then warp 0 combines the 8 warp totals
// the same way), and the chunk totals are reduced again by the same kernel until one
// value is left.  Exact monoids (min, max, or, and, any, integer sums) give the same
// value in any order; Float32 / Float64 sums and products give this order's value.
#include "gg_semiring.cuh"

namespace gg {

static const int kRedThreads = 256;
static const int kRedPerThread = 32;
static const int kRedChunk = kRedThreads * kRedPerThread;  // 8192 values per block

static int ew_grid(gg_ctx* ctx, int64_t n) {
  int64_t g = (n + 255) / 256;
  const int64_t cap = (int64_t)ctx->num_sms * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

template <int TC>
__global__ void k_ewise(int op, void* z, int tz, const void* __restrict__ x, int tx,
                        const void* __restrict__ y, int ty, int64_t n, const void* __restrict__ mask,
                        int tmask, int64_t ibase) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (mask && raw_is_zero(load_raw(mask, tmask, i), tmask)) continue;
    const Raw a = load_raw(x, tx, i), b = load_raw(y, ty, i);
    const int64_t r1 = ibase + i + 1;  // the entry's 1-based index for index operators
    const typename CType<TC>::T v =
        apply_op<TC>(op, raw_to<TC>(a, tx), raw_to<TC>(b, ty), b, ty, r1, 1, r1, 1);
    store_as<TC>(z, tz, i, v);
  }
}

// same (non-Bool) element type everywhere, no mask, 16-byte aligned: 16 bytes of each
// operand per load (kV values), two vectors per thread in flight; the tail [nv * kV, n)
// is left to k_ewise
template <int TC>
__global__ void k_ewise_vec(int op, void* z, const void* __restrict__ x,
                            const void* __restrict__ y, int64_t nv) {
  typedef typename CType<TC>::T T;
  const int kV = 16 / sizeof(T);
  const uint4* xv = static_cast<const uint4*>(x);
  const uint4* yv = static_cast<const uint4*>(y);
  uint4* zv = static_cast<uint4*>(z);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += 2 * stride) {
    const bool two = v + stride < nv;
    uint4 a0 = __ldcs(xv + v), b0 = __ldcs(yv + v), a1 = a0, b1 = b0;
    if (two) {
      a1 = __ldcs(xv + v + stride);
      b1 = __ldcs(yv + v + stride);
    }
    const T* pa0 = reinterpret_cast<const T*>(&a0);
    const T* pb0 = reinterpret_cast<const T*>(&b0);
    const T* pa1 = reinterpret_cast<const T*>(&a1);
    const T* pb1 = reinterpret_cast<const T*>(&b1);
    uint4 r0, r1;
    T* q0 = reinterpret_cast<T*>(&r0);
    T* q1 = reinterpret_cast<T*>(&r1);
#pragma unroll
    for (int e = 0; e < kV; ++e) {
      const int64_t i0 = v * kV + e, i1 = (v + stride) * kV + e;
      Raw b;
      b.d = 0;
      b.i = 0;
      if (dtype_is_float(TC)) b.d = static_cast<double>(pb0[e]); else b.i = static_cast<int64_t>(pb0[e]);
      q0[e] = apply_op<TC>(op, pa0[e], pb0[e], b, TC, i0 + 1, 1, i0 + 1, 1);
      if (dtype_is_float(TC)) b.d = static_cast<double>(pb1[e]); else b.i = static_cast<int64_t>(pb1[e]);
      q1[e] = apply_op<TC>(op, pa1[e], pb1[e], b, TC, i1 + 1, 1, i1 + 1, 1);
    }
    __stcs(zv + v, r0);
    if (two) __stcs(zv + v + stride, r1);
  }
}

// s is the bound scalar, already read in its own type ts
template <int TC>
__global__ void k_apply(int op, void* z, int tz, const void* __restrict__ x, int tx, Raw s,
                        int ts, int s_first, int64_t n, const void* __restrict__ mask, int tmask) {
  typedef typename CType<TC>::T T;
  const T sc = raw_to<TC>(s, ts);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (mask && raw_is_zero(load_raw(mask, tmask, i), tmask)) continue;
    const Raw a = load_raw(x, tx, i);
    const T v = s_first ? apply_op<TC>(op, sc, raw_to<TC>(a, tx), a, tx, i + 1, 1, i + 1, 1)
                        : apply_op<TC>(op, raw_to<TC>(a, tx), sc, s, ts, i + 1, 1, i + 1, 1);
    store_as<TC>(z, tz, i, v);
  }
}

template <typename T> __device__ __forceinline__ T red_xor(T v, int o) {
  return __shfl_xor_sync(0xffffffffu, v, o);
}
template <> __device__ __forceinline__ uint8_t red_xor<uint8_t>(uint8_t v, int o) {
  return static_cast<uint8_t>(__shfl_xor_sync(0xffffffffu, static_cast<int>(v), o));
}

template <int TC>
__device__ __forceinline__ typename CType<TC>::T red_add(int add, typename CType<TC>::T a,
                                                         typename CType<TC>::T b) {
  Raw z;
  z.i = 0;
  z.d = 0;
  return apply_op<TC>(add, a, b, z, TC, 0, 0, 0, 0);
}

// one block per chunk of kRedChunk values: out[chunk] = the chunk's total
template <int TC>
__global__ void __launch_bounds__(kRedThreads)
    k_reduce(int add, const typename CType<TC>::T* __restrict__ in, int64_t n,
             typename CType<TC>::T* out) {
  typedef typename CType<TC>::T T;
  __shared__ T ws[kRedThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const T neutral = neutral_of<T>(add);
  const int64_t c0 = (int64_t)blockIdx.x * kRedChunk;
  T acc = neutral;
#pragma unroll 8
  for (int u = 0; u < kRedPerThread; ++u) {
    const int64_t i = c0 + threadIdx.x + (int64_t)u * kRedThreads;
    if (i < n) acc = red_add<TC>(add, acc, in[i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = red_add<TC>(add, acc, red_xor<T>(acc, o));
  if (lane == 0) ws[wid] = acc;
  __syncthreads();
  if (wid == 0) {
    T v = lane < kRedThreads / 32 ? ws[lane] : neutral;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = red_add<TC>(add, v, red_xor<T>(v, o));
    if (lane == 0) out[blockIdx.x] = v;
  }
}

template <int TC>
static int ewise_t(gg_ctx* ctx, int op, void* z, int tz, const void* x, int tx, const void* y,
                   int ty, int64_t n, const void* mask, int tmask) {
  typedef typename CType<TC>::T T;
  const int kV = 16 / (int)sizeof(T);
  const bool aligned = ((reinterpret_cast<uintptr_t>(z) | reinterpret_cast<uintptr_t>(x) |
                         reinterpret_cast<uintptr_t>(y)) & 15u) == 0;
  if (TC != GG_BOOL && !mask && tx == TC && ty == TC && tz == TC && aligned && n >= kV) {
    const int64_t nv = n / kV;
    k_ewise_vec<TC><<<ew_grid(ctx, nv), 256, 0, ctx->stream>>>(op, z, x, y, nv);
    GG_CUDA(cudaGetLastError());
    trace_count(ctx, 1);
    const int64_t done = nv * kV;
    if (done == n) return GG_OK;
    // the last n - done values, shifted so that entry i keeps its index
    T* zt = static_cast<T*>(z) + done;
    k_ewise<TC><<<1, 256, 0, ctx->stream>>>(op, zt, tz, static_cast<const T*>(x) + done, tx,
                                            static_cast<const T*>(y) + done, ty, n - done,
                                            nullptr, 0, done);
    GG_CUDA(cudaGetLastError());
    trace_count(ctx, 1);
    return GG_OK;
  }
  k_ewise<TC><<<ew_grid(ctx, n), 256, 0, ctx->stream>>>(op, z, tz, x, tx, y, ty, n, mask, tmask, 0);
  GG_CUDA(cudaGetLastError());
  trace_count(ctx, 1);
  return GG_OK;
}

template <int TC>
static int apply_t(gg_ctx* ctx, int op, void* z, int tz, const void* x, int tx, Raw s, int ts,
                   int s_first, int64_t n, const void* mask, int tmask) {
  k_apply<TC><<<ew_grid(ctx, n), 256, 0, ctx->stream>>>(op, z, tz, x, tx, s, ts, s_first, n, mask,
                                                        tmask);
  GG_CUDA(cudaGetLastError());
  trace_count(ctx, 1);
  return GG_OK;
}

template <int TC>
static int reduce_t(gg_ctx* ctx, int add, const void* x, int64_t n, void* out) {
  typedef typename CType<TC>::T T;
  T result = neutral_of<T>(add);
  if (n > 0) {
    const int64_t c1 = (n + kRedChunk - 1) / kRedChunk;
    const int64_t c2 = (c1 + kRedChunk - 1) / kRedChunk;
    T* buf = nullptr;
    GG_CUDA(cudaMalloc((void**)&buf, (c1 + c2 + 1) * sizeof(T)));
    const T* in = static_cast<const T*>(x);
    T* a = buf;
    T* b = buf + c1;
    int64_t cnt = n;
    cudaError_t e = cudaSuccess;
    int launches = 0;
    // pass p reads `in` and writes its chunk totals to a; the buffers alternate
    while (e == cudaSuccess) {
      const int64_t chunks = (cnt + kRedChunk - 1) / kRedChunk;
      k_reduce<TC><<<(unsigned)chunks, kRedThreads, 0, ctx->stream>>>(add, in, cnt, a);
      e = cudaGetLastError();
      ++launches;
      cnt = chunks;
      in = a;
      if (cnt == 1) break;
      a = (a == buf) ? b : buf;
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&result, in, sizeof(T), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_error(e, "reduce");
    trace_count(ctx, launches);
  }
  *static_cast<T*>(out) = result;
  return GG_OK;
}

static Raw host_raw(const void* p, int t) {
  Raw r;
  r.i = 0;
  r.d = 0.0;
  switch (t) {
    case GG_BOOL: r.i = *static_cast<const uint8_t*>(p) != 0; break;
    case GG_INT32: r.i = *static_cast<const int32_t*>(p); break;
    case GG_INT64: r.i = *static_cast<const int64_t*>(p); break;
    case GG_FLOAT32: r.d = *static_cast<const float*>(p); break;
    default: r.d = *static_cast<const double*>(p); break;
  }
  return r;
}

// type rule of the element-wise calls: compute in promote_type(a, b) (Int32 / Int64 at
// least for the index operators), result type wide enough for it
static int ewise_types(int op, int ta, int tb, int tz, int* tc_out) {
  if (!dtype_valid(ta) || !dtype_valid(tb) || !dtype_valid(tz))
    return set_error(GG_ERR_ARGUMENT, "unknown element type code");
  if (op < GG_OP_FIRST || op > GG_OP_SECONDJ) return set_error(GG_ERR_ARGUMENT, "unknown operator code");
  const int tc = compute_type(ta, tb, op);
  const int tp = ta > tb ? ta : tb;
  if (tz < tc || tz < tp)
    return set_error(GG_ERR_TYPE, "Result type must be able to hold the result of the operation");
  // an (x, x) semiring check gives the operator-defined rule of gg_spmv for op
  int dummy = 0;
  GG_CHECK(check_semiring(tc, tc, tz, op, GG_OP_MIN, GG_OP_SECOND, &dummy));
  *tc_out = tc;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_ewise(gg_ctx* ctx, int op, void* z, int z_dtype, const void* x, int x_dtype,
             const void* y, int y_dtype, int64_t n, const void* mask, int mask_dtype) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  if (n < 0) return set_error(GG_ERR_DIMENSION, "negative length");
  int tc = 0;
  GG_CHECK(ewise_types(op, x_dtype, y_dtype, z_dtype, &tc));
  if (mask && !dtype_valid(mask_dtype)) return set_error(GG_ERR_ARGUMENT, "unknown mask element type");
  if (n == 0) return GG_OK;
  if (!z || !x || !y) return set_error(GG_ERR_ARGUMENT, "NULL vector");
  GG_CUDA(cudaSetDevice(ctx->device));
  switch (tc) {
    case GG_BOOL: return ewise_t<GG_BOOL>(ctx, op, z, z_dtype, x, x_dtype, y, y_dtype, n, mask, mask_dtype);
    case GG_INT32: return ewise_t<GG_INT32>(ctx, op, z, z_dtype, x, x_dtype, y, y_dtype, n, mask, mask_dtype);
    case GG_INT64: return ewise_t<GG_INT64>(ctx, op, z, z_dtype, x, x_dtype, y, y_dtype, n, mask, mask_dtype);
    case GG_FLOAT32: return ewise_t<GG_FLOAT32>(ctx, op, z, z_dtype, x, x_dtype, y, y_dtype, n, mask, mask_dtype);
    default: return ewise_t<GG_FLOAT64>(ctx, op, z, z_dtype, x, x_dtype, y, y_dtype, n, mask, mask_dtype);
  }
}

int gg_apply(gg_ctx* ctx, int op, void* z, int z_dtype, const void* x, int x_dtype,
             const void* s, int s_dtype, int s_first, int64_t n, const void* mask,
             int mask_dtype) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  if (n < 0) return set_error(GG_ERR_DIMENSION, "negative length");
  if (!s) return set_error(GG_ERR_ARGUMENT, "NULL scalar");
  int tc = 0;
  GG_CHECK(s_first ? ewise_types(op, s_dtype, x_dtype, z_dtype, &tc)
                   : ewise_types(op, x_dtype, s_dtype, z_dtype, &tc));
  if (mask && !dtype_valid(mask_dtype)) return set_error(GG_ERR_ARGUMENT, "unknown mask element type");
  if (n == 0) return GG_OK;
  if (!z || !x) return set_error(GG_ERR_ARGUMENT, "NULL vector");
  const Raw sr = host_raw(s, s_dtype);
  GG_CUDA(cudaSetDevice(ctx->device));
  switch (tc) {
    case GG_BOOL: return apply_t<GG_BOOL>(ctx, op, z, z_dtype, x, x_dtype, sr, s_dtype, s_first, n, mask, mask_dtype);
    case GG_INT32: return apply_t<GG_INT32>(ctx, op, z, z_dtype, x, x_dtype, sr, s_dtype, s_first, n, mask, mask_dtype);
    case GG_INT64: return apply_t<GG_INT64>(ctx, op, z, z_dtype, x, x_dtype, sr, s_dtype, s_first, n, mask, mask_dtype);
    case GG_FLOAT32: return apply_t<GG_FLOAT32>(ctx, op, z, z_dtype, x, x_dtype, sr, s_dtype, s_first, n, mask, mask_dtype);
    default: return apply_t<GG_FLOAT64>(ctx, op, z, z_dtype, x, x_dtype, sr, s_dtype, s_first, n, mask, mask_dtype);
  }
}

int gg_reduce(gg_ctx* ctx, int add, const void* x, int x_dtype, int64_t n, void* out) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  if (n < 0) return set_error(GG_ERR_DIMENSION, "negative length");
  if (!out) return set_error(GG_ERR_ARGUMENT, "NULL result");
  if (!dtype_valid(x_dtype)) return set_error(GG_ERR_ARGUMENT, "unknown element type code");
  int tc = 0;
  GG_CHECK(check_semiring(x_dtype, x_dtype, x_dtype, GG_OP_FIRST, add, GG_OP_SECOND, &tc));
  if (n > 0 && !x) return set_error(GG_ERR_ARGUMENT, "NULL vector");
  GG_CUDA(cudaSetDevice(ctx->device));
  switch (x_dtype) {
    case GG_BOOL: return reduce_t<GG_BOOL>(ctx, add, x, n, out);
    case GG_INT32: return reduce_t<GG_INT32>(ctx, add, x, n, out);
    case GG_INT64: return reduce_t<GG_INT64>(ctx, add, x, n, out);
    case GG_FLOAT32: return reduce_t<GG_FLOAT32>(ctx, add, x, n, out);
    default: return reduce_t<GG_FLOAT64>(ctx, add, x, n, out);
  }
}

}  // extern "C"
