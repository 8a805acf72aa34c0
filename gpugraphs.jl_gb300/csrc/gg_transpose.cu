// gg_transpose.cu -- semiring SpMV with the transpose of a CSR handle (y = A' x).
//
// This is the semiring-correct form of the reference's CSC SpMV (src/spmv/CSC.jl:2-61,
// marked "not properly supported yet" there: it adds with an atomic += whatever the
// semiring).  A CSC matrix B is the CSR storage of B' (same colptr / rowval / nzval),
// so B x = (CSR of B')' x: a caller wraps B's arrays in a CSR handle and asks for the
// transposed product.  The first call builds the CSR storage of A' on the handle:
// entries are ordered by (column, position in A) with a stable radix sort of the
// column ids, so each row of A' lists its entries by ascending row of A, and the
// values are gathered once.  Every later call is a plain SpMV of that copy through the
// same kernels and rules as gg_spmv (storage-order folds, absorb early exit, masks,
// ranges, the first-hit any), i.e.
//     y[j] = accum(y[j], add over rows i of A with an entry in column j, ascending, of
//                        mul(A[i, j], x[i], j, i, i, 1)).
// The copy keeps the values the handle had when it was built (handles are immutable).
#include <cub/device/device_radix_sort.cuh>

#include "gg_semiring.cuh"

namespace gg {

__global__ void k_tp_keys(int64_t nnz, const int32_t* __restrict__ colval, int32_t* keys,
                          int32_t* idx) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x) {
    keys[k] = colval[k] - 1;
    idx[k] = (int32_t)k;
  }
}

__global__ void k_tp_count(int64_t nnz, const int32_t* __restrict__ colval, int32_t* cnt) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + (colval[k] - 1), 1);
}

// entry t of A' (position k = idx[t] in A): its column in A' is the row of A holding k
// (binary search of rowptr), its value A's value k
__global__ void k_tp_fill(int64_t nnz, int64_t m, const int32_t* __restrict__ rowptr,
                          const int32_t* __restrict__ idx, const char* __restrict__ nz, int esz,
                          int32_t* colval_t, char* nz_t) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnz;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = idx[t];
    int64_t lo = 0, hi = m - 1;  // last row r with rowptr[r] - 1 <= k
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (rowptr[mid] - 1 <= k) lo = mid; else hi = mid - 1;
    }
    colval_t[t] = (int32_t)lo + 1;
    for (int b = 0; b < esz; ++b) nz_t[t * esz + b] = nz[(int64_t)k * esz + b];
  }
}

static int tp_grid(gg_ctx* ctx, int64_t work) {
  int64_t g = (work + 255) / 256;
  const int64_t cap = (int64_t)ctx->num_sms * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

static int build_transpose(gg_ctx* ctx, gg_mat* A) {
  if (A->tr_copy) return GG_OK;
  const int64_t m = A->m, n = A->n, nnz = A->nnz;
  const int esz = dtype_size(A->dtype);
  gg_mat* T = new gg_mat();
  T->format = GG_FMT_CSR;
  T->m = n;
  T->n = m;
  T->nnz = nnz;
  T->dtype = A->dtype;
  T->device = ctx->device;
  int32_t *keys = nullptr, *keys2 = nullptr, *idx = nullptr, *idx2 = nullptr, *cnt = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  const int64_t nn = nnz > 0 ? nnz : 1;
  cudaError_t e = cudaMalloc((void**)&T->rowptr, (n + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&T->colval, nn * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&T->nzval, nn * esz);
  if (e == cudaSuccess) e = cudaMalloc((void**)&cnt, (n > 0 ? n : 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, (n > 0 ? n : 1) * sizeof(int32_t), ctx->stream);
  if (e == cudaSuccess && nnz > 0) {
    k_tp_count<<<tp_grid(ctx, nnz), 256, 0, ctx->stream>>>(nnz, A->colval, cnt);
    e = cudaGetLastError();
  }
  int rc = GG_OK;
  if (e == cudaSuccess) rc = scan_counts(ctx, cnt, n, T->rowptr, 1);
  if (e == cudaSuccess && rc == GG_OK && nnz > 0) {
    e = cudaMalloc((void**)&keys, nnz * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&keys2, nnz * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&idx, nnz * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&idx2, nnz * sizeof(int32_t));
    if (e == cudaSuccess) {
      k_tp_keys<<<tp_grid(ctx, nnz), 256, 0, ctx->stream>>>(nnz, A->colval, keys, idx);
      e = cudaGetLastError();
    }
    int end_bit = 1;
    while (end_bit < 31 && ((int64_t)1 << end_bit) < n) ++end_bit;
    if (e == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, idx, idx2, nnz, 0,
                                          end_bit, ctx->stream);
    if (e == cudaSuccess) e = cudaMalloc(&tmp, tmp_bytes > 0 ? tmp_bytes : 1);
    // LSD radix sort is stable: equal columns keep ascending positions, i.e. rows
    if (e == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, idx, idx2, nnz, 0, end_bit,
                                          ctx->stream);
    if (e == cudaSuccess) {
      k_tp_fill<<<tp_grid(ctx, nnz), 256, 0, ctx->stream>>>(
          nnz, m, A->rowptr, idx2, static_cast<const char*>(A->nzval), esz, T->colval,
          static_cast<char*>(T->nzval));
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(keys);
  cudaFree(keys2);
  cudaFree(idx);
  cudaFree(idx2);
  cudaFree(tmp);
  cudaFree(cnt);
  if (e != cudaSuccess || rc != GG_OK) {
    gg_mat_destroy(T);
    return rc != GG_OK ? rc : cuda_error(e, "transpose");
  }
  A->tr_copy = T;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_spmv_t(gg_ctx* ctx, const gg_mat* A_, int mul, int add, int accum, void* y, int y_dtype,
              int64_t y_len, const void* x, int x_dtype, int64_t x_len, const void* mask,
              int mask_dtype, int64_t mask_len, int64_t range_lo, int64_t range_hi) {
  if (!ctx || !A_) return set_error(GG_ERR_ARGUMENT, "ctx / A is NULL");
  gg_mat* A = const_cast<gg_mat*>(A_);
  if (A->format != GG_FMT_CSR)
    return set_error(GG_ERR_UNSUPPORTED, "the transposed SpMV takes a CSR handle");
  // the dimension checks of gpu_spmv! for the CSC matrix A' (src/spmv/CSC.jl:40-45)
  if (A->m != x_len) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  if (y_len != A->n) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  int tc = 0;
  GG_CHECK(check_semiring(A->dtype, x_dtype, y_dtype, mul, add, accum, &tc));
  if (mask) {
    if (!dtype_valid(mask_dtype)) return set_error(GG_ERR_ARGUMENT, "unknown mask element type");
    if (mask_len != A->n)
      return set_error(GG_ERR_DIMENSION, "Mask length must be equal to the number of rows in A");
  }
  if (range_lo != 0 && range_lo <= range_hi && (range_lo < 1 || range_hi > A->n))
    return set_error(GG_ERR_BOUNDS, "range %lld:%lld outside 1:%lld", (long long)range_lo,
                     (long long)range_hi, (long long)A->n);
  if ((A->n > 0 && !y) || (A->m > 0 && !x)) return set_error(GG_ERR_ARGUMENT, "NULL vector");
  if (range_lo != 0 && range_lo > range_hi) return GG_OK;
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_CHECK(build_transpose(ctx, A));
  return spmv_dispatch(ctx, A->tr_copy, tc, mul, add, accum, y, y_dtype, x, x_dtype, mask,
                       mask_dtype, range_lo, range_hi);
}

}  // extern "C"
