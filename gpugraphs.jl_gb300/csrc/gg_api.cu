// gg_api.cu -- context, storage handles and argument checking of libgpugraphs.
//
// Storage follows GPUGraphs.jl exactly: CSR keeps 1-based Int32 rowptr / colval and
// the value array (src/storage/CSR.jl:14-92); SELL keeps slice_ptr (1-based), a
// slice-column-major colval padded with -1 and nzval padded with 0
// (src/storage/SELL.jl:99-181), and, for sigma > 1, the row permutation.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "gg_common.cuh"

namespace gg {

static thread_local std::string g_err;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? GG_ERR_OOM : GG_ERR_CUDA;
  (void)cudaGetLastError();  // clear a sticky-free error so the context stays usable
  return set_error(code, "%s: %s", what, cudaGetErrorString(e));
}

int ensure_scratch(gg_ctx* ctx, size_t bytes) {
  if (ctx->scratch_bytes >= bytes) return GG_OK;
  if (ctx->scratch) {
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
  }
  size_t want = bytes < (1u << 20) ? (1u << 20) : bytes;
  GG_CUDA(cudaMalloc(&ctx->scratch, want));
  ctx->scratch_bytes = want;
  return GG_OK;
}

// ---- semiring validity (same rules as the oracle's check_semiring) ----
static bool is_index_op(int op) {
  return op == GG_OP_FIRSTI || op == GG_OP_FIRSTJ || op == GG_OP_SECONDI || op == GG_OP_SECONDJ;
}
static bool op_valid(int op) { return op >= GG_OP_FIRST && op <= GG_OP_SECONDJ; }
static bool op_defined(int op, int t) {
  switch (op) {
    case GG_OP_ADD: case GG_OP_SAFE_ADD: case GG_OP_MINUS: case GG_OP_RMINUS:
      return t != GG_BOOL;
    case GG_OP_LOR: case GG_OP_LAND: case GG_OP_BOR: case GG_OP_BAND: case GG_OP_BXOR:
      return !dtype_is_float(t);
  }
  return true;
}
static bool has_neutral(int add, int t) {
  switch (add) {
    case GG_OP_ADD: case GG_OP_SAFE_ADD: case GG_OP_ANY: case GG_OP_MUL: case GG_OP_MIN:
    case GG_OP_MAX: return true;
    case GG_OP_BOR: case GG_OP_BAND: return !dtype_is_float(t);
    case GG_OP_LOR: case GG_OP_LAND: return t == GG_BOOL;
  }
  return false;
}

int compute_type(int tv, int tx, int mul) {
  int tc = tv > tx ? tv : tx;
  if ((mul == GG_OP_FIRSTJ || mul == GG_OP_SECONDI) && tc < GG_INT32) tc = GG_INT32;
  if ((mul == GG_OP_FIRSTI || mul == GG_OP_SECONDJ) && tc < GG_INT64) tc = GG_INT64;
  return tc;
}

int check_semiring(int tv, int tx, int ty, int mul, int add, int accum, int* tc_out) {
  if (!dtype_valid(tv) || !dtype_valid(tx) || !dtype_valid(ty))
    return set_error(GG_ERR_ARGUMENT, "unknown element type code");
  if (!op_valid(mul) || !op_valid(add) || !op_valid(accum))
    return set_error(GG_ERR_ARGUMENT, "unknown operator code");
  const int tc = compute_type(tv, tx, mul);
  const int tp = tv > tx ? tv : tx;
  if (ty < tp || ty < tc)
    return set_error(GG_ERR_TYPE, "Result type must be able to hold the result of the multiplication");
  if (!is_index_op(mul) && !op_defined(mul, tc))
    return set_error(GG_ERR_UNSUPPORTED, "mul operator %d has no method for element type %d", mul, tc);
  if (!op_defined(add, tc) || !has_neutral(add, tc))
    return set_error(GG_ERR_UNSUPPORTED, "monoid_neutral not implemented for type %d and operation %d", tc, add);
  if (!is_index_op(accum) && !op_defined(accum, ty))
    return set_error(GG_ERR_UNSUPPORTED, "accum operator %d has no method for element type %d", accum, ty);
  *tc_out = tc;
  return GG_OK;
}

int spmm_dispatch(gg_ctx* ctx, gg_mat* A, int tc, int mul, int add, int accum, void* C, int tcm,
                  int64_t ldc, const void* B, int tb, int64_t ldb, int64_t k, int layout,
                  const void* mask, int tmask, int64_t lo, int64_t hi);

// ---- storage kernels ----
__global__ void k_validate_csr(int64_t m, int64_t n, int64_t nnz, const int32_t* rowptr,
                               const int32_t* colval, unsigned* flags) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned bad = 0;
  if (t0 == 0) {
    if (rowptr[0] != 1) bad |= 1u;
    if ((int64_t)rowptr[m] != nnz + 1) bad |= 1u;
  }
  for (int64_t i = t0; i < m; i += stride)
    if (rowptr[i] > rowptr[i + 1]) bad |= 2u;
  for (int64_t i = t0; i < nnz; i += stride) {
    const int32_t c = colval[i];
    if (c < 1 || (int64_t)c > n) bad |= 4u;
  }
  if (bad) atomicOr(flags, bad);
}

// one thread per stored SELL row: copy its entries into the slice-column-major layout
__global__ void k_sell_fill(int64_t m, int64_t C, const int32_t* rowptr, const int32_t* colval,
                            const char* nzval, int esz, const int32_t* perm,
                            const int32_t* slice_ptr, int32_t* s_colval, char* s_nzval) {
  const int64_t total = ((m + C - 1) / C) * C;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / C, o = t - s * C;
    const int64_t base = (int64_t)slice_ptr[s] - 1;
    const int64_t mx = ((int64_t)slice_ptr[s + 1] - slice_ptr[s]) / C;
    int64_t start = 0, len = 0;
    if (t < m) {
      const int64_t r = (int64_t)perm[t] - 1;
      start = (int64_t)rowptr[r] - 1;
      len = (int64_t)rowptr[r + 1] - rowptr[r];
    }
    for (int64_t j = 0; j < mx; ++j) {
      const int64_t dst = base + j * C + o;
      if (j < len) {
        s_colval[dst] = colval[start + j];
        for (int b = 0; b < esz; ++b) s_nzval[dst * esz + b] = nzval[(start + j) * esz + b];
      } else {
        s_colval[dst] = -1;
        for (int b = 0; b < esz; ++b) s_nzval[dst * esz + b] = 0;
      }
    }
  }
}

__global__ void k_invert_perm(int64_t m, const int32_t* perm, int32_t* iperm) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x)
    iperm[perm[t] - 1] = (int32_t)t;
}

static void free_mat_storage(gg_mat* A);
// everything built from the handle's arrays on first use (plans, copies, analyses)
static void free_derived(gg_mat* A) {
  if (A->blocks) {
    RowBlocks* rb = A->blocks;
    cudaFree(rb->blocks);
    cudaFree(rb->segs);
    cudaFree(rb->long_first_seg);
    cudaFree(rb->long_rows);
    cudaFree(rb->long_count);
    cudaFree(rb->partials);
    delete rb;
    A->blocks = nullptr;
  }
  free_graph_aux(A);
  if (A->sell_copy) {
    free_mat_storage(A->sell_copy);
    delete A->sell_copy;
    A->sell_copy = nullptr;
  }
  if (A->tr_copy) {
    free_mat_storage(A->tr_copy);
    delete A->tr_copy;
    A->tr_copy = nullptr;
  }
  if (A->colperm) {
    cudaFree(A->colperm->colval_r);
    cudaFree(A->colperm->inv);
    cudaFree(A->colperm->xr);
    delete A->colperm;
    A->colperm = nullptr;
  }
  free_win_plan(A);
  free_spv_plan(A);
  if (A->hubplan) {
    cudaFree(A->hubplan->hubs);
    cudaFree(A->hubplan->pieces);
    cudaFree(A->hubplan->acc);
    cudaFree(A->hubplan->mid);
    cudaFree(A->hubplan->order);
    cudaFree(A->hubplan->d_norder);
    delete A->hubplan;
    A->hubplan = nullptr;
  }
  if (A->mmplan) {
    cudaFree(A->mmplan->segs);
    cudaFree(A->mmplan->first);
    cudaFree(A->mmplan->rows);
    cudaFree(A->mmplan->items);
    cudaFree(A->mmplan->short_rows);
    delete A->mmplan;
    A->mmplan = nullptr;
  }
  free_hubwin_plan(A);
  if (A->sellplan) {
    free_sell_plan(A->sellplan);
    A->sellplan = nullptr;
  }
}

static void free_mat_storage(gg_mat* A) {
  cudaFree(A->rowptr);
  cudaFree(A->colval);
  cudaFree(A->nzval);
  cudaFree(A->slice_ptr);
  cudaFree(A->perm);
  cudaFree(A->iperm);
  free_derived(A);
}

static int blocks_for(gg_ctx* ctx, int64_t work) {
  int64_t g = (work + 255) / 256;
  int64_t cap = (int64_t)(ctx->num_sms > 0 ? ctx->num_sms : 132) * 16;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace gg

using namespace gg;

extern "C" {

const char* gg_last_error(void) { return g_err.c_str(); }

const char* gg_version(void) { return "gpugraphs-gb300 0.1 (sm_103a)"; }

int gg_init(int device, gg_ctx** out) {
  if (!out) return set_error(GG_ERR_ARGUMENT, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  GG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev)
    return set_error(GG_ERR_ARGUMENT, "device %d out of range (%d devices)", device, ndev);
  GG_CUDA(cudaSetDevice(device));
  gg_ctx* c = new gg_ctx();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_flags, 64 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_flags, 64 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(unsigned));
  if (e != cudaSuccess) {
    cudaFree(c->d_flags);
    cudaFree(c->d_err);
    delete c;
    return cuda_error(e, "gg_init");
  }
  *out = c;
  return GG_OK;
}

int gg_destroy(gg_ctx* ctx) {
  if (!ctx) return GG_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->scratch);
  cudaFree(ctx->d_flags);
  cudaFreeHost(ctx->h_flags);
  cudaFree(ctx->d_err);
  if (ctx->trace_ev) {
    for (int i = 0; i < 2 * kTraceMax; ++i) cudaEventDestroy(ctx->trace_ev[i]);
    delete[] ctx->trace_ev;
  }
  delete ctx;
  return GG_OK;
}

int gg_trace_begin(gg_ctx* ctx) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  GG_CUDA(cudaSetDevice(ctx->device));
  if (!ctx->trace_ev) {
    ctx->trace_ev = new cudaEvent_t[2 * kTraceMax]();
    for (int i = 0; i < 2 * kTraceMax; ++i) {
      cudaError_t e = cudaEventCreate(&ctx->trace_ev[i]);
      if (e != cudaSuccess) {
        for (int j = 0; j < i; ++j) cudaEventDestroy(ctx->trace_ev[j]);
        delete[] ctx->trace_ev;
        ctx->trace_ev = nullptr;
        return cuda_error(e, "gg_trace_begin");
      }
    }
  }
  ctx->trace_on = true;
  ctx->trace_launches = 0;
  ctx->trace_used = 0;
  return GG_OK;
}

int gg_trace_end(gg_ctx* ctx, int64_t* launches, int64_t* timed, double* timed_ms) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  double tot = 0.0;
  for (int i = 0; i < ctx->trace_used; ++i) {
    float ms = 0.f;
    GG_CUDA(cudaEventElapsedTime(&ms, ctx->trace_ev[2 * i], ctx->trace_ev[2 * i + 1]));
    tot += ms;
  }
  if (launches) *launches = ctx->trace_launches;
  if (timed) *timed = ctx->trace_used;
  if (timed_ms) *timed_ms = tot;
  ctx->trace_on = false;
  return GG_OK;
}

int gg_set_stream(gg_ctx* ctx, void* stream) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  ctx->stream = static_cast<cudaStream_t>(stream);
  return GG_OK;
}

int gg_set_wait_limit(gg_ctx* ctx, uint64_t polls) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  ctx->wait_polls = polls;
  return GG_OK;
}

int gg_stream_sync(gg_ctx* ctx) {
  if (!ctx) return set_error(GG_ERR_ARGUMENT, "ctx is NULL");
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ctx->d_err) {  // a bounded device-side wait ran out since the last check
    unsigned e = 0;
    GG_CUDA(cudaMemcpy(&e, ctx->d_err, sizeof(e), cudaMemcpyDeviceToHost));
    if (e) {
      GG_CUDA(cudaMemset(ctx->d_err, 0, sizeof(unsigned)));
      return set_error(GG_ERR_TIMEOUT, "a device-side wait ran out (results of the calls since the last sync are invalid)");
    }
  }
  return GG_OK;
}

int gg_csr_create(gg_ctx* ctx, int64_t m, int64_t n, int64_t nnz, const int32_t* rowptr,
                  const int32_t* colval, const void* nzval, int dtype, int on_device,
                  gg_mat** out) {
  if (!ctx || !out) return set_error(GG_ERR_ARGUMENT, "ctx / out is NULL");
  *out = nullptr;
  if (m < 0 || n < 0 || nnz < 0) return set_error(GG_ERR_ARGUMENT, "negative size");
  if (nnz > INT32_MAX - 1 || m > INT32_MAX - 1 || n > INT32_MAX)
    return set_error(GG_ERR_ARGUMENT, "sizes exceed the Int32 index range");
  if (!dtype_valid(dtype)) return set_error(GG_ERR_ARGUMENT, "unknown element type %d", dtype);
  if (!rowptr || (nnz > 0 && (!colval || !nzval)))
    return set_error(GG_ERR_ARGUMENT, "NULL array");
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_mat* A = new gg_mat();
  A->format = GG_FMT_CSR;
  A->m = m;
  A->n = n;
  A->nnz = nnz;
  A->dtype = dtype;
  A->device = ctx->device;
  const size_t esz = dtype_size(dtype);
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  cudaError_t e = cudaMalloc((void**)&A->rowptr, (m + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&A->colval, (nnz > 0 ? nnz : 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&A->nzval, (nnz > 0 ? nnz : 1) * esz);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(A->rowptr, rowptr, (m + 1) * sizeof(int32_t), kind, ctx->stream);
  if (e == cudaSuccess && nnz > 0)
    e = cudaMemcpyAsync(A->colval, colval, nnz * sizeof(int32_t), kind, ctx->stream);
  if (e == cudaSuccess && nnz > 0) e = cudaMemcpyAsync(A->nzval, nzval, nnz * esz, kind, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream);
  if (e == cudaSuccess) {
    k_validate_csr<<<blocks_for(ctx, (m > nnz ? m : nnz) + 1), 256, 0, ctx->stream>>>(
        m, n, nnz, A->rowptr, A->colval, ctx->d_flags);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    free_mat_storage(A);
    delete A;
    return cuda_error(e, "gg_csr_create");
  }
  const unsigned bad = ctx->h_flags[0];
  if (bad) {
    free_mat_storage(A);
    delete A;
    if (bad & 4u) return set_error(GG_ERR_ARGUMENT, "colval contains an index out of bounds");
    if (bad & 1u)
      return set_error(GG_ERR_ARGUMENT,
                       "rowptr[1] must be equal to 1 and rowptr[m+1] must be equal to length(colval) + 1");
    return set_error(GG_ERR_ARGUMENT, "rowptr must be non-decreasing");
  }
  *out = A;
  return GG_OK;
}

int gg_sell_create(gg_ctx* ctx, const gg_mat* csr, int64_t slice_size, int64_t sigma,
                   gg_mat** out) {
  if (!ctx || !csr || !out) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (csr->format != GG_FMT_CSR) return set_error(GG_ERR_ARGUMENT, "source must be a CSR matrix");
  if (slice_size < 1) return set_error(GG_ERR_ARGUMENT, "slice_size must be >= 1");
  if (sigma < 1) return set_error(GG_ERR_ARGUMENT, "sigma must be >= 1");
  GG_CUDA(cudaSetDevice(ctx->device));
  const int64_t m = csr->m;
  std::vector<int32_t> rp(m + 1);
  GG_CUDA(cudaMemcpyAsync(rp.data(), csr->rowptr, (m + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  // slice height clamped to m (src/storage/SELL.jl:108)
  const int64_t C = slice_size < m ? slice_size : m;
  const int64_t ns = C > 0 ? (m + C - 1) / C : 0;
  std::vector<int32_t> perm(m);
  std::iota(perm.begin(), perm.end(), 1);
  if (sigma > 1) {
    for (int64_t w0 = 0; w0 < m; w0 += sigma) {
      const int64_t w1 = std::min<int64_t>(w0 + sigma, m);
      std::stable_sort(perm.begin() + w0, perm.begin() + w1, [&](int32_t a, int32_t b) {
        return (rp[a] - rp[a - 1]) > (rp[b] - rp[b - 1]);
      });
    }
  }
  std::vector<int32_t> sp(ns + 1);
  sp[0] = 1;
  int64_t acc = 1;
  for (int64_t s = 0; s < ns; ++s) {
    int64_t mx = 0;
    for (int64_t r = s * C; r < std::min<int64_t>((s + 1) * C, m); ++r)
      mx = std::max<int64_t>(mx, rp[perm[r]] - rp[perm[r] - 1]);
    acc += mx * C;
    if (acc > (int64_t)INT32_MAX - 4096)  // kernels step Int32 positions past the end
      return set_error(GG_ERR_ARGUMENT, "SELL n_stored exceeds the Int32 index range (use a larger sigma)");
    sp[s + 1] = (int32_t)acc;
  }
  gg_mat* S = new gg_mat();
  S->format = GG_FMT_SELL;
  S->m = m;
  S->n = csr->n;
  S->nnz = csr->nnz;
  S->dtype = csr->dtype;
  S->device = ctx->device;
  S->slice_size = C;
  S->nslices = ns;
  S->n_stored = acc - 1;
  S->sigma = sigma;
  const size_t esz = dtype_size(csr->dtype);
  const int64_t nst = S->n_stored;
  cudaError_t e = cudaMalloc((void**)&S->slice_ptr, (ns + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&S->colval, (nst > 0 ? nst : 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&S->nzval, (nst > 0 ? nst : 1) * esz);
  if (e == cudaSuccess) e = cudaMalloc((void**)&S->perm, (m > 0 ? m : 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&S->iperm, (m > 0 ? m : 1) * sizeof(int32_t));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(S->slice_ptr, sp.data(), (ns + 1) * sizeof(int32_t), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess && m > 0)
    e = cudaMemcpyAsync(S->perm, perm.data(), m * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && ns > 0) {
    k_sell_fill<<<blocks_for(ctx, ns * C), 256, 0, ctx->stream>>>(
        m, C, csr->rowptr, csr->colval, static_cast<const char*>(csr->nzval), (int)esz, S->perm,
        S->slice_ptr, S->colval, static_cast<char*>(S->nzval));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && m > 0) {
    k_invert_perm<<<blocks_for(ctx, m), 256, 0, ctx->stream>>>(m, S->perm, S->iperm);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    free_mat_storage(S);
    delete S;
    return cuda_error(e, "gg_sell_create");
  }
  *out = S;
  return GG_OK;
}

int gg_mat_destroy(gg_mat* A) {
  if (!A) return GG_OK;
  cudaSetDevice(A->device);
  free_mat_storage(A);
  delete A;
  return GG_OK;
}

int gg_mat_values_changed(gg_ctx* ctx, gg_mat* A) {
  if (!ctx || !A) return set_error(GG_ERR_ARGUMENT, "ctx / A is NULL");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  free_derived(A);
  return GG_OK;
}

int gg_mat_info(const gg_mat* A, int* format, int64_t* m, int64_t* n, int64_t* nnz, int* dtype,
                int64_t* n_stored, int64_t* slice_size, int64_t* nslices) {
  if (!A) return set_error(GG_ERR_ARGUMENT, "A is NULL");
  if (format) *format = A->format;
  if (m) *m = A->m;
  if (n) *n = A->n;
  if (nnz) *nnz = A->nnz;
  if (dtype) *dtype = A->dtype;
  if (n_stored) *n_stored = A->format == GG_FMT_SELL ? A->n_stored : A->nnz;
  if (slice_size) *slice_size = A->slice_size;
  if (nslices) *nslices = A->nslices;
  return GG_OK;
}

int gg_mat_arrays(const gg_mat* A, void** ptr, void** colval, void** nzval, void** perm) {
  if (!A) return set_error(GG_ERR_ARGUMENT, "A is NULL");
  if (ptr) *ptr = A->format == GG_FMT_CSR ? (void*)A->rowptr : (void*)A->slice_ptr;
  if (colval) *colval = A->colval;
  if (nzval) *nzval = A->nzval;
  if (perm) *perm = A->perm;
  return GG_OK;
}

static int check_rows(const gg_mat* A, const void* mask, int mask_dtype, int64_t mask_len,
                      int64_t range_lo, int64_t range_hi, int dim_code) {
  if (mask) {
    if (!dtype_valid(mask_dtype)) return set_error(GG_ERR_ARGUMENT, "unknown mask element type");
    if (mask_len != A->m)
      return set_error(dim_code, "Mask length must be equal to the number of rows in A");
  }
  if (range_lo != 0 && range_lo <= range_hi && (range_lo < 1 || range_hi > A->m))
    return set_error(dim_code == GG_ERR_ASSERTION ? GG_ERR_ASSERTION : GG_ERR_BOUNDS,
                     "range %lld:%lld outside 1:%lld", (long long)range_lo, (long long)range_hi,
                     (long long)A->m);
  return GG_OK;
}

int gg_spmv(gg_ctx* ctx, const gg_mat* A, int mul, int add, int accum, void* y, int y_dtype,
            int64_t y_len, const void* x, int x_dtype, int64_t x_len, const void* mask,
            int mask_dtype, int64_t mask_len, int64_t range_lo, int64_t range_hi) {
  if (!ctx || !A) return set_error(GG_ERR_ARGUMENT, "ctx / A is NULL");
  // _validate_args order: dimensions, types, mask (src/spmv/CSR.jl:373-407)
  if (A->n != x_len) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  if (y_len != A->m) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  int tc = 0;
  GG_CHECK(check_semiring(A->dtype, x_dtype, y_dtype, mul, add, accum, &tc));
  GG_CHECK(check_rows(A, mask, mask_dtype, mask_len, range_lo, range_hi, GG_ERR_DIMENSION));
  if ((A->m > 0 && !y) || (A->n > 0 && !x)) return set_error(GG_ERR_ARGUMENT, "NULL vector");
  if (range_lo != 0 && range_lo > range_hi) return GG_OK;  // empty range
  GG_CUDA(cudaSetDevice(ctx->device));
  return spmv_dispatch(ctx, const_cast<gg_mat*>(A), tc, mul, add, accum, y, y_dtype, x, x_dtype,
                       mask, mask_dtype, range_lo, range_hi);
}

int gg_spmm(gg_ctx* ctx, const gg_mat* A, int mul, int add, int accum, void* C, int c_dtype,
            int64_t c_rows, int64_t ldc, const void* B, int b_dtype, int64_t b_rows, int64_t ldb,
            int64_t k, int layout, const void* mask, int mask_dtype, int64_t mask_len,
            int64_t range_lo, int64_t range_hi) {
  if (!ctx || !A) return set_error(GG_ERR_ARGUMENT, "ctx / A is NULL");
  // @assert size(A,2) == size(B,1); size(C,1) == size(A,1) (src/spmm/CSR.jl:131-133)
  if (A->n != b_rows) return set_error(GG_ERR_ASSERTION, "size(A, 2) == size(B, 1)");
  if (c_rows != A->m) return set_error(GG_ERR_ASSERTION, "size(C, 1) == size(A, 1)");
  if (k < 0) return set_error(GG_ERR_ASSERTION, "size(C, 2) == size(B, 2)");
  if (layout != GG_COL_MAJOR && layout != GG_ROW_MAJOR)
    return set_error(GG_ERR_ARGUMENT, "unknown layout");
  if (layout == GG_COL_MAJOR ? (ldb < b_rows || ldc < c_rows) : (ldb < k || ldc < k))
    return set_error(GG_ERR_ARGUMENT, "leading dimension too small");
  if (mask && range_lo != 0) return set_error(GG_ERR_ASSERTION, "mask === nothing");
  int tc = 0;
  GG_CHECK(check_semiring(A->dtype, b_dtype, c_dtype, mul, add, accum, &tc));
  GG_CHECK(check_rows(A, mask, mask_dtype, mask_len, range_lo, range_hi, GG_ERR_ASSERTION));
  if (k == 0 || A->m == 0) return GG_OK;
  if (!C || (A->n > 0 && !B)) return set_error(GG_ERR_ARGUMENT, "NULL matrix");
  if (range_lo != 0 && range_lo > range_hi) return GG_OK;
  GG_CUDA(cudaSetDevice(ctx->device));
  return spmm_dispatch(ctx, const_cast<gg_mat*>(A), tc, mul, add, accum, C, c_dtype, ldc, B, b_dtype,
                       ldb, k, layout, mask, mask_dtype, range_lo, range_hi);
}

}  // extern "C"
