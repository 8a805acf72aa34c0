// gg_tune.cu -- per-matrix autotuner for the plus-times kernels.
//
// The reference fixes its layouts (thread per row on CSR; SELL with a caller-chosen
// slice height and no row sorting, src/storage/SELL.jl:99-181).  Here one call times,
// on the matrix itself, every configuration of a small grid and keeps the fastest:
//  * SpMV (Float32 plus-times on a CSR handle): the CSR row-block kernel with
//    32 / 64 / 128 / 256 rows per block, and SELL-C-sigma copies with C in {8, 16, 32}
//    and sigma in {1, 64, 1024, m} (copies whose padding would exceed half of nnz are
//    not built);
//  * SpMM: the dense-column tile, 32 x {1, 2, 4} columns per warp pass.
// Each configuration is warmed up twice and timed 7 times with CUDA events on the
// context's stream; the median decides.  Results stay exact whatever is chosen: the
// candidates are the library's own kernels, which all fold rows in storage order
// within their work items.
#include <algorithm>
#include <vector>

#include "gg_common.cuh"

namespace gg {

static int time_median(gg_ctx* ctx, double* ms_out, int (*fn)(void*), void* arg) {
  cudaEvent_t e0, e1;
  GG_CUDA(cudaEventCreate(&e0));
  GG_CUDA(cudaEventCreate(&e1));
  int rc = GG_OK;
  for (int i = 0; i < 2 && rc == GG_OK; ++i) rc = fn(arg);
  std::vector<float> t;
  for (int i = 0; i < 7 && rc == GG_OK; ++i) {
    cudaEventRecord(e0, ctx->stream);
    rc = fn(arg);
    cudaEventRecord(e1, ctx->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = cuda_error(cudaGetLastError(), "tune timing");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    t.push_back(ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != GG_OK) return rc;
  std::sort(t.begin(), t.end());
  *ms_out = t[t.size() / 2];
  return GG_OK;
}

struct SpmvArgs {
  gg_ctx* ctx;
  gg_mat* A;
  float* x;
  float* y;
};
static int run_spmv(void* p) {
  SpmvArgs* a = static_cast<SpmvArgs*>(p);
  return gg_spmv(a->ctx, a->A, GG_OP_MUL, GG_OP_ADD, GG_OP_SECOND, a->y, GG_FLOAT32, a->A->m, a->x,
                 GG_FLOAT32, a->A->n, nullptr, 0, 0, 0, 0);
}

struct SpmmArgs {
  gg_ctx* ctx;
  gg_mat* A;
  float* B;
  float* C;
  int64_t k;
};
static int run_spmm(void* p) {
  SpmmArgs* a = static_cast<SpmmArgs*>(p);
  return gg_spmm(a->ctx, a->A, GG_OP_MUL, GG_OP_ADD, GG_OP_SECOND, a->C, GG_FLOAT32, a->A->m, a->k,
                 a->B, GG_FLOAT32, a->A->n, a->k, a->k, GG_ROW_MAJOR, nullptr, 0, 0, 0, 0);
}

// stored entries of SELL-C-sigma for row lengths len (same rule as gg_sell_create)
static int64_t sell_stored(std::vector<int32_t> len, int64_t C, int64_t sigma) {
  const int64_t m = (int64_t)len.size();
  if (C > m) C = m;
  if (sigma > 1)
    for (int64_t w0 = 0; w0 < m; w0 += sigma)
      std::sort(len.begin() + w0, len.begin() + std::min<int64_t>(w0 + sigma, m),
                [](int32_t a, int32_t b) { return a > b; });
  int64_t tot = 0;
  for (int64_t s0 = 0; s0 < m; s0 += C) {
    int32_t mx = 0;
    for (int64_t r = s0; r < std::min<int64_t>(s0 + C, m); ++r) mx = std::max(mx, len[r]);
    tot += (int64_t)mx * C;
  }
  return tot;
}

static void drop_blocks(gg_mat* A) {
  if (!A->blocks) return;
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

static int tune_spmv(gg_ctx* ctx, gg_mat* A, gg_tune_result* out) {
  float *x = nullptr, *y = nullptr;
  GG_CUDA(cudaMalloc((void**)&x, (A->n > 0 ? A->n : 1) * sizeof(float)));
  cudaError_t e = cudaMalloc((void**)&y, (A->m > 0 ? A->m : 1) * sizeof(float));
  if (e != cudaSuccess) {
    cudaFree(x);
    return cuda_error(e, "tune buffers");
  }
  int rc = gg_gen_uniform_f32(ctx, A->n, 12345, x);
  SpmvArgs args{ctx, A, x, y};
  const int saved_kind = A->tuned_spmv;
  if (rc == GG_OK) {
    A->tuned_spmv = 0;
    rc = time_median(ctx, &out->spmv_default_ms, run_spmv, &args);
  }
  double best = out->spmv_default_ms;
  int best_kind = 0, best_rows = 0, best_variant = 0, best_hot = 32768;
  int64_t best_C = 0, best_sigma = 0;
  gg_mat* best_copy = A->sell_copy;  // the built-in choice's copy (if it made one)
  A->sell_copy = nullptr;
  int cand = 1;
  if (rc == GG_OK && A->format == GG_FMT_CSR) {
    // CSR row blocks
    for (int R : {32, 64, 128, 256}) {
      drop_blocks(A);
      A->tuned_spmv = 1;
      A->block_rows = R;
      double ms = 0;
      rc = time_median(ctx, &ms, run_spmv, &args);
      if (rc != GG_OK) break;
      ++cand;
      if (ms < best) {
        best = ms;
        best_kind = 1;
        best_rows = R;
      }
    }
    // column-window tiles (large power-law matrices only)
    if (rc == GG_OK && A->m >= (1 << 16)) {
      A->tuned_spmv = 3;
      double ms = 0;
      rc = time_median(ctx, &ms, run_spmv, &args);
      if (rc == GG_OK && A->winplan && A->winplan->enabled) {
        ++cand;
        if (ms < best) {
          best = ms;
          best_kind = 3;
        }
      }
    }
    // SELL copies
    std::vector<int32_t> rp(A->m + 1), len(A->m);
    if (rc == GG_OK) {
      e = cudaMemcpy(rp.data(), A->rowptr, (A->m + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) rc = cuda_error(e, "tune rowptr");
    }
    for (int64_t r = 0; r < A->m && rc == GG_OK; ++r) len[r] = rp[r + 1] - rp[r];
    for (int64_t C : {8, 16, 32}) {
      for (int64_t sg : {(int64_t)1, (int64_t)64, (int64_t)1024, A->m}) {
        if (rc != GG_OK) break;
        if (sg < 1) continue;
        const int64_t st = sell_stored(len, C, sg);
        if (st > A->nnz + A->nnz / 2 || st > (int64_t)INT32_MAX) continue;
        gg_mat* S = nullptr;
        if (gg_sell_create(ctx, A, C, sg, &S) != GG_OK) continue;  // e.g. out of memory
        A->sell_copy = S;
        A->tuned_spmv = 2;
        bool keep = false;
        // kernels over the copy: register loads with 32768 or 16384 hot x values in
        // shared memory, the bulk-copy staged kernel and register loads with the hub
        // rows from column windows (SELL-32 only)
        const int nvar = C == 32 ? 4 : 2;
        for (int vi = 0; vi < nvar && rc == GG_OK; ++vi) {
          const int variant = vi == 2 ? 1 : (vi == 3 ? 2 : 0);
          const int hc = vi == 1 ? 16384 : 32768;
          S->sell_variant = variant;
          S->hot_cols = hc;
          double ms = 0;
          rc = time_median(ctx, &ms, run_spmv, &args);
          if (rc != GG_OK) break;
          ++cand;
          if (ms < best) {
            best = ms;
            best_kind = 2;
            best_C = C;
            best_sigma = sg;
            best_variant = variant;
            best_hot = hc;
            keep = true;
          }
        }
        A->sell_copy = nullptr;
        if (rc != GG_OK) {
          gg_mat_destroy(S);
          break;
        }
        if (keep) {
          if (best_copy) gg_mat_destroy(best_copy);
          S->sell_variant = best_variant;
          S->hot_cols = best_hot;
          best_copy = S;
        } else {
          gg_mat_destroy(S);
        }
      }
    }
  }
  // apply the winner
  drop_blocks(A);
  if (rc != GG_OK) {
    A->tuned_spmv = saved_kind;
    A->block_rows = 0;
    A->sell_copy = best_copy;
  } else if (best_kind == 0) {
    A->tuned_spmv = 0;
    A->block_rows = 0;
    A->sell_copy = best_copy;
    const gg_mat* L = A->format == GG_FMT_SELL ? A : best_copy;  // the layout that ran
    out->spmv_kernel = L ? 2 : 1;
    if (L) {
      out->slice_size = L->slice_size;
      out->sigma = L->sigma;
      out->sell_variant = L->sell_variant;
      out->hot_cols = L->hot_cols > 0 ? L->hot_cols : 32768;
    } else {
      out->block_rows = kBlockRows;
    }
  } else if (best_kind == 3) {
    A->tuned_spmv = 3;
    A->block_rows = 0;
    if (best_copy) gg_mat_destroy(best_copy);
    A->sell_copy = nullptr;
    out->spmv_kernel = 3;
  } else if (best_kind == 1) {
    A->tuned_spmv = 1;
    A->block_rows = best_rows;
    if (best_copy) gg_mat_destroy(best_copy);
    A->sell_copy = nullptr;
    out->spmv_kernel = 1;
    out->block_rows = best_rows;
  } else {
    A->tuned_spmv = 2;
    A->block_rows = 0;
    A->sell_copy = best_copy;
    out->spmv_kernel = 2;
    out->slice_size = best_C;
    out->sigma = best_sigma;
    out->sell_variant = best_variant;
    out->hot_cols = best_hot;
  }
  if (A->tuned_spmv != 3) free_win_plan(A);  // keep the window layout only when chosen
  out->spmv_ms = best;
  out->candidates += cand;
  cudaFree(x);
  cudaFree(y);
  return rc;
}

static int tune_spmm(gg_ctx* ctx, gg_mat* A, int64_t k, gg_tune_result* out) {
  float *B = nullptr, *C = nullptr;
  GG_CUDA(cudaMalloc((void**)&B, (A->n * k > 0 ? A->n * k : 1) * sizeof(float)));
  cudaError_t e = cudaMalloc((void**)&C, (A->m * k > 0 ? A->m * k : 1) * sizeof(float));
  if (e != cudaSuccess) {
    cudaFree(B);
    return cuda_error(e, "tune buffers");
  }
  int rc = gg_gen_uniform_f32(ctx, A->n * k, 54321, B);
  SpmmArgs args{ctx, A, B, C, k};
  double best = 0;
  int best_cpl = 1;
  for (int cpl : {1, 2, 4}) {
    if (rc != GG_OK) break;
    if (cpl > 1 && (k < 32 * cpl || A->format != GG_FMT_CSR)) continue;
    A->mm_cpl = cpl;
    double ms = 0;
    rc = time_median(ctx, &ms, run_spmm, &args);
    if (rc != GG_OK) break;
    out->candidates += 1;
    if (cpl == 1 || ms < best) {
      best = ms;
      best_cpl = cpl;
    }
  }
  A->mm_cpl = best_cpl;
  out->mm_cols_per_lane = best_cpl;
  out->spmm_ms = best;
  cudaFree(B);
  cudaFree(C);
  return rc;
}

}  // namespace gg

using namespace gg;

extern "C" int gg_tune(gg_ctx* ctx, gg_mat* A, int64_t spmm_k, gg_tune_result* out) {
  if (!ctx || !A || !out) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (spmm_k < 0) return set_error(GG_ERR_ARGUMENT, "spmm_k must be >= 0");
  *out = gg_tune_result();
  GG_CUDA(cudaSetDevice(ctx->device));
  if (A->dtype != GG_FLOAT32)
    return set_error(GG_ERR_UNSUPPORTED, "gg_tune times the Float32 plus-times kernels");
  if (A->m == 0 || A->n == 0) return GG_OK;
  GG_CHECK(tune_spmv(ctx, A, out));
  if (spmm_k > 0) GG_CHECK(tune_spmm(ctx, A, spmm_k, out));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}

extern "C" int gg_spmv_layout(const gg_mat* A) { return A ? A->last_layout : 0; }

extern "C" int gg_tune_apply(gg_ctx* ctx, gg_mat* A, const gg_tune_result* choice) {
  if (!ctx || !A || !choice) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  const int cpl = choice->mm_cols_per_lane;
  if (cpl != 0 && cpl != 1 && cpl != 2 && cpl != 4)
    return set_error(GG_ERR_ARGUMENT, "mm_cols_per_lane must be 1, 2 or 4");
  GG_CUDA(cudaSetDevice(ctx->device));
  if (choice->spmv_kernel == 1) {
    const int R = choice->block_rows;
    if (R < 1 || R > kBlockRows)
      return set_error(GG_ERR_ARGUMENT, "block_rows must be in 1:%d", kBlockRows);
    if (A->format != GG_FMT_CSR) return set_error(GG_ERR_ARGUMENT, "row blocks need a CSR handle");
    drop_blocks(A);
    if (A->sell_copy) gg_mat_destroy(A->sell_copy);
    A->sell_copy = nullptr;
    A->tuned_spmv = 1;
    A->block_rows = R;
  } else if (choice->spmv_kernel == 2 && A->format == GG_FMT_CSR) {
    gg_mat* S = nullptr;
    GG_CHECK(gg_sell_create(ctx, A, choice->slice_size, choice->sigma, &S));
    if (A->sell_copy) gg_mat_destroy(A->sell_copy);
    A->sell_copy = S;
    A->tuned_spmv = 2;
    A->block_rows = 0;
  } else if (choice->spmv_kernel == 3) {
    if (A->format != GG_FMT_CSR) return set_error(GG_ERR_ARGUMENT, "window tiles need a CSR handle");
    if (A->sell_copy) gg_mat_destroy(A->sell_copy);
    A->sell_copy = nullptr;
    A->tuned_spmv = 3;
    A->block_rows = 0;
  } else if (choice->spmv_kernel != 0 && choice->spmv_kernel != 2) {
    return set_error(GG_ERR_ARGUMENT, "spmv_kernel must be 0, 1, 2 or 3");
  }
  if (cpl) A->mm_cpl = cpl;
  if (choice->sell_variant >= 0 && choice->sell_variant <= 2) {
    A->sell_variant = choice->sell_variant;
    if (A->sell_copy) A->sell_copy->sell_variant = choice->sell_variant;
  }
  if (choice->hot_cols > 0) {
    if (choice->hot_cols > 53248) return set_error(GG_ERR_ARGUMENT, "hot_cols must be at most 53248");
    A->hot_cols = choice->hot_cols;
    if (A->sell_copy) A->sell_copy->hot_cols = choice->hot_cols;
  }
  return GG_OK;
}
