// gg_spmv_tma.cu -- plus-times Float32 SpMV over the sorted, relabelled SELL-32 copy
// with the matrix stream staged into shared memory by the bulk-copy (TMA) engine.
//
// Why: in the register-load kernel (k_sell_hot32) the L1/TEX unit is the busiest
// unit -- every scattered 4-byte gather of x costs one L1 tag cycle per distinct
// line, and the coalesced column / value loads of the matrix add a third of that
// work.  Here the column and value words of each work item are copied HBM -> shared
// memory with cp.async.bulk (1-D bulk copies, completion counted on an mbarrier), so
// the L1 pipeline only sees the cold gathers of x; the hot part of x (the most
// frequent relabelled columns) is read from shared memory as before.
//
// Layout of dynamic shared memory: hot x values | per warp, kTStages stage buffers
// of kTCols slice columns (column words, then value words, 512 bytes each) | one
// mbarrier per stage buffer.  Each warp is its own producer: lane 0 keeps up to
// kTStages stages in flight along the warp's sequence of work items (the same
// items, in the same order, as k_sell_hot32), refilling a buffer as soon as the warp
// has read it.  Folding order and results are identical to k_sell_hot32.
//
// Measured on GB300 (R-MAT scale 22): 0.64 ms against 0.32 ms for k_sell_hot32 --
// 512-byte bulk copies per stage and one wait per 4 columns cost more than the L1
// work they remove.  It stays available as an autotuner candidate (sell_variant 1).
//
// Every wait on an mbarrier is bounded: after `polls` polls (the context's limit) the
// kernel records a timeout in `err`, waits for the copies it issued (bounded by the
// built-in kTWaitPolls, whatever the context's limit, so that none is left in flight
// when the CTA ends), and returns.
#include "gg_semiring.cuh"
#include "gg_tma.cuh"

namespace gg {

static const int kTW = 32;                 // warps per CTA
static const int kTStages = 4;             // stage buffers per warp
static const int kTCols = 4;               // slice columns per stage
static const int kTStageWords = kTCols * 32;
static const int kTHot = 22528;            // hot x values held in shared memory (88 KB)
static const unsigned kTWaitPolls = 1u << 22;

static const size_t kTSmemHot = (size_t)kTHot * 4;
static const size_t kTSmemStages = (size_t)kTW * kTStages * kTStageWords * 8;
static const size_t kTSmemBars = (size_t)kTW * kTStages * 8;
static const size_t kTSmem = kTSmemHot + kTSmemStages + kTSmemBars;

// columns of a work item (groups: the sum of their 4-bit slice widths)
__device__ __forceinline__ int item_cols(const int4& d) {
  if (d.z >= 0) return d.z;
  int t = 0;
  for (int s = 0; s < -d.z; ++s) t += ((uint32_t)d.w >> (4 * s)) & 15u;
  return t;
}

struct TmaProducer {
  int64_t it;   // work item of the next stage
  int32_t col;  // its first column
  int4 d;
  int cols;
  int64_t issued;
};

__global__ void __launch_bounds__(kTW * 32, 1)
    k_sell_tma32(const float* __restrict__ nz, const float* __restrict__ xr, float* __restrict__ y,
                 const int32_t* __restrict__ colval, const int32_t* __restrict__ perm, int64_t m,
                 const int4* __restrict__ pitems, int64_t nitems, float* partials, int hot,
                 unsigned* err, unsigned polls) {
  extern __shared__ __align__(128) unsigned char smem[];
  float* sx = reinterpret_cast<float*>(smem);
  int32_t* sbuf = reinterpret_cast<int32_t*>(smem + kTSmemHot);
  uint64_t* sbar = reinterpret_cast<uint64_t*>(smem + kTSmemHot + kTSmemStages);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < hot; i += blockDim.x) sx[i] = __ldg(xr + i);
  int32_t* wbuf = sbuf + (size_t)warp * kTStages * kTStageWords * 2;  // [stage][cols | vals]
  const uint32_t wbar = smem_u32(sbar + warp * kTStages);
  if (lane == 0)
    for (int s = 0; s < kTStages; ++s) mbar_init(wbar + 8 * s, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();

  const int64_t gw = (int64_t)blockIdx.x * kTW + warp;
  const int64_t nw = (int64_t)gridDim.x * kTW;
  TmaProducer pr;
  pr.it = gw;
  pr.col = 0;
  pr.d = gw < nitems ? __ldg(pitems + gw) : make_int4(0, 0, 0, 0);
  pr.cols = gw < nitems ? item_cols(pr.d) : 0;
  pr.issued = 0;
  // issue the next stage of the warp's item sequence (all lanes track the iterator,
  // lane 0 issues the copies); false when the sequence is exhausted
  auto issue_next = [&]() -> bool {
    while (pr.it < nitems) {
      if (pr.col < pr.cols) {
        const int nc = pr.cols - pr.col < kTCols ? pr.cols - pr.col : kTCols;
        const int slot = (int)(pr.issued % kTStages);
        if (lane == 0) {
          const uint32_t bytes = (uint32_t)nc * 32 * 4;
          const uint32_t bar = wbar + 8 * slot;
          int32_t* dcol = wbuf + (size_t)slot * kTStageWords * 2;
          const int64_t pos = (int64_t)pr.d.x + (int64_t)pr.col * 32;
          mbar_expect_tx(bar, 2 * bytes);
          bulk_g2s(smem_u32(dcol), colval + pos, bytes, bar);
          bulk_g2s(smem_u32(dcol + kTStageWords), nz + pos, bytes, bar);
        }
        pr.col += kTCols;
        ++pr.issued;
        return true;
      }
      pr.it += nw;
      pr.col = 0;
      if (pr.it < nitems) {
        pr.d = __ldg(pitems + pr.it);
        pr.cols = item_cols(pr.d);
      }
    }
    return false;
  };
  for (int s = 0; s < kTStages; ++s)
    if (!issue_next()) break;

  int64_t consumed = 0;
  bool failed = false;
  // wait for stage `consumed`, bounded; the warp agrees on the outcome
  auto wait_stage = [&]() -> bool {
    const int slot = (int)(consumed % kTStages);
    const uint32_t parity = (uint32_t)((consumed / kTStages) & 1);
    unsigned ok = 0;
    if (lane == 0) {
      for (unsigned p = 0; p < polls; ++p)
        if (mbar_try_wait(wbar + 8 * slot, parity)) {
          ok = 1;
          break;
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    return ok != 0;
  };
  // after the warp has read stage `consumed` into registers: refill its buffer
  auto release_stage = [&]() {
    __syncwarp();
    ++consumed;
    if (lane == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    issue_next();
  };

  for (int64_t it = gw; it < nitems && !failed; it += nw) {
    const int4 d = __ldg(pitems + it);
    if (d.z < 0) {
      // group of narrow slices: all its (<= 8) columns, then a fold per slice
      const int ns = -d.z;
      const uint32_t widths = (uint32_t)d.w;
      const int total = item_cols(d);
      int32_t c[2 * kTCols];
      float a[2 * kTCols];
#pragma unroll
      for (int u = 0; u < 2 * kTCols; ++u) {
        c[u] = -1;
        a[u] = 0.0f;
      }
      for (int st = 0; st * kTCols < total; ++st) {
        if (!wait_stage()) {
          failed = true;
          break;
        }
        const int32_t* b = wbuf + (size_t)(consumed % kTStages) * kTStageWords * 2;
#pragma unroll
        for (int u = 0; u < kTCols; ++u) {
          if (st * kTCols + u < total) {
            // st is 0 or 1 (a group holds at most 8 columns)
            if (st == 0) {
              c[u] = b[u * 32 + lane];
              a[u] = __int_as_float(b[kTStageWords + u * 32 + lane]);
            } else {
              c[kTCols + u] = b[u * 32 + lane];
              a[kTCols + u] = __int_as_float(b[kTStageWords + u * 32 + lane]);
            }
          }
        }
        release_stage();
      }
      if (failed) break;
      float p[2 * kTCols];
#pragma unroll
      for (int u = 0; u < 2 * kTCols; ++u) {
        const int32_t col = c[u];
        float xv = 0.0f;
        if (col > 0) xv = col <= hot ? sx[col - 1] : __ldg(xr + (col - 1));
        p[u] = __fmul_rn(a[u], xv);
      }
      int u0 = 0;
      for (int t = 0; t < ns; ++t) {
        const int w = (int)((widths >> (4 * t)) & 15u);
        float acc = 0.0f;
#pragma unroll
        for (int u = 0; u < 2 * kTCols; ++u)
          if (u >= u0 && u < u0 + w) acc = __fadd_rn(acc, p[u]);
        u0 += w;
        const int64_t srow = (int64_t)d.y + t * 32 + lane;
        if (srow < m) {
          const int32_t r1 = perm ? __ldg(perm + srow) : (int32_t)(srow + 1);
          __stcs(y + (r1 - 1), acc);
        }
      }
      continue;
    }
    // chunk of one wide slice: stages of kTCols columns folded in column order;
    // padding columns (-1) add +0.0
    const int64_t srow = (int64_t)d.y + lane;
    const bool live = srow < m;
    const int32_t r1 = (live && perm) ? __ldg(perm + srow) : (int32_t)(srow + 1);
    float acc = 0.0f;
    for (int32_t j = 0; j < d.z; j += kTCols) {
      if (!wait_stage()) {
        failed = true;
        break;
      }
      const int32_t* b = wbuf + (size_t)(consumed % kTStages) * kTStageWords * 2;
      int32_t c[kTCols];
      float a[kTCols];
#pragma unroll
      for (int u = 0; u < kTCols; ++u) {
        const bool in = j + u < d.z;
        c[u] = in ? b[u * 32 + lane] : -1;
        a[u] = in ? __int_as_float(b[kTStageWords + u * 32 + lane]) : 0.0f;
      }
      release_stage();
      float p[kTCols];
#pragma unroll
      for (int u = 0; u < kTCols; ++u) {
        const int32_t col = c[u];
        float xv = 0.0f;
        if (col > 0) xv = col <= hot ? sx[col - 1] : __ldg(xr + (col - 1));
        p[u] = __fmul_rn(a[u], xv);
      }
#pragma unroll
      for (int u = 0; u < kTCols; ++u) acc = __fadd_rn(acc, p[u]);
    }
    if (failed) break;
    if (!live) continue;
    if (d.w < 0) __stcs(y + (r1 - 1), acc);
    else partials[(int64_t)d.w * 32 + lane] = acc;
  }
  if (failed) {
    // record the timeout, then let the copies this warp issued land (bounded)
    if (lane == 0) {
      if (err) atomicExch(err, 1u);
      for (int64_t k = consumed; k < pr.issued; ++k) {
        const int slot = (int)(k % kTStages);
        const uint32_t parity = (uint32_t)((k / kTStages) & 1);
        for (unsigned p = 0; p < kTWaitPolls; ++p)
          if (mbar_try_wait(wbar + 8 * slot, parity)) break;
      }
    }
    __syncwarp();
  }
}

int launch_sell_tma(gg_ctx* ctx, gg_mat* A, const float* nzv, const float* xr, float* y,
                    const int32_t* colval) {
  SellPlan* P = A->sellplan;
  const int hot = (int)(A->n < kTHot ? A->n : kTHot);
  static bool attr_set[64] = {false};
  if (ctx->device < 64 && !attr_set[ctx->device]) {
    GG_CUDA(cudaFuncSetAttribute(k_sell_tma32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTSmem));
    attr_set[ctx->device] = true;
  }
  if (P->npitems > 0) {
    const int tr = trace_main_begin(ctx);
    k_sell_tma32<<<ctx->num_sms, kTW * 32, kTSmem, ctx->stream>>>(
        nzv, xr, y, colval, A->sigma > 1 ? A->perm : nullptr, A->m, P->pitems, P->npitems,
        static_cast<float*>(P->partials), hot, ctx->d_err, copy_polls(ctx));
    trace_main_end(ctx, tr);
    trace_count(ctx, 1);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg
