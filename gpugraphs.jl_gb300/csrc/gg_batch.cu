// gg_batch.cu -- many BFS / shortest-path sources in one pass over the graph.
//
// The reference's only batched entry point is shortest_path(A_T, sources)
// (src/algorithms/shortest_path.jl:88-161): a min-plus SpMM per round over an
// n x S distance matrix.  Here (kernels in gg_msearch.cuh):
//  * gg_bfs_levels_batch: up to 256 sources per group as bits of W <= 8 words per
//    vertex, one bottom-up level per launch; column q equals
//    bfs_distances(A_T, sources[q]).
//  * gg_sssp_batch: 32 sources per group, one relaxation round per launch; column q
//    equals shortest_path(A_T, sources[q]).
#include <algorithm>
#include <vector>

#include "gg_msearch.cuh"

namespace gg {

__global__ void k_fill_cols_i32(int32_t* d, int64_t n, int64_t ld, int64_t S, int32_t v) {
  const int64_t total = n * S;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = t / n, i = t - q * n;
    d[q * ld + i] = v;
  }
}

// seed the group: bit q of vertex sources[q] in frontier and visited, level 0
__global__ void k_bb_seed(const int64_t* src, int64_t S, int W, unsigned* F, unsigned* V,
                          int32_t* dist, int64_t ld) {
  for (int64_t q = threadIdx.x; q < S; q += blockDim.x) {
    const int64_t s = src[q] - 1;
    atomicOr(F + s * W + (q >> 5), 1u << (q & 31));
    atomicOr(V + s * W + (q >> 5), 1u << (q & 31));
    dist[q * ld + s] = 0;
  }
}

// build (once per matrix) the hub list of the graph's CSR view
int build_hub_plan(gg_ctx* ctx, gg_mat* A, const int32_t* rowptr, int64_t n) {
  if (A->hubplan) return GG_OK;
  std::vector<int32_t> rp(n + 1);
  GG_CUDA(cudaMemcpyAsync(rp.data(), rowptr, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> hubs, mid;
  std::vector<int4> pieces;
  for (int64_t v = 0; v < n; ++v) {
    const int64_t k0 = rp[v] - 1, k1 = rp[v + 1] - 1;
    if (k1 - k0 > 32 && k1 - k0 <= kHubDegB) mid.push_back((int32_t)v);
    if (k1 - k0 <= kHubDegB) continue;
    const int hi = (int)hubs.size();
    hubs.push_back((int32_t)v);
    for (int64_t kb = k0; kb < k1; kb += kHubPieceB)
      pieces.push_back(make_int4(hi, (int)kb, (int)(kb + kHubPieceB < k1 ? kb + kHubPieceB : k1), 0));
  }
  // largest pieces first for the round-robin warp assignment
  std::stable_sort(pieces.begin(), pieces.end(),
                   [](const int4& a, const int4& b) { return (a.z - a.y) > (b.z - b.y); });
  std::stable_sort(mid.begin(), mid.end(),
                   [&](int32_t a, int32_t b) { return rp[a + 1] - rp[a] > rp[b + 1] - rp[b]; });
  std::vector<int32_t> order(mid);
  for (int64_t v = 0; v < n; ++v)
    if (rp[v + 1] - rp[v] <= 32) order.push_back((int32_t)v);
  const unsigned long long norder = (unsigned long long)order.size();
  HubPlan* P = new HubPlan();
  P->nhub = (int64_t)hubs.size();
  P->npiece = (int64_t)pieces.size();
  P->nmid = (int64_t)mid.size();
  P->norder = (int64_t)norder;
  cudaError_t e = cudaSuccess;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(dst, bytes > 0 ? bytes : 16);
    if (e == cudaSuccess && bytes > 0)
      e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  };
  up((void**)&P->hubs, hubs.data(), hubs.size() * sizeof(int32_t));
  up((void**)&P->pieces, pieces.data(), pieces.size() * sizeof(int4));
  up((void**)&P->mid, mid.data(), mid.size() * sizeof(int32_t));
  up((void**)&P->order, order.data(), order.size() * sizeof(int32_t));
  up((void**)&P->d_norder, &norder, sizeof(norder));
  if (e == cudaSuccess) e = cudaMalloc(&P->acc, (P->nhub + 1) * kMaxW * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(P->hubs);
    cudaFree(P->pieces);
    cudaFree(P->acc);
    cudaFree(P->mid);
    cudaFree(P->order);
    cudaFree(P->d_norder);
    delete P;
    return cuda_error(e, "hub analysis");
  }
  A->hubplan = P;
  return GG_OK;
}

template <int W>
static int bb_group(gg_ctx* ctx, int64_t n, const BatchGraph& g, const HubPlan* hp,
                    const int64_t* dsrc, int64_t S, int32_t* dist, int64_t ld, unsigned* F,
                    unsigned* Fn, unsigned* V, unsigned* act, unsigned long long* cnt,
                    int64_t* levels) {
  const size_t bytes = (size_t)n * W * sizeof(unsigned);
  GG_CUDA(cudaMemsetAsync(F, 0, bytes, ctx->stream));
  GG_CUDA(cudaMemsetAsync(V, 0, bytes, ctx->stream));
  if (hp->nhub > 0)
    GG_CUDA(cudaMemsetAsync(hp->acc, 0, hp->nhub * kMaxW * sizeof(unsigned), ctx->stream));
  unsigned hm[2 * kMaxW];
  for (int w = 0; w < kMaxW; ++w) {
    const int64_t lo = (int64_t)w * 32;
    hm[w] = S >= lo + 32 ? 0xffffffffu : (S > lo ? ((1u << (S - lo)) - 1u) : 0u);
    hm[kMaxW + w] = 0;
  }
  GG_CUDA(cudaMemcpyAsync(act, hm, sizeof(hm), cudaMemcpyHostToDevice, ctx->stream));
  k_bb_seed<<<1, 256, 0, ctx->stream>>>(dsrc, S, W, F, V, dist, ld);
  GG_CUDA(cudaGetLastError());
  int64_t g_blocks = (n + 255) / 256;
  if (g_blocks > (int64_t)ctx->num_sms * 8) g_blocks = (int64_t)ctx->num_sms * 8;
  if (g_blocks < 1) g_blocks = 1;
  int64_t p_blocks = (hp->npiece * 32 + 255) / 256;
  if (p_blocks > (int64_t)ctx->num_sms * 8) p_blocks = (int64_t)ctx->num_sms * 8;
  unsigned long long* h = reinterpret_cast<unsigned long long*>(ctx->h_flags);
  unsigned* a_cur = act;
  unsigned* a_nxt = act + kMaxW;
  int32_t level = 0;
  for (;;) {
    ++level;
    GG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream));
    GG_CUDA(cudaMemsetAsync(a_nxt, 0, kMaxW * sizeof(unsigned), ctx->stream));
    const LevelOutMatrix out{dist, ld, level};
    k_ms_level<W, LevelOutMatrix><<<(int)g_blocks, 256, 0, ctx->stream>>>(n, g, F, Fn, V, a_cur,
                                                                          a_nxt, out, cnt);
    GG_CUDA(cudaGetLastError());
    if (hp->nhub > 0) {
      unsigned* hacc = static_cast<unsigned*>(hp->acc);
      k_ms_hub<W><<<(int)p_blocks, 256, 0, ctx->stream>>>(g, hp->pieces, hp->npiece, hp->hubs, F,
                                                          V, a_cur, hacc);
      k_ms_hub_final<W, LevelOutMatrix><<<(int)((hp->nhub + 255) / 256), 256, 0, ctx->stream>>>(
          hp->hubs, hp->nhub, hacc, Fn, V, a_cur, a_nxt, out, cnt);
      GG_CUDA(cudaGetLastError());
    }
    GG_CUDA(cudaMemcpyAsync(h, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h[0] == 0) break;
    unsigned* t = F;
    F = Fn;
    Fn = t;
    t = a_cur;
    a_cur = a_nxt;
    a_nxt = t;
  }
  if (levels) *levels += level;
  return GG_OK;
}

// ---------------------------------------------------------------------------------
// batched shortest paths: 32 source columns, lane = source
// ---------------------------------------------------------------------------------
template <typename T>
__global__ void k_bs_init(T* D, int64_t n, const int64_t* src, int64_t S, unsigned* changed) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * 32;
       t += (int64_t)gridDim.x * blockDim.x)
    D[t] = Lim<T>::max();
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    changed[v] = 0;
}

template <typename T>
__global__ void k_bs_seed(T* D, const int64_t* src, int64_t S, unsigned* changed, int32_t* cq) {
  for (int64_t q = threadIdx.x; q < S; q += blockDim.x) {
    const int64_t s = src[q] - 1;
    D[s * 32 + q] = T(0);
    atomicOr(changed + s, 1u << q);
    cq[q] = (int32_t)s;  // the first round's changed vertices
  }
}

// vertex-major 32-column block -> caller's column-major dist
template <typename T>
__global__ void k_bs_out(const T* D, int64_t n, int64_t S, T* dist, int64_t ld) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * S;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = t / n, v = t - q * n;
    dist[q * ld + v] = D[v * 32 + q];
  }
}

// out-edges of the changed vertices of a round (the work of a restricted next round's
// marking, and a bound of its pulls): sum over cq[0, *ncq) into *out
__global__ void k_ms_degsum(const int32_t* __restrict__ cq, const unsigned long long* ncq,
                            const int32_t* __restrict__ prow, unsigned long long* out) {
  const int64_t total = (int64_t)*((volatile const unsigned long long*)ncq);
  unsigned long long s = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = cq[i];
    s += (unsigned long long)(prow[v + 1] - prow[v]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

static const int kBsStreams = 8;  // 32-source groups run at once (8 x 32 bytes of ctx->h_flags)
// with the SELL-32 full rounds a round is restricted to the marked vertices while the
// out-edges of the changed vertices stay below nnz / kBsSellRestrict
#ifndef GG_BS_SELL_RESTRICT
#define GG_BS_SELL_RESTRICT 16
#endif
static const int64_t kBsSellRestrict = GG_BS_SELL_RESTRICT;

// Work buffers of one batched shortest-path call.  ctr: [0] vertices changed this
// round, [1] / [2] lengths of the changed queues cq[0] / cq[1], [3] marked vertices.
template <typename T>
struct BsWork {
  T* D;
  unsigned* c[2];  // columns of each vertex that dropped in the previous / this round
  int32_t* cq[2];
  int32_t* vlist;
  unsigned* mark;
  int32_t* mhq;    // hubs among the changed vertices, marked in pieces
  int32_t* mhoff;  // their piece offsets
  unsigned long long* ctr;
};

// Rounds run over every vertex while many vertices change, and over the marked
// out-neighbours of the changed ones (k_ms_mark) once few do: a round's work then
// follows the frontier instead of the whole graph.  Both kinds compute the same
// in-place relaxation, so the fixpoint is unchanged.  One BsRun is one group of up to
// 32 sources; several groups run at once, each on its own stream, because a single
// group's rounds are latency-bound and leave most of the GPU idle.
template <typename T>
struct BsRun {
  BsWork<T> w;
  cudaStream_t st = nullptr;
  unsigned long long* h = nullptr;  // pinned counters of the last round
  const int64_t* dsrc = nullptr;
  int64_t S = 0, nchanged = 0, mchanged = 0, r = 0;  // changed vertices, their out-edges
  T* dist = nullptr;
  int cur = 0;
  bool restricted = false, done = false;
};

template <typename T>
static int bs_alloc(BsWork<T>& w, int64_t n, int64_t qcap, cudaStream_t st) {
  unsigned* c = nullptr;
  GG_CUDA(cudaMallocAsync((void**)&w.D, (size_t)n * 32 * sizeof(T), st));
  GG_CUDA(cudaMallocAsync((void**)&c, ((size_t)2 * n + 64) * sizeof(unsigned), st));
  GG_CUDA(cudaMallocAsync((void**)&w.cq[0], (size_t)qcap * sizeof(int32_t), st));
  GG_CUDA(cudaMallocAsync((void**)&w.cq[1], (size_t)qcap * sizeof(int32_t), st));
  GG_CUDA(cudaMallocAsync((void**)&w.vlist, (size_t)(n + 64) * sizeof(int32_t), st));
  GG_CUDA(cudaMallocAsync((void**)&w.mark, (size_t)((n + 31) / 32 + 2) * sizeof(unsigned), st));
  GG_CUDA(cudaMallocAsync((void**)&w.mhq, (size_t)(n + 64) * sizeof(int32_t), st));
  GG_CUDA(cudaMallocAsync((void**)&w.mhoff, (size_t)(n + 65) * sizeof(int32_t), st));
  GG_CUDA(cudaMallocAsync((void**)&w.ctr, 64, st));
  w.c[0] = c;
  w.c[1] = c + n;
  return GG_OK;
}

template <typename T>
static void bs_free(BsWork<T>& w, cudaStream_t st) {
  cudaFreeAsync(w.D, st);
  cudaFreeAsync(w.c[0], st);
  cudaFreeAsync(w.cq[0], st);
  cudaFreeAsync(w.cq[1], st);
  cudaFreeAsync(w.vlist, st);
  cudaFreeAsync(w.mark, st);
  cudaFreeAsync(w.mhq, st);
  cudaFreeAsync(w.mhoff, st);
  cudaFreeAsync(w.ctr, st);
}

template <typename T>
static int bs_start(gg_ctx* ctx, int64_t n, BsRun<T>& R) {
  int64_t gb = (n * 32 + 255) / 256;
  if (gb > (int64_t)ctx->num_sms * 8) gb = (int64_t)ctx->num_sms * 8;
  k_bs_init<T><<<(int)gb, 256, 0, R.st>>>(R.w.D, n, R.dsrc, R.S, R.w.c[0]);
  k_bs_seed<T><<<1, 64, 0, R.st>>>(R.w.D, R.dsrc, R.S, R.w.c[0], R.w.cq[0]);
  GG_CUDA(cudaGetLastError());
  R.h[0] = 0;
  R.h[1] = (unsigned long long)R.S;
  R.h[2] = 0;
  R.h[3] = 0;
  GG_CUDA(cudaMemcpyAsync(R.w.ctr, R.h, 4 * sizeof(unsigned long long), cudaMemcpyHostToDevice, R.st));
  R.nchanged = R.S;
  R.mchanged = -1;  // unknown before the first round
  return GG_OK;
}

// ctr[3] (the marked count, used inside a restricted round only) becomes the out-edge
// count of this round's changed vertices once the round's kernels are done
static int bs_degsum(gg_ctx* ctx, const int32_t* prow, const int32_t* cq,
                     const unsigned long long* ncq, unsigned long long* ctr, cudaStream_t st) {
  GG_CUDA(cudaMemsetAsync(ctr + 3, 0, sizeof(unsigned long long), st));
  k_ms_degsum<<<ctx->num_sms * 4, 256, 0, st>>>(cq, ncq, prow, ctr + 3);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// one round of group R, enqueued on its stream; the counters land in R.h
template <typename T>
static int bs_issue(gg_ctx* ctx, int64_t n, int64_t nnz, const BatchGraph& g, const HubPlan* hp,
                    const int32_t* prow, const int32_t* pcol, const gg_mat* sell, BsRun<T>& R) {
  int64_t gb = (n * 32 + 255) / 256;
  if (gb > (int64_t)ctx->num_sms * 8) gb = (int64_t)ctx->num_sms * 8;
  int64_t pb = (hp->npiece * 32 + 255) / 256;
  if (pb > (int64_t)ctx->num_sms * 8) pb = (int64_t)ctx->num_sms * 8;
  if (pb < 1) pb = 1;
  const int64_t gcap = (int64_t)ctx->num_sms * 8;
  const int64_t avg_deg = n > 0 ? (nnz + n - 1) / n : 1;
  BsWork<T>& w = R.w;
  const int cur = R.cur;
  unsigned long long* ncq_cur = w.ctr + 1 + cur;
  unsigned long long* ncq_nxt = w.ctr + 1 + (cur ^ 1);
  GG_CUDA(cudaMemsetAsync(w.ctr, 0, sizeof(unsigned long long), R.st));
  GG_CUDA(cudaMemsetAsync(ncq_nxt, 0, sizeof(unsigned long long), R.st));
  GG_CUDA(cudaMemsetAsync(w.c[cur ^ 1], 0, (size_t)n * sizeof(unsigned), R.st));
  // with the SELL-32 full rounds (about half the vertex rounds' cost) a round is
  // restricted to the marked vertices only while the changed ones are fewer
  R.restricted = (sell && R.mchanged >= 0) ? R.mchanged * kBsSellRestrict < nnz
                                            : R.nchanged * avg_deg * 4 < nnz;
  if (R.restricted) {
    GG_CUDA(cudaMemsetAsync(w.mark, 0, ((n + 31) / 32) * sizeof(unsigned), R.st));
    GG_CUDA(cudaMemsetAsync(w.ctr + 3, 0, sizeof(unsigned long long), R.st));
    GG_CUDA(launch_ms_mark(R.st, ctx->num_sms, R.nchanged, prow, pcol, w.cq[cur], ncq_cur, w.mark,
                           w.vlist, w.ctr + 3, w.mhq, w.ctr + 4, w.mhoff));
    k_ms_round<T><<<(int)gcap, 256, 0, R.st>>>(n, g, w.D, w.c[cur], w.c[cur ^ 1], w.ctr, nullptr,
                                               w.vlist, w.ctr + 3, w.cq[cur ^ 1], ncq_nxt);
  } else if (sell) {
    // every vertex over the SELL-32 copy (hubs included, as chunks of their rows)
    if constexpr (sizeof(T) == 4) {
      const size_t smem = kMsSellWarps * sizeof(MsSellWarpSmem<T>);
      k_ms_round_sell<T><<<ctx->num_sms * 4, kMsSellWarps * 32, smem, R.st>>>(
          sell->colval, sell->nzval, sell->dtype, sell->perm, sell->m, sell->sellplan->pitems,
          sell->sellplan->npitems, w.D, w.c[cur], w.c[cur ^ 1], w.ctr, nullptr, w.cq[cur ^ 1],
          ncq_nxt);
      GG_CUDA(cudaGetLastError());
      GG_CHECK(bs_degsum(ctx, prow, w.cq[cur ^ 1], ncq_nxt, w.ctr, R.st));
      GG_CUDA(cudaMemcpyAsync(R.h, w.ctr, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, R.st));
      return GG_OK;
    }
  } else {
    // every non-hub vertex, in the plan's order: the long rows first, spread over the warps
    k_ms_round<T><<<(int)gb, 256, 0, R.st>>>(n, g, w.D, w.c[cur], w.c[cur ^ 1], w.ctr, nullptr,
                                             hp->order, hp->d_norder, w.cq[cur ^ 1], ncq_nxt);
  }
  GG_CUDA(cudaGetLastError());
  if (hp->npiece > 0) {
    k_ms_round_hub<T><<<(int)pb, 256, 0, R.st>>>(g, hp->pieces, hp->npiece, hp->hubs, w.D,
                                                 w.c[cur], w.c[cur ^ 1], w.ctr, nullptr,
                                                 R.restricted ? w.mark : nullptr, w.cq[cur ^ 1],
                                                 ncq_nxt);
    GG_CUDA(cudaGetLastError());
  }
  GG_CHECK(bs_degsum(ctx, prow, w.cq[cur ^ 1], ncq_nxt, w.ctr, R.st));
  GG_CUDA(cudaMemcpyAsync(R.h, w.ctr, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, R.st));
  return GG_OK;
}

template <typename T>
static int sssp_batch_t(gg_ctx* ctx, gg_mat* A, const BatchGraph& g, const int64_t* sources,
                        int64_t S, T* dist, int64_t ld, int64_t* rounds) {
  const int64_t n = A->m;
  GG_CHECK(build_hub_plan(ctx, A, g.rowptr, n));
  const int32_t* prow = nullptr;
  const int32_t* pcol = nullptr;
  GG_CHECK(push_view(ctx, A, &prow, &pcol));
  const HubPlan* hp = A->hubplan;
  // full rounds over the SELL-32 copy of large CSR graphs (4-byte distances: a warp
  // keeps 32 rows x 32 columns of minima in registers)
  const gg_mat* sell = nullptr;
  if constexpr (sizeof(T) == 4) {
    const int prc = pull_sell_copy(ctx, A, &sell);
    if (prc == GG_ERR_OOM) sell = nullptr;  // no room for the copy: vertex rounds only
    else GG_CHECK(prc);
    if (sell)
      GG_CUDA(cudaFuncSetAttribute(k_ms_round_sell<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(kMsSellWarps * sizeof(MsSellWarpSmem<T>))));
  }
  // a hub may enter a changed queue once per piece
  const int64_t qcap = n + hp->npiece + 64;
  const int64_t nnz = (int64_t)A->nnz;
  const int64_t ngroups = (S + 31) / 32;
  const int64_t conc = ngroups < kBsStreams ? ngroups : kBsStreams;  // groups at once
  int64_t* dsrc = nullptr;
  GG_CUDA(cudaMallocAsync((void**)&dsrc, (size_t)S * sizeof(int64_t) + 8, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(dsrc, sources, S * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  cudaEvent_t ready;
  GG_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  GG_CUDA(cudaEventRecord(ready, ctx->stream));
  std::vector<BsRun<T>> runs(conc);
  unsigned long long* hbase = reinterpret_cast<unsigned long long*>(ctx->h_flags);
  int rc = GG_OK;
  for (int64_t i = 0; i < conc && rc == GG_OK; ++i) {
    BsRun<T>& R = runs[i];
    if (cudaStreamCreateWithFlags(&R.st, cudaStreamNonBlocking) != cudaSuccess) {
      R.st = nullptr;
      rc = set_error(GG_ERR_CUDA, "stream creation failed");
      break;
    }
    R.h = hbase + 4 * i;
    if (cudaStreamWaitEvent(R.st, ready, 0) != cudaSuccess) rc = set_error(GG_ERR_CUDA, "stream wait");
    if (rc == GG_OK) rc = bs_alloc<T>(R.w, n, qcap, R.st);
    R.done = true;  // not started
  }
  int64_t next_group = 0;
  auto start_next = [&](BsRun<T>& R) -> int {
    if (next_group >= ngroups) return GG_OK;
    const int64_t q0 = next_group * 32;
    R.S = S - q0 < 32 ? S - q0 : 32;
    R.dsrc = dsrc + q0;
    R.dist = dist + q0 * ld;
    R.cur = 0;
    R.r = 0;
    R.done = false;
    ++next_group;
    return bs_start<T>(ctx, n, R);
  };
  for (int64_t i = 0; i < conc && rc == GG_OK; ++i) rc = start_next(runs[i]);
  int64_t gb = (n * 32 + 255) / 256;
  if (gb > (int64_t)ctx->num_sms * 8) gb = (int64_t)ctx->num_sms * 8;
  bool active = rc == GG_OK;
  while (active && rc == GG_OK) {
    active = false;
    for (auto& R : runs)
      if (!R.done && rc == GG_OK) rc = bs_issue<T>(ctx, n, nnz, g, hp, prow, pcol, sell, R);
    for (auto& R : runs) {
      if (R.done || rc != GG_OK) continue;
      if (cudaStreamSynchronize(R.st) != cudaSuccess) {
        rc = cuda_error(cudaGetLastError(), "batched shortest paths");
        break;
      }
      if (rounds) *rounds += 1;
      ++R.r;
      if (R.h[0] == 0) {  // converged: write the group out, take the next one
        k_bs_out<T><<<(int)gb, 256, 0, R.st>>>(R.w.D, n, R.S, R.dist, ld);
        R.done = true;
        rc = start_next(R);
      } else if (R.r > n + 1) {
        rc = set_error(GG_ERR_NOT_CONVERGED, "batched shortest paths did not converge");
      } else {
        R.nchanged = (int64_t)R.h[1 + (R.cur ^ 1)];
        R.mchanged = (int64_t)R.h[3];
        R.cur ^= 1;
      }
      if (!R.done) active = true;
    }
  }
  // join: the caller's stream waits for every group's last work
  for (auto& R : runs) {
    if (!R.st) continue;
    bs_free<T>(R.w, R.st);
    cudaEvent_t fin;
    if (cudaEventCreateWithFlags(&fin, cudaEventDisableTiming) == cudaSuccess) {
      cudaEventRecord(fin, R.st);
      cudaStreamWaitEvent(ctx->stream, fin, 0);
      cudaEventDestroy(fin);
    }
    cudaStreamDestroy(R.st);
  }
  cudaEventDestroy(ready);
  cudaFreeAsync(dsrc, ctx->stream);
  if (rc == GG_OK) GG_CUDA(cudaGetLastError());
  return rc;
}

static int dist_type_b(int tv) { return tv == GG_BOOL ? GG_INT32 : tv; }

static int batch_prepare(gg_ctx* ctx, const gg_mat* A_T, const int64_t* sources, int64_t S,
                         BatchGraph* g, bool* nonneg) {
  if (!ctx || !A_T || (S > 0 && !sources)) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (A_T->m != A_T->n) return set_error(GG_ERR_DIMENSION, "A_T must be square");
  for (int64_t q = 0; q < S; ++q)
    if (sources[q] < 1 || sources[q] > A_T->m)
      return set_error(GG_ERR_BOUNDS, "source %lld out of 1:%lld", (long long)sources[q],
                       (long long)A_T->m);
  GG_CUDA(cudaSetDevice(ctx->device));
  bool all_odd = false;
  const int32_t* rp;
  const int32_t* cv;
  const void* nz;
  GG_CHECK(graph_view(ctx, const_cast<gg_mat*>(A_T), &rp, &cv, &nz, &all_odd, nonneg));
  g->rowptr = rp;
  g->colval = cv;
  g->nz = nz;
  g->tv = A_T->dtype;
  g->odd_only = !all_odd;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_bfs_levels_batch(gg_ctx* ctx, const gg_mat* A_T, const int64_t* sources, int64_t S,
                        int32_t* dist, int64_t ld, int64_t* levels_out) {
  BatchGraph g;
  bool nonneg = false;
  GG_CHECK(batch_prepare(ctx, A_T, sources, S, &g, &nonneg));
  if (dtype_is_float(A_T->dtype))
    return set_error(GG_ERR_UNSUPPORTED, "GPUGraphs_band has no method for floating-point matrices");
  const int64_t n = A_T->m;
  if (ld < n) return set_error(GG_ERR_DIMENSION, "leading dimension of dist must be >= n");
  if (!dist && S > 0) return set_error(GG_ERR_ARGUMENT, "NULL dist");
  if (levels_out) *levels_out = 0;
  if (S == 0 || n == 0) return GG_OK;
  GG_CHECK(build_hub_plan(ctx, const_cast<gg_mat*>(A_T), g.rowptr, n));
  const int64_t gs = S < 256 ? S : 256;
  const int W = (int)((gs + 31) / 32);
  unsigned *F = nullptr, *Fn = nullptr, *V = nullptr, *gm = nullptr;
  int64_t* dsrc = nullptr;
  unsigned long long* cnt = nullptr;
  const size_t bytes = (size_t)n * W * sizeof(unsigned);
  GG_CUDA(cudaMallocAsync((void**)&F, bytes, ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&Fn, bytes, ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&V, bytes, ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&gm, 2 * kMaxW * sizeof(unsigned), ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&cnt, 64, ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&dsrc, S * sizeof(int64_t) + 8, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(dsrc, sources, S * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  int64_t gb = (n * S + 255) / 256;
  if (gb > (int64_t)ctx->num_sms * 16) gb = (int64_t)ctx->num_sms * 16;
  k_fill_cols_i32<<<(int)(gb < 1 ? 1 : gb), 256, 0, ctx->stream>>>(dist, n, ld, S, INT32_MAX);
  int rc = GG_OK;
  for (int64_t q0 = 0; q0 < S && rc == GG_OK; q0 += 256) {
    const int64_t Sg = S - q0 < 256 ? S - q0 : 256;
    int32_t* dq = dist + q0 * ld;
    switch ((Sg + 31) / 32) {
      case 1: rc = bb_group<1>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
      case 2: rc = bb_group<2>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
      case 3: rc = bb_group<3>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
      case 4: rc = bb_group<4>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
      case 5: rc = bb_group<5>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
      case 6: rc = bb_group<6>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
      case 7: rc = bb_group<7>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
      default: rc = bb_group<8>(ctx, n, g, A_T->hubplan, dsrc + q0, Sg, dq, ld, F, Fn, V, gm, cnt, levels_out); break;
    }
  }
  cudaFreeAsync(F, ctx->stream);
  cudaFreeAsync(Fn, ctx->stream);
  cudaFreeAsync(V, ctx->stream);
  cudaFreeAsync(gm, ctx->stream);
  cudaFreeAsync(cnt, ctx->stream);
  cudaFreeAsync(dsrc, ctx->stream);
  if (rc == GG_OK) GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return rc;
}

int gg_sssp_batch(gg_ctx* ctx, const gg_mat* A_T, const int64_t* sources, int64_t S, void* dist,
                  int dist_dtype, int64_t ld, int64_t* rounds_out) {
  BatchGraph g;
  bool nonneg = false;
  GG_CHECK(batch_prepare(ctx, A_T, sources, S, &g, &nonneg));
  const int64_t n = A_T->m;
  if (ld < n) return set_error(GG_ERR_DIMENSION, "leading dimension of dist must be >= n");
  if (dist_dtype != dist_type_b(A_T->dtype))
    return set_error(GG_ERR_TYPE, "dist element type must be Int32 for Bool matrices, else eltype(A_T)");
  if (!nonneg)
    return set_error(GG_ERR_UNSUPPORTED, "batched shortest paths need non-negative weights (use gg_sssp)");
  if (rounds_out) *rounds_out = 0;
  if (S == 0 || n == 0) return GG_OK;
  int rc;
  switch (dist_dtype) {
    case GG_INT32: rc = sssp_batch_t<int32_t>(ctx, const_cast<gg_mat*>(A_T), g, sources, S, (int32_t*)dist, ld, rounds_out); break;
    case GG_INT64: rc = sssp_batch_t<int64_t>(ctx, const_cast<gg_mat*>(A_T), g, sources, S, (int64_t*)dist, ld, rounds_out); break;
    case GG_FLOAT32: rc = sssp_batch_t<float>(ctx, const_cast<gg_mat*>(A_T), g, sources, S, (float*)dist, ld, rounds_out); break;
    default: rc = sssp_batch_t<double>(ctx, const_cast<gg_mat*>(A_T), g, sources, S, (double*)dist, ld, rounds_out); break;
  }
  if (rc == GG_OK) GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return rc;
}

}  // extern "C"
