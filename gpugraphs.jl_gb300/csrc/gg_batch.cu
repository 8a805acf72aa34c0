// gg_batch.cu -- many BFS / shortest-path sources in one pass over the graph.
//
// The reference's only batched entry point is shortest_path(A_T, sources)
// (src/algorithms/shortest_path.jl:88-161): a min-plus SpMM per round over an
// n x S distance matrix.  Here:
//  * gg_bfs_levels_batch: up to 256 sources per group, their frontiers and visited
//    sets packed as bits of W <= 8 words per vertex.  One bottom-up level ORs the
//    frontier words of every in-neighbour (over edges with odd / true values, the
//    levels semiring of bfs.jl:52-59) into the vertex's unvisited bits; lane = vertex,
//    so each in-neighbour costs one 32-byte read and the level writes of a warp are
//    coalesced per source column.  Only sources whose frontier is non-empty are
//    looked for, and a vertex stops scanning once all of them reached it.  Vertices
//    of more than 32 in-edges are scanned by their whole warp, hubs of more than
//    kHubDegB in pieces by separate warps (OR-combined, then finished by one thread
//    per hub).  Column q equals bfs_distances(A_T, sources[q]).
//  * gg_sssp_batch: 32 sources per warp pass, lane = source, distances kept
//    vertex-major so one in-neighbour costs one 128-byte read; each round relaxes
//    only from vertices whose distances changed in the previous round, in place
//    (the fixpoint is the same, shortest_path.jl:61-80).  Hubs are relaxed in pieces
//    with atomic min.  Column q equals shortest_path(A_T, sources[q]).
#include <algorithm>
#include <vector>

#include "gg_semiring.cuh"

namespace gg {

static const unsigned kFullB = 0xffffffffu;
static const int kMaxW = 8;  // 256 sources per BFS group

struct BatchGraph {  // CSR view of A_T used by the batched kernels
  const int32_t* rowptr;
  const int32_t* colval;
  const void* nz;
  int tv;
  bool odd_only;
};

int graph_view(gg_ctx* ctx, gg_mat* A, const int32_t** rp, const int32_t** cv, const void** nz,
               bool* all_odd, bool* nonneg);  // gg_graph.cu

__device__ __forceinline__ bool b_odd(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<const uint8_t*>(nz)[k] & 1;
    case GG_INT32: return static_cast<const int32_t*>(nz)[k] & 1;
    case GG_INT64: return static_cast<const int64_t*>(nz)[k] & 1;
  }
  return false;
}

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

static const int kCoopDeg = 32;  // in-degree above which the whole warp scans a vertex

// build (once per matrix) the hub list of the graph's CSR view
static int build_hub_plan(gg_ctx* ctx, gg_mat* A, const int32_t* rowptr, int64_t n) {
  if (A->hubplan) return GG_OK;
  std::vector<int32_t> rp(n + 1);
  GG_CUDA(cudaMemcpyAsync(rp.data(), rowptr, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> hubs;
  std::vector<int4> pieces;
  for (int64_t v = 0; v < n; ++v) {
    const int64_t k0 = rp[v] - 1, k1 = rp[v + 1] - 1;
    if (k1 - k0 <= kHubDegB) continue;
    const int hi = (int)hubs.size();
    hubs.push_back((int32_t)v);
    for (int64_t kb = k0; kb < k1; kb += kHubPieceB)
      pieces.push_back(make_int4(hi, (int)kb, (int)(kb + kHubPieceB < k1 ? kb + kHubPieceB : k1), 0));
  }
  // largest pieces first for the round-robin warp assignment
  std::stable_sort(pieces.begin(), pieces.end(),
                   [](const int4& a, const int4& b) { return (a.z - a.y) > (b.z - b.y); });
  HubPlan* P = new HubPlan();
  P->nhub = (int64_t)hubs.size();
  P->npiece = (int64_t)pieces.size();
  cudaError_t e = cudaSuccess;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(dst, bytes > 0 ? bytes : 16);
    if (e == cudaSuccess && bytes > 0)
      e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  };
  up((void**)&P->hubs, hubs.data(), hubs.size() * sizeof(int32_t));
  up((void**)&P->pieces, pieces.data(), pieces.size() * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc(&P->acc, (P->nhub + 1) * kMaxW * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(P->hubs);
    cudaFree(P->pieces);
    cudaFree(P->acc);
    delete P;
    return cuda_error(e, "hub analysis");
  }
  A->hubplan = P;
  return GG_OK;
}

// OR of the frontier words of in-edges [k0, k1) of one vertex, the whole warp
// scanning 32 edges per step; stops once every bit of m is set.  Uniform result.
template <int W>
__device__ __forceinline__ void warp_scan_or(const BatchGraph& g, const unsigned* __restrict__ F,
                                             int64_t k0, int64_t k1, const unsigned (&m)[W],
                                             unsigned (&acc)[W], int lane) {
#pragma unroll
  for (int w = 0; w < W; ++w) acc[w] = 0;
  for (int64_t kb = k0; kb < k1; kb += 32) {
    const int64_t k = kb + lane;
    unsigned f[W];
#pragma unroll
    for (int w = 0; w < W; ++w) f[w] = 0;
    if (k < k1 && (!g.odd_only || b_odd(g.nz, g.tv, k))) {
      const int64_t u = (int64_t)__ldg(g.colval + k) - 1;
#pragma unroll
      for (int w = 0; w < W; ++w) f[w] = __ldg(F + u * W + w);
    }
    bool full = true;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      acc[w] |= __reduce_or_sync(kFullB, f[w]);
      full &= (acc[w] & m[w]) == m[w];
    }
    if (full) break;
  }
}

// one bottom-up level for a group of sources (W words per vertex); act holds the
// sources whose frontier is non-empty, act_next collects those of the next level
template <int W>
__global__ void __launch_bounds__(256)
    k_bb_level(int64_t n, BatchGraph g, const unsigned* __restrict__ F, unsigned* Fn,
               unsigned* V, const unsigned* __restrict__ act, unsigned* act_next, int32_t level,
               int32_t* dist, int64_t ld, unsigned long long* count) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned am[W];
#pragma unroll
  for (int w = 0; w < W; ++w) am[w] = act[w];
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t v = base + threadIdx.x;
    unsigned m[W], acc[W];
    bool open = false, hub = false;
    int64_t k0 = 0, k1 = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      m[w] = 0;
      acc[w] = 0;
    }
    if (v < n) {
      k0 = (int64_t)g.rowptr[v] - 1;
      k1 = (int64_t)g.rowptr[v + 1] - 1;
      hub = k1 - k0 > kHubDegB;
      if (!hub) {
#pragma unroll
        for (int w = 0; w < W; ++w) {
          m[w] = ~V[v * W + w] & am[w];
          open |= m[w] != 0;
        }
      }
    }
    const bool light = open && k1 - k0 <= kCoopDeg;
    if (light) {
      for (int64_t k = k0; k < k1; ++k) {
        if (g.odd_only && !b_odd(g.nz, g.tv, k)) continue;
        const int64_t u = (int64_t)__ldg(g.colval + k) - 1;
        bool full = true;
#pragma unroll
        for (int w = 0; w < W; ++w) {
          acc[w] |= __ldg(F + u * W + w);
          full &= (acc[w] & m[w]) == m[w];
        }
        if (full) break;  // every open source reached this vertex
      }
    }
    unsigned coop = __ballot_sync(kFullB, open && !light);
    while (coop) {
      const int h = __ffs(coop) - 1;
      coop &= coop - 1;
      unsigned hm[W], ha[W];
#pragma unroll
      for (int w = 0; w < W; ++w) hm[w] = __shfl_sync(kFullB, m[w], h);
      warp_scan_or<W>(g, F, __shfl_sync(kFullB, k0, h), __shfl_sync(kFullB, k1, h), hm, ha, lane);
      if (lane == h) {
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] = ha[w];
      }
    }
    unsigned anynew = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      acc[w] &= m[w];
      anynew |= acc[w];
      if (v < n && !hub) {  // hubs are finished by k_bb_hub_final
        if (acc[w]) V[v * W + w] |= acc[w];
        Fn[v * W + w] = acc[w];
      }
    }
    // level writes, one source column at a time (coalesced over the warp's vertices)
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const unsigned any_w = __reduce_or_sync(kFullB, acc[w]);
      if (lane == 0 && any_w) atomicOr(act_next + w, any_w);
      unsigned u = any_w;
      while (u) {
        const int b = __ffs(u) - 1;
        u &= u - 1;
        if ((acc[w] >> b) & 1u) dist[(int64_t)(w * 32 + b) * ld + v] = level;
      }
    }
    const unsigned bal = __ballot_sync(kFullB, anynew != 0);
    if (lane == 0 && bal) atomicAdd(count, (unsigned long long)__popc(bal));
  }
}

// hub pieces: one warp per piece ORs its in-neighbours' frontier words into the
// hub's accumulator
template <int W>
__global__ void __launch_bounds__(256)
    k_bb_hub(BatchGraph g, const int4* __restrict__ pieces, int64_t npiece,
             const int32_t* __restrict__ hubs, const unsigned* __restrict__ F,
             const unsigned* __restrict__ V, const unsigned* __restrict__ act, unsigned* hacc) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < npiece;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int4 p = pieces[i];
    const int64_t v = hubs[p.x];
    unsigned m[W], ha[W];
    bool open = false;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      m[w] = ~V[v * W + w] & act[w];
      open |= m[w] != 0;
    }
    if (!open) continue;
    warp_scan_or<W>(g, F, p.y, p.z, m, ha, lane);
    if (lane == 0) {
#pragma unroll
      for (int w = 0; w < W; ++w)
        if (ha[w] & m[w]) atomicOr(hacc + (int64_t)p.x * kMaxW + w, ha[w] & m[w]);
    }
  }
}

// one thread per hub: new bits, visited, next frontier, levels
template <int W>
__global__ void k_bb_hub_final(const int32_t* __restrict__ hubs, int64_t nhub, unsigned* hacc,
                               unsigned* Fn, unsigned* V, const unsigned* __restrict__ act,
                               unsigned* act_next, int32_t level, int32_t* dist, int64_t ld,
                               unsigned long long* count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nhub;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = hubs[i];
    bool any = false;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const unsigned m = ~V[v * W + w] & act[w];
      const unsigned a = hacc[i * kMaxW + w] & m;
      hacc[i * kMaxW + w] = 0;
      Fn[v * W + w] = a;
      if (!a) continue;
      any = true;
      V[v * W + w] |= a;
      atomicOr(act_next + w, a);
      unsigned u = a;
      while (u) {
        const int b = __ffs(u) - 1;
        u &= u - 1;
        dist[(int64_t)(w * 32 + b) * ld + v] = level;
      }
    }
    if (any) atomicAdd(count, 1ull);
  }
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
    k_bb_level<W><<<(int)g_blocks, 256, 0, ctx->stream>>>(n, g, F, Fn, V, a_cur, a_nxt, level,
                                                          dist, ld, cnt);
    GG_CUDA(cudaGetLastError());
    if (hp->nhub > 0) {
      unsigned* hacc = static_cast<unsigned*>(hp->acc);
      k_bb_hub<W><<<(int)p_blocks, 256, 0, ctx->stream>>>(g, hp->pieces, hp->npiece, hp->hubs, F,
                                                          V, a_cur, hacc);
      k_bb_hub_final<W><<<(int)((hp->nhub + 255) / 256), 256, 0, ctx->stream>>>(
          hp->hubs, hp->nhub, hacc, Fn, V, a_cur, a_nxt, level, dist, ld, cnt);
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
template <typename T> __device__ __forceinline__ T b_relax(T w, T d) {
  return (w == Lim<T>::max() || d == Lim<T>::max()) ? Lim<T>::max() : w_add(w, d);
}

template <typename T>
__device__ __forceinline__ T b_weight(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<T>(static_cast<const uint8_t*>(nz)[k]);
    case GG_INT32: return static_cast<T>(static_cast<const int32_t*>(nz)[k]);
    case GG_INT64: return static_cast<T>(static_cast<const int64_t*>(nz)[k]);
    case GG_FLOAT32: return static_cast<T>(static_cast<const float*>(nz)[k]);
  }
  return static_cast<T>(static_cast<const double*>(nz)[k]);
}

template <typename T>
__global__ void k_bs_init(T* D, int64_t n, const int64_t* src, int64_t S, uint8_t* changed) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * 32;
       t += (int64_t)gridDim.x * blockDim.x)
    D[t] = Lim<T>::max();
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    changed[v] = 0;
}

template <typename T>
__global__ void k_bs_seed(T* D, const int64_t* src, int64_t S, uint8_t* changed) {
  for (int64_t q = threadIdx.x; q < S; q += blockDim.x) {
    const int64_t s = src[q] - 1;
    D[s * 32 + q] = T(0);
    changed[s] = 1;
  }
}

// pull over in-edges [k0, k1) of v from in-neighbours that changed last round:
// per-lane (source column) minimum of D[u] + w
template <typename T>
__device__ __forceinline__ bool bs_pull(const BatchGraph& g, const T* D,
                                        const uint8_t* __restrict__ chg, int64_t k0, int64_t k1,
                                        int lane, T& best) {
  bool any = false;
  for (int64_t kb = k0; kb < k1; kb += 32) {
    const int64_t kk = kb + lane;
    int32_t u = -1;
    if (kk < k1) {
      const int32_t c = __ldg(g.colval + kk) - 1;
      if (chg[c]) u = c;
    }
    unsigned act = __ballot_sync(kFullB, u >= 0);
    while (act) {
      const int src_lane = __ffs(act) - 1;
      act &= act - 1;
      const int32_t uu = __shfl_sync(kFullB, u, src_lane);
      const T w = b_weight<T>(g.nz, g.tv, kb + src_lane);
      const T cand = b_relax(w, D[(int64_t)uu * 32 + lane]);
      if (cand < best) best = cand;
      any = true;
    }
  }
  return any;
}

// one round: warp per vertex v, lane = source column; pull from in-neighbours that
// changed last round, lower D[v] in place, flag v when any column dropped (chg_next
// is cleared before the round).  Hubs are left to k_bs_hub.
template <typename T>
__global__ void __launch_bounds__(256)
    k_bs_round(int64_t n, BatchGraph g, T* D, const uint8_t* __restrict__ chg,
               uint8_t* chg_next, unsigned long long* count) {
  const int lane = threadIdx.x & 31;
  for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n;
       v += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t k0 = (int64_t)g.rowptr[v] - 1, k1 = (int64_t)g.rowptr[v + 1] - 1;
    if (k1 - k0 > kHubDegB) continue;
    T best = Lim<T>::max();
    const bool any = bs_pull<T>(g, D, chg, k0, k1, lane, best);
    bool dropped = false;
    if (any) {
      T* dv = D + v * 32 + lane;
      if (best < *dv) {
        *dv = best;
        dropped = true;
      }
    }
    const unsigned b = __ballot_sync(kFullB, dropped);
    if (lane == 0 && b) {
      chg_next[v] = 1;
      atomicAdd(count, 1ull);
    }
  }
}

template <typename T> __device__ __forceinline__ T b_atomic_min(T* p, T v);
template <> __device__ __forceinline__ int32_t b_atomic_min<int32_t>(int32_t* p, int32_t v) {
  return atomicMin(p, v);
}
template <> __device__ __forceinline__ int64_t b_atomic_min<int64_t>(int64_t* p, int64_t v) {
  return (int64_t)atomicMin((long long*)p, (long long)v);
}
// distances are non-negative here (never -0.0: +0.0 + w), so floats order like
// their bit patterns
template <> __device__ __forceinline__ float b_atomic_min<float>(float* p, float v) {
  return __int_as_float(atomicMin((int*)p, __float_as_int(v)));
}
template <> __device__ __forceinline__ double b_atomic_min<double>(double* p, double v) {
  return __longlong_as_double(atomicMin((long long*)p, __double_as_longlong(v)));
}

// hub pieces: one warp per piece, atomic min into the hub's 32 columns
template <typename T>
__global__ void __launch_bounds__(256)
    k_bs_hub(BatchGraph g, const int4* __restrict__ pieces, int64_t npiece,
             const int32_t* __restrict__ hubs, T* D, const uint8_t* __restrict__ chg,
             uint8_t* chg_next, unsigned long long* count) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < npiece;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int4 p = pieces[i];
    const int64_t v = hubs[p.x];
    T best = Lim<T>::max();
    const bool any = bs_pull<T>(g, D, chg, p.y, p.z, lane, best);
    bool dropped = false;
    if (any) {
      T* dv = D + v * 32 + lane;
      if (best < *dv) dropped = best < b_atomic_min<T>(dv, best);
    }
    const unsigned b = __ballot_sync(kFullB, dropped);
    if (lane == 0 && b) {
      chg_next[v] = 1;
      atomicAdd(count, 1ull);
    }
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

template <typename T>
static int bs_group(gg_ctx* ctx, int64_t n, const BatchGraph& g, const HubPlan* hp,
                    const int64_t* dsrc, int64_t S,
                    T* dist, int64_t ld, T* D, uint8_t* c0, uint8_t* c1, unsigned long long* cnt,
                    int64_t* rounds) {
  int64_t gb = (n * 32 + 255) / 256;
  if (gb > (int64_t)ctx->num_sms * 8) gb = (int64_t)ctx->num_sms * 8;
  int64_t pb = (hp->npiece * 32 + 255) / 256;
  if (pb > (int64_t)ctx->num_sms * 8) pb = (int64_t)ctx->num_sms * 8;
  k_bs_init<T><<<(int)gb, 256, 0, ctx->stream>>>(D, n, dsrc, S, c0);
  k_bs_seed<T><<<1, 64, 0, ctx->stream>>>(D, dsrc, S, c0);
  GG_CUDA(cudaGetLastError());
  unsigned long long* h = reinterpret_cast<unsigned long long*>(ctx->h_flags);
  for (int64_t r = 0;; ++r) {
    if (r > n + 1) return set_error(GG_ERR_NOT_CONVERGED, "batched shortest paths did not converge");
    GG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream));
    GG_CUDA(cudaMemsetAsync(c1, 0, (size_t)n, ctx->stream));
    k_bs_round<T><<<(int)gb, 256, 0, ctx->stream>>>(n, g, D, c0, c1, cnt);
    GG_CUDA(cudaGetLastError());
    if (hp->npiece > 0) {
      k_bs_hub<T><<<(int)pb, 256, 0, ctx->stream>>>(g, hp->pieces, hp->npiece, hp->hubs, D, c0, c1,
                                                     cnt);
      GG_CUDA(cudaGetLastError());
    }
    GG_CUDA(cudaMemcpyAsync(h, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (rounds) *rounds += 1;
    if (h[0] == 0) break;
    uint8_t* t = c0;
    c0 = c1;
    c1 = t;
  }
  k_bs_out<T><<<(int)gb, 256, 0, ctx->stream>>>(D, n, S, dist, ld);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

template <typename T>
static int sssp_batch_t(gg_ctx* ctx, gg_mat* A, const BatchGraph& g, const int64_t* sources,
                        int64_t S, T* dist, int64_t ld, int64_t* rounds) {
  const int64_t n = A->m;
  GG_CHECK(build_hub_plan(ctx, A, g.rowptr, n));
  T* D = nullptr;
  uint8_t* c = nullptr;
  int64_t* dsrc = nullptr;
  unsigned long long* cnt = nullptr;
  GG_CUDA(cudaMallocAsync((void**)&D, (size_t)n * 32 * sizeof(T), ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&c, (size_t)2 * n + 64, ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&dsrc, (size_t)S * sizeof(int64_t) + 8, ctx->stream));
  GG_CUDA(cudaMallocAsync((void**)&cnt, 64, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(dsrc, sources, S * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  int rc = GG_OK;
  for (int64_t q0 = 0; q0 < S && rc == GG_OK; q0 += 32) {
    const int64_t Sg = S - q0 < 32 ? S - q0 : 32;
    rc = bs_group<T>(ctx, n, g, A->hubplan, dsrc + q0, Sg, dist + q0 * ld, ld, D, c, c + n, cnt, rounds);
  }
  cudaFreeAsync(D, ctx->stream);
  cudaFreeAsync(c, ctx->stream);
  cudaFreeAsync(dsrc, ctx->stream);
  cudaFreeAsync(cnt, ctx->stream);
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
