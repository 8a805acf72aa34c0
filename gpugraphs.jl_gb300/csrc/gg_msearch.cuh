// gg_msearch.cuh -- device code shared by the batched searches (gg_batch.cu) and
// the query server (gg_serve.cu): many BFS / shortest-path sources advanced together
// over one graph.
//  * BFS: the sources' frontier / visited sets are bits of W <= 8 words per vertex.
//    A level (k_ms_level) ORs the frontier words of a vertex's in-neighbours (edges
//    with odd / true values, the levels semiring of src/algorithms/bfs.jl:52-59) into
//    its unvisited bits, for the sources in `act` only (those whose frontier is not
//    empty); a vertex stops scanning once all of them reached it.  Vertices with more
//    than kCoopDeg in-edges are scanned by the whole warp; hubs (more than kHubDegB)
//    in pieces by separate warps (k_ms_hub), finished by k_ms_hub_final.  New levels
//    are written through an output policy (a distance matrix, or per-query buffers).
//  * Shortest paths: 32 source columns, lane = column, distances vertex-major so one
//    in-neighbour costs one 128-byte read.  A round (k_ms_round) pulls from the
//    in-neighbours whose distances changed in the previous round and lowers D in
//    place; hubs are relaxed in pieces with atomic min (k_ms_round_hub).  The fixpoint
//    is that of shortest_path's Jacobi rounds (src/algorithms/shortest_path.jl:61-80).
#pragma once

#include "gg_semiring.cuh"

namespace gg {

int graph_view(gg_ctx* ctx, gg_mat* A, const int32_t** rp, const int32_t** cv, const void** nz,
               bool* all_odd, bool* nonneg);  // gg_graph.cu
int build_hub_plan(gg_ctx* ctx, gg_mat* A, const int32_t* rowptr, int64_t n);  // gg_batch.cu
int push_view(gg_ctx* ctx, gg_mat* A, const int32_t** prow, const int32_t** pcol);  // gg_graph.cu
int sssp_prepare(gg_ctx* ctx, gg_mat* A);  // gg_graph.cu
int pull_sell_copy(gg_ctx* ctx, gg_mat* A, const gg_mat** out);  // gg_graph.cu

namespace {

static const unsigned kFullB = 0xffffffffu;
static const int kMaxW = 8;  // 256 sources per BFS group

struct BatchGraph {  // CSR view of A_T used by the batched kernels
  const int32_t* rowptr;
  const int32_t* colval;
  const void* nz;
  int tv;
  bool odd_only;
};

__device__ __forceinline__ bool b_odd(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<const uint8_t*>(nz)[k] & 1;
    case GG_INT32: return static_cast<const int32_t*>(nz)[k] & 1;
    case GG_INT64: return static_cast<const int64_t*>(nz)[k] & 1;
  }
  return false;
}

static const int kCoopDeg = 32;  // in-degree above which the whole warp scans a vertex

// output policies of the BFS kernels: source column q reached vertex v this level
struct LevelOutMatrix {  // dist[q * ld + v] = level
  int32_t* dist;
  int64_t ld;
  int32_t level;
  __device__ __forceinline__ void put(int q, int64_t v) const { dist[(int64_t)q * ld + v] = level; }
};
struct LevelOutSlots {  // per-query buffers: out[q][v] = tick - start[q]
  int32_t* const* outp;
  const int32_t* start;
  int32_t tick;
  __device__ __forceinline__ void put(int q, int64_t v) const { outp[q][v] = tick - start[q]; }
};

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
template <int W, class Out>
__global__ void __launch_bounds__(256)
    k_ms_level(int64_t n, BatchGraph g, const unsigned* __restrict__ F, unsigned* Fn,
               unsigned* V, const unsigned* __restrict__ act, unsigned* act_next, Out out,
               unsigned long long* count) {
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
      if (v < n && !hub) {  // hubs are finished by k_ms_hub_final
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
        if ((acc[w] >> b) & 1u) out.put(w * 32 + b, v);
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
    k_ms_hub(BatchGraph g, const int4* __restrict__ pieces, int64_t npiece,
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
template <int W, class Out>
__global__ void k_ms_hub_final(const int32_t* __restrict__ hubs, int64_t nhub, unsigned* hacc,
                               unsigned* Fn, unsigned* V, const unsigned* __restrict__ act,
                               unsigned* act_next, Out out, unsigned long long* count) {
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
        out.put(w * 32 + b, v);
      }
    }
    if (any) atomicAdd(count, 1ull);
  }
}

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

// pull over in-edges [k0, k1) of v from in-neighbours that changed last round or
// already in this one: per-lane (source column) minimum of D[u] + w.  chg[u] holds the
// columns of u that dropped in the previous round, chg_cur[u] those dropped so far in
// this round (a drop made earlier in the round travels on at once, so fewer rounds
// are needed; any order of relaxations reaches the same fixpoint); only those lanes
// read D[u], so a vertex whose distances changed for few sources costs few 32-byte
// sectors.
template <typename T>
__device__ __forceinline__ bool bs_pull(const BatchGraph& g, const T* D,
                                        const unsigned* __restrict__ chg, const unsigned* chg_cur,
                                        int64_t k0, int64_t k1, int lane, T& best) {
  bool any = false;
  for (int64_t kb = k0; kb < k1; kb += 32) {
    const int64_t kk = kb + lane;
    int32_t u = -1;
    unsigned cm = 0;
    T wl = T(0);
    if (kk < k1) {
      const int32_t c = __ldg(g.colval + kk) - 1;
      cm = __ldcg(chg + c) | __ldcg(chg_cur + c);
      if (cm) {
        u = c;
        wl = b_weight<T>(g.nz, g.tv, kk);
      }
    }
    unsigned act = __ballot_sync(kFullB, u >= 0);
    // changed in-neighbours 8 at a time: their rows of D are read together, so a warp
    // keeps up to 8 reads in flight (the minimum does not depend on the order)
    while (act) {
      int32_t su[8];
      unsigned sm[8];
      T sw[8], dv[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int src_lane = act ? __ffs(act) - 1 : 0;
        const bool valid = act != 0;
        act &= act - 1;
        su[t] = __shfl_sync(kFullB, u, src_lane);
        sm[t] = valid ? __shfl_sync(kFullB, cm, src_lane) : 0u;
        sw[t] = __shfl_sync(kFullB, wl, src_lane);
      }
#pragma unroll
      for (int t = 0; t < 8; ++t)
        dv[t] = ((sm[t] >> lane) & 1u) ? D[(int64_t)su[t] * 32 + lane] : Lim<T>::max();
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        if ((sm[t] >> lane) & 1u) {
          const T cand = b_relax(sw[t], dv[t]);
          if (cand < best) best = cand;
          any = true;
        }
      }
    }
  }
  return any;
}

// Changed-vertex bookkeeping of a round: chg_next[v] gets the columns that dropped and,
// when cq is given, v is appended to the changed queue cq (count *ncq) that drives the
// next round's marking.
__device__ __forceinline__ void ms_changed(int64_t v, unsigned cols, unsigned* chg_next,
                                           unsigned long long* count, int32_t* cq,
                                           unsigned long long* ncq) {
  atomicOr(chg_next + v, cols);
  atomicAdd(count, 1ull);
  if (cq) cq[atomicAdd(ncq, 1ull)] = (int32_t)v;
}

// one round: warp per vertex v (every vertex, or the marked ones in vlist[0, *nlist)),
// lane = source column; pull from in-neighbours that changed last round, lower D[v]
// in place, flag v when any column dropped (chg_next is cleared before the round).
// Hubs are left to k_ms_round_hub.
template <typename T>
__global__ void __launch_bounds__(256)
    k_ms_round(int64_t n, BatchGraph g, T* D, const unsigned* __restrict__ chg,
               unsigned* chg_next, unsigned long long* count, unsigned* drop,
               const int32_t* __restrict__ vlist, const unsigned long long* nlist, int32_t* cq,
               unsigned long long* ncq) {
  const int lane = threadIdx.x & 31;
  unsigned dropped_cols = 0;
  const int64_t total = vlist ? (int64_t)*((volatile const unsigned long long*)nlist) : n;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // the warp's vertices gw, gw + nw, ... taken 32 at a time: vertex j of a batch has its
  // id and row bounds loaded by lane j up front, and the batch's changed vertices are
  // counted and queued with one atomic each
  for (int64_t i0 = gw; i0 < total; i0 += 32 * nw) {
    const int64_t ij = i0 + (int64_t)lane * nw;
    int64_t vj = -1, k0j = 0, k1j = 0;
    if (ij < total) {
      vj = vlist ? (int64_t)vlist[ij] : ij;
      k0j = (int64_t)g.rowptr[vj] - 1;
      k1j = (int64_t)g.rowptr[vj + 1] - 1;
    }
    const unsigned live = __ballot_sync(kFullB, vj >= 0);
    unsigned my_cols = 0;  // lane j: the columns that dropped for vertex j
    for (int j = 0; j < 32 && ((live >> j) & 1u); ++j) {
      const int64_t v = __shfl_sync(kFullB, vj, j);
      const int64_t k0 = __shfl_sync(kFullB, k0j, j), k1 = __shfl_sync(kFullB, k1j, j);
      if (k1 - k0 > kHubDegB) continue;
      T best = Lim<T>::max();
      const bool any = bs_pull<T>(g, D, chg, chg_next, k0, k1, lane, best);
      bool dropped = false;
      if (any) {
        T* dv = D + v * 32 + lane;
        if (best < *dv) {
          *dv = best;
          dropped = true;
        }
      }
      const unsigned b = __ballot_sync(kFullB, dropped);
      dropped_cols |= b;
      if (lane == j) my_cols = b;
    }
    if (my_cols) atomicOr(chg_next + vj, my_cols);
    const unsigned cm = __ballot_sync(kFullB, my_cols != 0);
    if (cm) {
      unsigned long long qb = 0;
      if (lane == 0) {
        atomicAdd(count, (unsigned long long)__popc(cm));
        if (cq) qb = atomicAdd(ncq, (unsigned long long)__popc(cm));
      }
      qb = __shfl_sync(kFullB, qb, 0);
      if (cq && my_cols) cq[qb + __popc(cm & ((1u << lane) - 1u))] = (int32_t)vj;
    }
  }
  if (drop && lane == 0 && dropped_cols) atomicOr(drop, dropped_cols);
}

// marking for a frontier-restricted round: the out-neighbours of the changed vertices
// cq[0, *ncq) are the only vertices whose distances can drop; each is marked once in
// the bitmap and listed in vlist.  A changed vertex with more than kMarkHub out-edges
// is not walked by one warp (a hub's list held one warp for milliseconds while the
// others idled): it is queued in mhq and its out-list marked in pieces of kMarkPiece
// edges by every warp (k_ms_mark_offsets, k_ms_mark_hub).
static const int kMarkHub = 1024, kMarkPiece = 1024;

__device__ __forceinline__ void ms_mark_range(const int32_t* __restrict__ pcol, int32_t k0,
                                              int32_t k1, int lane, unsigned* mark, int32_t* vlist,
                                              unsigned long long* nlist) {
  for (int32_t kb = k0; kb < k1; kb += 32) {
    const int32_t k = kb + lane;
    bool add = false;
    int32_t w = 0;
    if (k < k1) {
      w = __ldg(pcol + k);
      const unsigned bit = 1u << (w & 31);
      if (!(__ldcg(mark + (w >> 5)) & bit)) add = !(atomicOr(mark + (w >> 5), bit) & bit);
    }
    const unsigned b = __ballot_sync(kFullB, add);
    if (b) {
      const int leader = __ffs(b) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(nlist, (unsigned long long)__popc(b));
      base = __shfl_sync(kFullB, base, leader);
      if (add) vlist[base + __popc(b & ((1u << lane) - 1u))] = w;
    }
  }
}

__global__ void __launch_bounds__(256)
    k_ms_mark(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
              const int32_t* __restrict__ cq, const unsigned long long* ncq, unsigned* mark,
              int32_t* vlist, unsigned long long* nlist, int32_t* mhq, unsigned long long* nmh) {
  const int lane = threadIdx.x & 31;
  const int64_t total = (int64_t)*((volatile const unsigned long long*)ncq);
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < total;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t u = cq[i];
    const int32_t k0 = prow[u], k1 = prow[u + 1];
    if (k1 - k0 > kMarkHub) {  // left to the piece kernel
      if (lane == 0) mhq[atomicAdd(nmh, 1ull)] = u;
      continue;
    }
    ms_mark_range(pcol, k0, k1, lane, mark, vlist, nlist);
  }
}

// piece offsets of the queued hubs: mhoff[h] = pieces of hubs before h, mhoff[nh] = all
__global__ void __launch_bounds__(1024)
    k_ms_mark_offsets(const int32_t* __restrict__ prow, const int32_t* __restrict__ mhq,
                      const unsigned long long* nmh, int32_t* mhoff) {
  __shared__ int32_t wsum[32];
  __shared__ int32_t carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t nh = (int64_t)*((volatile const unsigned long long*)nmh);
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < nh; b0 += 1024) {
    const int64_t i = b0 + threadIdx.x;
    int32_t np = 0;
    if (i < nh) {
      const int32_t u = mhq[i];
      np = (prow[u + 1] - prow[u] + kMarkPiece - 1) / kMarkPiece;
    }
    int32_t x = np;  // inclusive scan within the warp, then over the warp totals
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t t = __shfl_up_sync(kFullB, x, o);
      if (lane >= o) x += t;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int32_t y = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(kFullB, y, o);
        if (lane >= o) y += t;
      }
      wsum[lane] = y;
    }
    __syncthreads();
    const int32_t incl = x + (wid > 0 ? wsum[wid - 1] : 0);
    const int32_t c = carry;
    if (i < nh) mhoff[i] = c + incl - np;
    __syncthreads();
    if (threadIdx.x == 1023) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) mhoff[nh] = carry;
}

__global__ void __launch_bounds__(256)
    k_ms_mark_hub(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                  const int32_t* __restrict__ mhq, const unsigned long long* nmh,
                  const int32_t* __restrict__ mhoff, unsigned* mark, int32_t* vlist,
                  unsigned long long* nlist) {
  const int lane = threadIdx.x & 31;
  const int64_t nh = (int64_t)*((volatile const unsigned long long*)nmh);
  if (nh == 0) return;
  const int64_t npieces = mhoff[nh];
  int64_t h = 0;
  for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < npieces;
       q += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    // the hub holding piece q (q only grows, so search forward from the last one)
    if (__ldg(mhoff + h + 1) <= q) {
      int64_t lo = h + 1, hi = nh - 1;
      while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (__ldg(mhoff + mid) <= q) lo = mid; else hi = mid - 1;
      }
      h = lo;
    }
    const int32_t u = mhq[h];
    const int32_t k0 = prow[u] + (int32_t)(q - mhoff[h]) * kMarkPiece;
    const int32_t k1 = min(prow[u + 1], k0 + kMarkPiece);
    ms_mark_range(pcol, k0, k1, lane, mark, vlist, nlist);
  }
}

// the three marking launches of a frontier-restricted round; nmh: a device counter,
// mhq / mhoff: room for n and n + 1 entries
static inline cudaError_t launch_ms_mark(cudaStream_t st, int num_sms, int64_t nchanged,
                                         const int32_t* prow, const int32_t* pcol,
                                         const int32_t* cq, const unsigned long long* ncq,
                                         unsigned* mark, int32_t* vlist, unsigned long long* nlist,
                                         int32_t* mhq, unsigned long long* nmh, int32_t* mhoff) {
  cudaError_t e = cudaMemsetAsync(nmh, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  int64_t mb = (nchanged * 32 + 255) / 256;
  const int64_t gcap = (int64_t)num_sms * 8;
  if (mb > gcap) mb = gcap;
  k_ms_mark<<<(int)(mb < 1 ? 1 : mb), 256, 0, st>>>(prow, pcol, cq, ncq, mark, vlist, nlist, mhq, nmh);
  k_ms_mark_offsets<<<1, 1024, 0, st>>>(prow, mhq, nmh, mhoff);
  k_ms_mark_hub<<<(int)gcap, 256, 0, st>>>(prow, pcol, mhq, nmh, mhoff, mark, vlist, nlist);
  return cudaGetLastError();
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

// Full round over the SELL-32 copy of the graph (4-byte distance types): a warp takes
// one work item of the copy's plan (a chunk of up to kSellChunk entry columns of a
// slice, or a group of narrow slices), i.e. 32 rows.  Entry columns are read 4 at a
// time (lane = row): in-neighbours, their changed-column masks and weights, all loads
// independent; the entries whose in-neighbour changed last round go to a per-warp
// queue in shared memory (6 KB per warp with the minima, so 4 CTAs of 8 warps fit an
// SM: the round waits on its loads, and 32 warps hide more of that than 24 did).  The queue is then drained 16 entries at a time, 4 entries
// per warp instruction (8 lanes per entry, 4 source columns per lane, 16-byte loads of
// D): 16 rows of D in flight per warp, candidates folded with shared-memory atomic min
// into the warp's 32 x 32 minima.  The vertex-per-warp round waits on
// one vertex's chain of loads at a time instead.  Rows are lowered in place with atomic
// min (a long row's chunks are separate items; min is exact in any order, so the
// fixpoint is unchanged), and a vertex enters the next changed queue once, by the warp
// whose atomic OR first set a bit of it.
static const int kMsSellWarps = 8;
static const int kMsSellQ = 4 * 32;  // queue entries of one 4-column step
static const int kMsSellBatch = 16;  // queue entries a warp drains per step (4 at once)

template <typename T>
struct MsSellWarpSmem {
  T acc[32 * 32];       // row l, column q at l * 32 + q
  int4 q[kMsSellQ];     // (in-neighbour, weight bits, changed columns, row)
};

template <typename T>
__device__ __forceinline__ int ms_bits(T w);
template <> __device__ __forceinline__ int ms_bits<int32_t>(int32_t w) { return w; }
template <> __device__ __forceinline__ int ms_bits<float>(float w) { return __float_as_int(w); }
template <typename T>
__device__ __forceinline__ T ms_unbits(int b);
template <> __device__ __forceinline__ int32_t ms_unbits<int32_t>(int b) { return b; }
template <> __device__ __forceinline__ float ms_unbits<float>(int b) { return __int_as_float(b); }

template <typename T>
__device__ __forceinline__ void ms_sell_slice(const int32_t* __restrict__ colval, const void* nz,
                                              int tv, int64_t pos0, int width, int64_t row0,
                                              int64_t m, const int32_t* __restrict__ perm, T* D,
                                              const unsigned* __restrict__ chg, unsigned* chg_next,
                                              unsigned long long* count, int32_t* cq,
                                              unsigned long long* ncq, int lane,
                                              MsSellWarpSmem<T>& sm, unsigned& dropped_cols) {
#pragma unroll 4
  for (int l = 0; l < 32; ++l) sm.acc[l * 32 + lane] = Lim<T>::max();
  for (int j0 = 0; j0 < width; j0 += kMsSellQ / 32) {
    int32_t c[kMsSellQ / 32];
    unsigned cm[kMsSellQ / 32];
    T wv[kMsSellQ / 32];
#pragma unroll
    for (int k = 0; k < kMsSellQ / 32; ++k) {
      c[k] = j0 + k < width ? __ldcs(colval + pos0 + (int64_t)(j0 + k) * 32 + lane) : -1;
      wv[k] = j0 + k < width ? b_weight<T>(nz, tv, pos0 + (int64_t)(j0 + k) * 32 + lane) : T(0);
    }
#pragma unroll
    for (int k = 0; k < kMsSellQ / 32; ++k)
      cm[k] = c[k] > 0 ? (__ldcg(chg + (c[k] - 1)) | __ldcg(chg_next + (c[k] - 1))) : 0u;
    __syncwarp();  // the previous step's queue has been drained
    int nq = 0;
#pragma unroll
    for (int k = 0; k < kMsSellQ / 32; ++k) {
      const unsigned b = __ballot_sync(kFullB, cm[k] != 0);
      if (cm[k]) sm.q[nq + __popc(b & ((1u << lane) - 1u))] = make_int4(c[k] - 1, ms_bits<T>(wv[k]), (int)cm[k], lane);
      nq += __popc(b);
    }
    __syncwarp();
    // 4 queue entries per warp step: lanes 8e .. 8e + 7 take entry e, 4 source columns
    // each (16-byte loads of D); kMsSellBatch / 4 steps' loads in flight.  Two entries
    // of one step may share a row, so the minima are folded with shared-memory atomic
    // min (distances are non-negative: floats order like their bit patterns).
    const int es = lane >> 3, cq4 = (lane & 7) * 4;
    for (int e0 = 0; e0 < nq; e0 += kMsSellBatch) {
      T dv[kMsSellBatch / 4][4];
      int4 qe[kMsSellBatch / 4];
#pragma unroll
      for (int b = 0; b < kMsSellBatch / 4; ++b) {
        const int e = e0 + b * 4 + es;
        qe[b] = e < nq ? sm.q[e] : make_int4(0, 0, 0, 0);
        const unsigned bits = ((unsigned)qe[b].z >> cq4) & 15u;
        dv[b][0] = dv[b][1] = dv[b][2] = dv[b][3] = Lim<T>::max();
        if (bits) {
          const T* row = D + (int64_t)qe[b].x * 32 + cq4;
          if constexpr (sizeof(T) == 4) {
            const int4 r4 = __ldcg(reinterpret_cast<const int4*>(row));
            if (bits & 1u) dv[b][0] = ms_unbits<T>(r4.x);
            if (bits & 2u) dv[b][1] = ms_unbits<T>(r4.y);
            if (bits & 4u) dv[b][2] = ms_unbits<T>(r4.z);
            if (bits & 8u) dv[b][3] = ms_unbits<T>(r4.w);
          }
        }
      }
#pragma unroll
      for (int b = 0; b < kMsSellBatch / 4; ++b) {
        if (e0 + b * 4 + es < nq) {
          const T w = ms_unbits<T>(qe[b].y);
          int* a = reinterpret_cast<int*>(sm.acc + qe[b].w * 32 + cq4);
          const int4 cur = *reinterpret_cast<const int4*>(a);  // may be stale: atomics decide
          const int cv[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int cb = ms_bits<T>(b_relax(w, dv[b][k]));
            if (cb < cv[k]) atomicMin(a + k, cb);
          }
        }
      }
    }
  }
  __syncwarp();
  // lower the rows 8 at a time: their D rows read together, the drops sent as atomic
  // min without waiting (a column counts as dropped when the minimum is below the value
  // read; another warp lowering it further in the meantime changed it as well), and
  // the changed-column bookkeeping of the 8 rows done by lanes 0..7 at once
  const int32_t vl = row0 + lane < m ? __ldg(perm + row0 + lane) - 1 : -1;
  for (int l0 = 0; l0 < 32; l0 += 8) {
    T best[8], cur[8];
    int32_t v[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      v[t] = __shfl_sync(kFullB, vl, l0 + t);
      best[t] = sm.acc[(l0 + t) * 32 + lane];
      cur[t] = (v[t] >= 0 && best[t] != Lim<T>::max()) ? __ldcg(D + (int64_t)v[t] * 32 + lane)
                                                        : Lim<T>::max();
    }
    unsigned mine = 0;
    int32_t myv = -1;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const bool dropped = best[t] < cur[t];
      if (dropped) b_atomic_min<T>(D + (int64_t)v[t] * 32 + lane, best[t]);
      const unsigned b = __ballot_sync(kFullB, dropped);
      dropped_cols |= b;
      if (lane == t) {
        mine = b;
        myv = v[t];
      }
    }
    if (mine && myv >= 0 && atomicOr(chg_next + myv, mine) == 0u) {
      atomicAdd(count, 1ull);
      if (cq) cq[atomicAdd(ncq, 1ull)] = myv;
    }
  }
  __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(kMsSellWarps * 32, 4)
    k_ms_round_sell(const int32_t* __restrict__ colval, const void* __restrict__ nz, int tv,
                    const int32_t* __restrict__ perm, int64_t m, const int4* __restrict__ pitems,
                    int64_t nitems, T* D, const unsigned* __restrict__ chg, unsigned* chg_next,
                    unsigned long long* count, unsigned* drop, int32_t* cq,
                    unsigned long long* ncq) {
  extern __shared__ __align__(16) unsigned char ms_smem[];
  unsigned dropped_cols = 0;  // source columns that dropped anywhere (drop, when given)
  const int lane = threadIdx.x & 31;
  MsSellWarpSmem<T>& sm = reinterpret_cast<MsSellWarpSmem<T>*>(ms_smem)[threadIdx.x >> 5];
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int4 dn = gw < nitems ? __ldg(pitems + gw) : make_int4(0, 0, 0, 0);
  for (int64_t it = gw; it < nitems; it += nw) {
    const int4 d = dn;  // first position, first stored row, columns (or -slices), partial
    if (it + nw < nitems) dn = __ldg(pitems + it + nw);
    if (d.z < 0) {  // -d.z narrow slices, widths in 4-bit fields of d.w
      int64_t pos = d.x;
      for (int t = 0; t < -d.z; ++t) {
        const int w = (int)(((uint32_t)d.w >> (4 * t)) & 15u);
        ms_sell_slice<T>(colval, nz, tv, pos, w, (int64_t)d.y + t * 32, m, perm, D, chg, chg_next,
                         count, cq, ncq, lane, sm, dropped_cols);
        pos += (int64_t)w * 32;
      }
    } else {
      ms_sell_slice<T>(colval, nz, tv, d.x, d.z, d.y, m, perm, D, chg, chg_next, count, cq, ncq,
                       lane, sm, dropped_cols);
    }
  }
  if (drop && lane == 0 && dropped_cols) atomicOr(drop, dropped_cols);
}

// hub pieces: one warp per piece, atomic min into the hub's 32 columns
// (with mark given, only hubs marked for this round are relaxed)
template <typename T>
__global__ void __launch_bounds__(256)
    k_ms_round_hub(BatchGraph g, const int4* __restrict__ pieces, int64_t npiece,
                   const int32_t* __restrict__ hubs, T* D, const unsigned* __restrict__ chg,
                   unsigned* chg_next, unsigned long long* count, unsigned* drop,
                   const unsigned* __restrict__ mark, int32_t* cq, unsigned long long* ncq) {
  const int lane = threadIdx.x & 31;
  unsigned dropped_cols = 0;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < npiece;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int4 p = pieces[i];
    const int64_t v = hubs[p.x];
    if (mark && !((__ldcg(mark + (v >> 5)) >> (v & 31)) & 1u)) continue;
    T best = Lim<T>::max();
    const bool any = bs_pull<T>(g, D, chg, chg_next, p.y, p.z, lane, best);
    bool dropped = false;
    if (any) {
      T* dv = D + v * 32 + lane;
      if (best < *dv) dropped = best < b_atomic_min<T>(dv, best);
    }
    const unsigned b = __ballot_sync(kFullB, dropped);
    dropped_cols |= b;
    if (lane == 0 && b) ms_changed(v, b, chg_next, count, cq, ncq);
  }
  if (drop && lane == 0 && dropped_cols) atomicOr(drop, dropped_cols);
}

}  // namespace
}  // namespace gg
