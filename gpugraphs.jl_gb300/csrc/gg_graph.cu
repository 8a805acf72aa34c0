// gg_graph.cu -- BFS (levels and parents) and Bellman-Ford shortest paths of
// GPUGraphs.jl (src/algorithms/bfs.jl, src/algorithms/shortest_path.jl).
//
// The reference runs level-synchronous masked SpMVs on A_T with host-side
// convergence checks.  Its results are properties of the graph alone, so any exact
// method reproduces them:
//  * BFS levels: hop distance along in-edges of A_T whose stored value is odd (the
//    reference tests band(A[v,u], curr[u]) with curr in {0,1}, bfs.jl:52-59).  Here:
//    direction-optimising BFS.  Push steps walk out-edges (the transpose of A_T,
//    built once per matrix) and claim vertices with an atomic OR on a visited
//    bitmap; pull steps scan the in-edges of unvisited vertices against a frontier
//    bitmap with early exit.  While the frontier is small, one CTA runs level after
//    level with only block barriers (high-diameter graphs never leave it).
//  * BFS parents: parent = first frontier column in storage order for CSR
//    (src/spmv/CSR.jl:147-171) or the largest for SELL (GPUGraphs_any = max,
//    algebra.jl:35); every stored edge counts.  Levels over all stored edges, then
//    one pass picks, per reached vertex, the rule's in-neighbour one level up.
//  * Shortest paths: the Jacobi fixpoint d(v) = min(d(v), min_u safe_add(w, d(u)))
//    is order independent for non-negative weights (floating addition is monotone),
//    so a frontier-based Bellman-Ford with atomicMin relaxations gives the same bits.
//    Negative or NaN weights run the reference's Jacobi rounds (min-plus SpMV).
#include <vector>

#include "gg_semiring.cuh"
#include "gg_tma.cuh"

namespace gg {

static const unsigned kFullG = 0xffffffffu;

struct PushCSR {       // out-edges (transpose of A_T), 0-based
  int32_t* rowptr = nullptr;  // n + 1
  int32_t* colval = nullptr;  // target vertex
  void* w = nullptr;          // weights in the distance type (SSSP only)
  int wtype = 0;
  int64_t nnz = 0;
  int64_t max_deg = 0;  // largest out-degree: frontier hubs above kPushHub go to pieces
  bool built = false;
};

struct GraphAux {
  int32_t* vrowptr = nullptr;  // CSR view of A_T in original row order (1-based)
  int32_t* vcolval = nullptr;
  void* vnz = nullptr;
  bool owns_view = false;
  bool flags_ready = false;
  bool all_odd = false;  // every stored value has bit 0 set (Bool true / odd integer)
  bool nonneg = false;   // every stored value is >= 0 and not NaN
  PushCSR push[3];       // 0: odd-valued edges, 1: all edges, 2: all edges + weights
  int64_t max_in_deg = -1;  // largest row of the view (-1: not computed yet)
  double avg_w = -1.0;      // mean stored weight in the distance type (-1: not yet)
  // shortest-path pull rounds of large CSR handles: SELL-32 copy of A_T with rows
  // sorted by length (coalesced column / weight loads, a lane per row)
  gg_mat* pull_sell = nullptr;
};

void free_graph_aux(gg_mat* A) {
  GraphAux* g = A->aux;
  if (!g) return;
  if (g->pull_sell) gg_mat_destroy(g->pull_sell);
  if (g->owns_view) {
    cudaFree(g->vrowptr);
    cudaFree(g->vcolval);
    cudaFree(g->vnz);
  }
  for (int i = 0; i < 3; ++i) {
    if (i == 1 && g->push[1].rowptr == g->push[0].rowptr) continue;
    cudaFree(g->push[i].rowptr);
    cudaFree(g->push[i].colval);
    cudaFree(g->push[i].w);
  }
  delete g;
  A->aux = nullptr;
}

static int gridsz(gg_ctx* ctx, int64_t work, int block = 256) {
  int64_t g = (work + block - 1) / block;
  const int64_t cap = (int64_t)ctx->num_sms * (2048 / block);
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------------
// exclusive scan of int32 counts -> int32 offsets (n + 1 entries, out[0] = base)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int32_t block_incl_scan(int32_t v, int32_t* wsum) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(kFullG, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t s = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(kFullG, s, o);
      if (lane >= o) s += y;
    }
    wsum[lane] = s;
  }
  __syncthreads();
  const int32_t r = x + (w > 0 ? wsum[w - 1] : 0);
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(const int32_t* in, int64_t n, int32_t* out,
                                                      int32_t* bsum) {
  __shared__ int32_t wsum[32];
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  const int32_t v = i < n ? in[i] : 0;
  const int32_t incl = block_incl_scan(v, wsum);
  if (i < n) out[i] = incl - v;
  if (threadIdx.x == 1023) bsum[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int32_t* bsum, int64_t nb, int32_t* total) {
  __shared__ int32_t wsum[32];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
    const int64_t i = b0 + threadIdx.x;
    const int32_t v = i < nb ? bsum[i] : 0;
    const int32_t incl = block_incl_scan(v, wsum);
    const int32_t c = carry;
    if (i < nb) bsum[i] = c + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int32_t* out, int64_t n, const int32_t* bsum, const int32_t* total,
                           int32_t base) {
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += bsum[blockIdx.x] + base;
  if (i == 0) out[n] = *total + base;
}

// out[0..n] = base + exclusive prefix sums of cnt[0..n-1]; out[n] = base + total
int scan_counts(gg_ctx* ctx, const int32_t* cnt, int64_t n, int32_t* out, int32_t base) {
  const int64_t nb = (n + 1023) / 1024;
  int32_t* tmp = nullptr;
  GG_CUDA(cudaMalloc((void**)&tmp, (nb + 2) * sizeof(int32_t)));
  if (n > 0) {
    k_scan_blocks<<<(unsigned)nb, 1024, 0, ctx->stream>>>(cnt, n, out, tmp);
    k_scan_sums<<<1, 1024, 0, ctx->stream>>>(tmp, nb, tmp + nb);
    k_scan_add<<<(unsigned)nb, 1024, 0, ctx->stream>>>(out, n, tmp, tmp + nb, base);
  } else {
    cudaMemcpyAsync(out, &base, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_error(e, "scan");
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ---------------------------------------------------------------------------------
// analysis: CSR view, value flags, push (transpose) structures
// ---------------------------------------------------------------------------------
__global__ void k_value_flags(const void* nz, int tv, int64_t nnz, unsigned* flags) {
  unsigned bad = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x) {
    const Raw r = load_raw(nz, tv, k);
    if (dtype_is_float(tv)) {
      bad |= 1u;  // band has no Float method: never "odd"
      if (!(r.d >= 0.0)) bad |= 2u;
    } else {
      if ((r.i & 1) == 0) bad |= 1u;
      if (r.i < 0) bad |= 2u;
    }
  }
  if (bad) atomicOr(flags, bad);
}

__global__ void k_sell_rowlen(int64_t m, int64_t C, const int32_t* slice_ptr, const int32_t* colval,
                              const int32_t* iperm, int32_t* len) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = iperm[r], s = t / C, o = t - s * C;
    const int64_t i0 = (int64_t)slice_ptr[s] - 1 + o, i1 = (int64_t)slice_ptr[s + 1] - 1;
    int32_t l = 0;
    for (int64_t i = i0; i < i1 && colval[i] != -1; i += C) ++l;
    len[r] = l;
  }
}

__global__ void k_sell_to_csr(int64_t m, int64_t C, const int32_t* slice_ptr, const int32_t* colval,
                              const char* nz, int esz, const int32_t* iperm, const int32_t* rowptr,
                              int32_t* ocol, char* onz) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = iperm[r], s = t / C, o = t - s * C;
    const int64_t i0 = (int64_t)slice_ptr[s] - 1 + o;
    const int64_t d0 = (int64_t)rowptr[r] - 1, len = (int64_t)rowptr[r + 1] - rowptr[r];
    for (int64_t j = 0; j < len; ++j) {
      const int64_t i = i0 + j * C;
      ocol[d0 + j] = colval[i];
      for (int b = 0; b < esz; ++b) onz[(d0 + j) * esz + b] = nz[i * esz + b];
    }
  }
}

__device__ __forceinline__ bool value_odd(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<const uint8_t*>(nz)[k] & 1;
    case GG_INT32: return static_cast<const int32_t*>(nz)[k] & 1;
    case GG_INT64: return static_cast<const int64_t*>(nz)[k] & 1;
  }
  return false;
}

// warp per row of A_T: count (mode 0: odd-valued edges only) out-degree of each column
__global__ void k_tr_count(int64_t n, const int32_t* rp, const int32_t* cv, const void* nz, int tv,
                           int odd_only, int32_t* cnt) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    for (int64_t k = (int64_t)rp[r] - 1 + lane; k < (int64_t)rp[r + 1] - 1; k += 32)
      if (!odd_only || value_odd(nz, tv, k)) atomicAdd(cnt + (cv[k] - 1), 1);
  }
}

template <typename TD>
__global__ void k_tr_scatter(int64_t n, const int32_t* rp, const int32_t* cv, const void* nz,
                             int tv, int odd_only, int32_t* cursor, int32_t* ocol, TD* ow) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    for (int64_t k = (int64_t)rp[r] - 1 + lane; k < (int64_t)rp[r + 1] - 1; k += 32) {
      if (odd_only && !value_odd(nz, tv, k)) continue;
      const int32_t pos = atomicAdd(cursor + (cv[k] - 1), 1);
      ocol[pos] = (int32_t)r;
      if (ow) {
        const Raw v = load_raw(nz, tv, k);
        ow[pos] = dtype_is_float(tv) ? static_cast<TD>(v.d) : static_cast<TD>(v.i);
      }
    }
  }
}

static int dist_type_of(int tv) { return tv == GG_BOOL ? GG_INT32 : tv; }

static int ensure_aux(gg_ctx* ctx, gg_mat* A) {
  if (A->aux && A->aux->flags_ready) return GG_OK;
  GraphAux* g = A->aux ? A->aux : new GraphAux();
  A->aux = g;
  const int64_t n = A->m;
  if (A->format == GG_FMT_CSR) {
    g->vrowptr = A->rowptr;
    g->vcolval = A->colval;
    g->vnz = A->nzval;
    g->owns_view = false;
  } else if (!g->vrowptr) {
    int32_t* len = nullptr;
    const int esz = dtype_size(A->dtype);
    GG_CUDA(cudaMalloc((void**)&len, (n > 0 ? n : 1) * sizeof(int32_t)));
    GG_CUDA(cudaMalloc((void**)&g->vrowptr, (n + 1) * sizeof(int32_t)));
    g->owns_view = true;
    if (n > 0)
      k_sell_rowlen<<<gridsz(ctx, n), 256, 0, ctx->stream>>>(n, A->slice_size, A->slice_ptr,
                                                             A->colval, A->iperm, len);
    int rc = scan_counts(ctx, len, n, g->vrowptr, 1);
    cudaFree(len);
    if (rc) return rc;
    GG_CUDA(cudaMalloc((void**)&g->vcolval, (A->nnz > 0 ? A->nnz : 1) * sizeof(int32_t)));
    GG_CUDA(cudaMalloc(&g->vnz, (A->nnz > 0 ? A->nnz : 1) * esz));
    if (n > 0)
      k_sell_to_csr<<<gridsz(ctx, n), 256, 0, ctx->stream>>>(
          n, A->slice_size, A->slice_ptr, A->colval, static_cast<const char*>(A->nzval), esz,
          A->iperm, g->vrowptr, g->vcolval, static_cast<char*>(g->vnz));
    GG_CUDA(cudaGetLastError());
  }
  GG_CUDA(cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream));
  if (A->nnz > 0)
    k_value_flags<<<gridsz(ctx, A->nnz), 256, 0, ctx->stream>>>(g->vnz, A->dtype, A->nnz, ctx->d_flags);
  GG_CUDA(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  g->all_odd = !(ctx->h_flags[0] & 1u);
  g->nonneg = !(ctx->h_flags[0] & 2u);
  g->flags_ready = true;
  return GG_OK;
}

// CSR view of A_T (1-based) and its value flags, for the batched kernels
static int ensure_push(gg_ctx* ctx, gg_mat* A, int which);

// out-edges of every vertex (transpose of A_T, 0-based, all stored entries)
int push_view(gg_ctx* ctx, gg_mat* A, const int32_t** prow, const int32_t** pcol) {
  GG_CHECK(ensure_push(ctx, A, 1));
  *prow = A->aux->push[1].rowptr;
  *pcol = A->aux->push[1].colval;
  return GG_OK;
}

int graph_view(gg_ctx* ctx, gg_mat* A, const int32_t** rp, const int32_t** cv, const void** nz,
               bool* all_odd, bool* nonneg) {
  GG_CHECK(ensure_aux(ctx, A));
  GraphAux* g = A->aux;
  *rp = g->vrowptr;
  *cv = g->vcolval;
  *nz = g->vnz;
  *all_odd = g->all_odd;
  *nonneg = g->nonneg;
  return GG_OK;
}

// which: 0 odd-valued edges, 1 all edges, 2 all edges with weights in the distance type
__global__ void k_max_deg(int64_t n, const int32_t* __restrict__ rp, unsigned* out) {
  unsigned mx = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const unsigned d = (unsigned)(rp[v + 1] - rp[v]);
    mx = d > mx ? d : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned t = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = t > mx ? t : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(out, mx);
}

static int ensure_push(gg_ctx* ctx, gg_mat* A, int which) {
  GG_CHECK(ensure_aux(ctx, A));
  GraphAux* g = A->aux;
  if (which == 0 && g->all_odd) which = 1;
  PushCSR& P = g->push[which];
  if (P.built) return GG_OK;
  if (which == 1 && g->all_odd && g->push[0].built) {
    P = g->push[0];
    return GG_OK;
  }
  const int64_t n = A->m;
  const int odd_only = which == 0 ? 1 : 0;
  int32_t* cnt = nullptr;
  GG_CUDA(cudaMalloc((void**)&cnt, (n > 0 ? n : 1) * sizeof(int32_t)));
  GG_CUDA(cudaMemsetAsync(cnt, 0, (n > 0 ? n : 1) * sizeof(int32_t), ctx->stream));
  if (n > 0)
    k_tr_count<<<gridsz(ctx, n * 32), 256, 0, ctx->stream>>>(n, g->vrowptr, g->vcolval, g->vnz,
                                                             A->dtype, odd_only, cnt);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMalloc((void**)&P.rowptr, (n + 1) * sizeof(int32_t)));
  int rc = scan_counts(ctx, cnt, n, P.rowptr, 0);
  if (rc) {
    cudaFree(cnt);
    return rc;
  }
  int32_t total = 0;
  GG_CUDA(cudaMemcpy(&total, P.rowptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost));
  P.nnz = total;
  GG_CUDA(cudaMemcpyAsync(cnt, P.rowptr, (n > 0 ? n : 1) * sizeof(int32_t),
                          cudaMemcpyDeviceToDevice, ctx->stream));
  GG_CUDA(cudaMalloc((void**)&P.colval, (total > 0 ? total : 1) * sizeof(int32_t)));
  const int td = dist_type_of(A->dtype);
  if (which == 2) {
    P.wtype = td;
    GG_CUDA(cudaMalloc(&P.w, (total > 0 ? total : 1) * dtype_size(td)));
  }
  if (n > 0) {
    const int grid = gridsz(ctx, n * 32);
    switch (which == 2 ? td : GG_INT32) {
      case GG_INT64:
        k_tr_scatter<int64_t><<<grid, 256, 0, ctx->stream>>>(n, g->vrowptr, g->vcolval, g->vnz, A->dtype,
                                                             odd_only, cnt, P.colval, (int64_t*)P.w);
        break;
      case GG_FLOAT32:
        k_tr_scatter<float><<<grid, 256, 0, ctx->stream>>>(n, g->vrowptr, g->vcolval, g->vnz, A->dtype,
                                                           odd_only, cnt, P.colval, (float*)P.w);
        break;
      case GG_FLOAT64:
        k_tr_scatter<double><<<grid, 256, 0, ctx->stream>>>(n, g->vrowptr, g->vcolval, g->vnz, A->dtype,
                                                            odd_only, cnt, P.colval, (double*)P.w);
        break;
      default:
        k_tr_scatter<int32_t><<<grid, 256, 0, ctx->stream>>>(n, g->vrowptr, g->vcolval, g->vnz, A->dtype,
                                                             odd_only, cnt, P.colval, (int32_t*)P.w);
    }
  }
  cudaError_t e = cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream);
  if (e == cudaSuccess && n > 0) {
    k_max_deg<<<gridsz(ctx, n), 256, 0, ctx->stream>>>(n, P.rowptr, ctx->d_flags);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(cnt);
  if (e != cudaSuccess) return cuda_error(e, "transpose");
  P.max_deg = ctx->h_flags[0];
  GG_CUDA(cudaGetLastError());
  P.built = true;
  return GG_OK;
}

// ---------------------------------------------------------------------------------
// BFS kernels
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool bit_of(const unsigned* bm, int32_t v) {
  return (bm[v >> 5] >> (v & 31)) & 1u;
}

// counters: [0] next frontier size, [1] sum of out-degrees of the next frontier
struct Counters {
  unsigned long long nf, mf, level, status;
  unsigned long long nh;  // frontier hubs deferred to the piece kernel
  unsigned long long pad[3];
};

// Frontier vertices with more than kPushHub out-edges are not walked by one warp:
// the push kernels defer them to a hub queue, and the hub kernels split each one into
// pieces of kPushPiece edges spread over all warps.
static const int kPushHub = 2048;
static const int kPushPiece = 1024;

// warp-aggregated append of the lanes with `want` into q (full warp must call)
__device__ __forceinline__ void warp_append(bool want, int32_t v, int32_t deg, int32_t* q,
                                            Counters* ctr) {
  const int lane = threadIdx.x & 31;
  const unsigned b = __ballot_sync(kFullG, want);
  if (!b) return;
  int32_t d = want ? deg : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(kFullG, d, o);
  const int leader = __ffs(b) - 1;
  unsigned long long base = 0;
  if (lane == leader) {
    base = atomicAdd(&ctr->nf, (unsigned long long)__popc(b));
    atomicAdd(&ctr->mf, (unsigned long long)d);
  }
  base = __shfl_sync(kFullG, base, leader);
  if (want) q[base + __popc(b & ((1u << lane) - 1u))] = v;
}

__global__ void k_bfs_init(int32_t s, unsigned* visited, int32_t* dist, int32_t* q) {
  visited[s >> 5] |= 1u << (s & 31);
  dist[s] = 0;
  q[0] = s;
}

// top-down level: warp per frontier vertex, lanes over its out-edges
__global__ void __launch_bounds__(256)
    k_bfs_push(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
               const int32_t* __restrict__ q, int64_t nf, int32_t level, unsigned* visited,
               int32_t* dist, int32_t* qn, Counters* ctr, int32_t* hq) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nf;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t u = q[i];
    const int32_t k0 = prow[u], k1 = prow[u + 1];
    if (hq && k1 - k0 > kPushHub) {  // left to k_bfs_push_hub
      if (lane == 0) hq[atomicAdd(&ctr->nh, 1ull)] = u;
      continue;
    }
    for (int32_t base = k0; base < k1; base += 32) {
      const int32_t k = base + lane;
      bool claim = false;
      int32_t w = 0, deg = 0;
      if (k < k1) {
        w = __ldg(pcol + k);
        const unsigned bit = 1u << (w & 31);
        if (!(__ldcg(visited + (w >> 5)) & bit)) claim = !(atomicOr(visited + (w >> 5), bit) & bit);
        if (claim) {
          dist[w] = level;
          deg = prow[w + 1] - prow[w];
        }
      }
      warp_append(claim, w, deg, qn, ctr);
    }
  }
}

// pieces of the deferred frontier hubs: piece p of hub h has the global index
// hoff[h] + p (hoff = exclusive prefix sums of the hubs' piece counts, hoff[nh] = total);
// warp w takes global pieces w, w + nw, ...
__global__ void __launch_bounds__(1024)
    k_hub_offsets(const int32_t* __restrict__ prow, const int32_t* __restrict__ hq,
                  const Counters* hctr, int32_t* hoff) {
  __shared__ int32_t wsum[32];
  __shared__ int32_t carry;
  const int64_t nh = (int64_t)*((volatile const unsigned long long*)&hctr->nh);
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < nh; b0 += 1024) {
    const int64_t i = b0 + threadIdx.x;
    int32_t np = 0;
    if (i < nh) {
      const int32_t u = hq[i];
      np = (prow[u + 1] - prow[u] + kPushPiece - 1) / kPushPiece;
    }
    const int32_t incl = block_incl_scan(np, wsum);
    const int32_t c = carry;
    if (i < nh) hoff[i] = c + incl - np;
    __syncthreads();
    if (threadIdx.x == 1023) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) hoff[nh] = carry;
}

// the hub holding global piece q, searching forward from hub h (q only grows)
__device__ __forceinline__ int64_t hub_of(const int32_t* __restrict__ hoff, int64_t nh, int64_t q,
                                          int64_t h) {
  if (__ldg(hoff + h + 1) > q) return h;
  int64_t lo = h + 1, hi = nh - 1;  // last index with hoff[idx] <= q
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (__ldg(hoff + mid) <= q) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(256)
    k_bfs_push_hub(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                   const int32_t* __restrict__ hq, int32_t level, unsigned* visited,
                   int32_t* dist, int32_t* qn, Counters* ctr, const Counters* hctr,
                   const int32_t* __restrict__ hoff) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nh = (int64_t)*((volatile const unsigned long long*)&hctr->nh);
  if (nh == 0) return;
  const int64_t npieces = hoff[nh];
  int64_t h = 0;
  for (int64_t q = gw; q < npieces; q += nw) {
    h = hub_of(hoff, nh, q, h);
    {
      const int32_t u = hq[h];
      const int32_t k0 = prow[u], k1 = prow[u + 1];
      const int64_t p = q - hoff[h];
      const int32_t kb = k0 + (int32_t)p * kPushPiece;
      const int32_t ke = kb + kPushPiece < k1 ? kb + kPushPiece : k1;
      for (int32_t base = kb; base < ke; base += 32) {
        const int32_t k = base + lane;
        bool claim = false;
        int32_t w = 0, deg = 0;
        if (k < ke) {
          w = __ldg(pcol + k);
          const unsigned bit = 1u << (w & 31);
          if (!(__ldcg(visited + (w >> 5)) & bit)) claim = !(atomicOr(visited + (w >> 5), bit) & bit);
          if (claim) {
            dist[w] = level;
            deg = prow[w + 1] - prow[w];
          }
        }
        warp_append(claim, w, deg, qn, ctr);
      }
    }
  }
}

// bottom-up level: thread per vertex; an unvisited vertex joins when one of its
// in-neighbours (A_T row) is in the frontier bitmap over an active edge
template <bool kOddOnly>
__global__ void __launch_bounds__(256)
    k_bfs_pull(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cv,
               const void* nz, int tv, const unsigned* __restrict__ fb, unsigned* visited,
               int32_t* dist, int32_t level, unsigned* fbn, int32_t* qn, Counters* ctr,
               const int32_t* __restrict__ prow) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t v = base + threadIdx.x;
    bool found = false;
    const unsigned vw = (v < n) ? visited[v >> 5] : ~0u;
    if (v < n && !((vw >> (v & 31)) & 1u)) {
      const int32_t k1 = rp[v + 1] - 1;
      for (int32_t k = rp[v] - 1; k < k1; ++k) {
        const int32_t u = __ldg(cv + k) - 1;
        if (bit_of(fb, u) && (!kOddOnly || value_odd(nz, tv, k))) {
          found = true;
          break;
        }
      }
    }
    const unsigned bal = __ballot_sync(kFullG, found);
    if (found) dist[v] = level;
    if (lane == 0 && bal) {
      const int64_t word = v >> 5;  // the warp's 32 vertices share one bitmap word
      visited[word] = vw | bal;
      fbn[word] = bal;
    }
    warp_append(found, (int32_t)v, found ? prow[v + 1] - prow[v] : 0, qn, ctr);
  }
}

__global__ void k_queue_to_bitmap(const int32_t* q, int64_t nf, unsigned* bm) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = q[i];
    atomicOr(bm + (v >> 5), 1u << (v & 31));
  }
}

// light frontier vertices (<= kLightDeg out-edges) are processed kBatch per thread
// with all their edge loads, then all their atomics, in flight together; heavier
// vertices go to a warp-per-vertex pass.  This keeps the per-level dependent chain
// at a few memory round trips, which bounds high-diameter searches.
static const int kLightDeg = 4;
static const int kBatch = 4;
static const int kHubDeg = 1024;  // beyond this a frontier vertex gets the whole block

// The single-CTA kernels stop once a frontier's out-edges exceed kSmallEdges (a hub
// reached early would otherwise be walked by one SM): the frontier and its edge count
// go back to the host, whose grid-wide kernels take over.
static const unsigned long long kSmallEdges = 8192;


// appends w to the next frontier; `edges` (per thread) sums the out-degrees appended
__device__ __forceinline__ void small_append(int32_t w, int32_t* nxt, int32_t* qg, int32_t cap,
                                             int32_t* s_nn, const int32_t* __restrict__ prow,
                                             unsigned long long& edges) {
  const int32_t pos = atomicAdd(s_nn, 1);
  if (pos < cap) nxt[pos] = w;
  else qg[pos] = w;
  edges += (unsigned long long)(__ldg(prow + w + 1) - __ldg(prow + w));
}

// adds every thread's `edges` into *s_ne (one shared atomic per warp; all threads)
__device__ __forceinline__ void small_edges_flush(unsigned long long& edges, unsigned long long* s_ne) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) edges += __shfl_xor_sync(0xffffffffu, edges, o);
  if ((threadIdx.x & 31) == 0 && edges) atomicAdd(s_ne, edges);
  edges = 0;
}

// out-edges of the first nf vertices of q, summed into *s_ne (block-wide)
__device__ __forceinline__ void small_edges(const int32_t* q, int32_t nf,
                                            const int32_t* __restrict__ prow,
                                            unsigned long long* s_ne) {
  unsigned long long e = 0;
  for (int32_t i = threadIdx.x; i < nf; i += blockDim.x)
    e += (unsigned long long)(__ldg(prow + q[i] + 1) - __ldg(prow + q[i]));
  small_edges_flush(e, s_ne);
}

// Small-frontier BFS: one CTA runs top-down levels back to back while the frontier
// fits in shared memory.  qg holds the starting frontier (nf0 <= cap) and receives
// the overflowing frontier when it grows past cap.  Out: ctr->nf = size of the last
// discovered frontier (0 when the search is finished), ctr->level = its level.
__global__ void __launch_bounds__(1024)
    k_bfs_small(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol, int32_t* qg,
                int32_t nf0, int32_t level0, int32_t cap, unsigned* visited, int32_t* dist,
                Counters* ctr, unsigned long long budget) {
  extern __shared__ int32_t smem[];
  int32_t* cur = smem;
  int32_t* nxt = smem + cap;
  int32_t* heavy = smem + 2 * cap;
  __shared__ int32_t s_nn, s_nh;
  __shared__ unsigned long long s_ne;
  unsigned long long edges = 0;  // out-degrees this thread appended in the current level
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) s_ne = 0;
  for (int32_t i = threadIdx.x; i < nf0; i += blockDim.x) cur[i] = qg[i];
  int32_t nf = nf0, level = level0;
  __syncthreads();
  small_edges(cur, nf0, prow, &s_ne);
  __syncthreads();
  if (s_ne > budget) {  // the starting frontier is already too heavy for one CTA
    if (threadIdx.x == 0) {
      ctr->nf = (unsigned long long)nf0;
      ctr->mf = s_ne;
      ctr->level = (unsigned long long)level0;
    }
    return;
  }
  __syncthreads();
  for (;;) {
    ++level;
    if (threadIdx.x == 0) {
      s_nn = 0;
      s_nh = 0;
      s_ne = 0;
    }
    __syncthreads();
    for (int32_t i0 = threadIdx.x; i0 < nf; i0 += blockDim.x * kBatch) {
      int32_t k0[kBatch], k1[kBatch];
#pragma unroll
      for (int b = 0; b < kBatch; ++b) {
        const int32_t i = i0 + b * (int32_t)blockDim.x;
        k0[b] = 0;
        k1[b] = 0;
        if (i < nf) {
          const int32_t u = cur[i];
          k0[b] = __ldg(prow + u);
          k1[b] = __ldg(prow + u + 1);
          if (k1[b] - k0[b] > kLightDeg) {
            heavy[atomicAdd(&s_nh, 1)] = u;
            k1[b] = k0[b];
          }
        }
      }
      int32_t w[kBatch][kLightDeg];
      unsigned old[kBatch][kLightDeg];
#pragma unroll
      for (int b = 0; b < kBatch; ++b)
#pragma unroll
        for (int j = 0; j < kLightDeg; ++j)
          w[b][j] = (k0[b] + j < k1[b]) ? __ldg(pcol + k0[b] + j) : -1;
#pragma unroll
      for (int b = 0; b < kBatch; ++b)
#pragma unroll
        for (int j = 0; j < kLightDeg; ++j)
          old[b][j] = (w[b][j] >= 0) ? atomicOr(visited + (w[b][j] >> 5), 1u << (w[b][j] & 31)) : ~0u;
#pragma unroll
      for (int b = 0; b < kBatch; ++b)
#pragma unroll
        for (int j = 0; j < kLightDeg; ++j)
          if (w[b][j] >= 0 && !((old[b][j] >> (w[b][j] & 31)) & 1u)) {
            dist[w[b][j]] = level;
            small_append(w[b][j], nxt, qg, cap, &s_nn, prow, edges);
          }
    }
    __syncthreads();
    const int32_t nh = s_nh;
    // heavy vertices: a warp each up to kHubDeg out-edges, the whole block beyond
    for (int32_t h = warp; h < nh; h += nwarps) {
      const int32_t u = heavy[h];
      const int32_t k0 = __ldg(prow + u), k1 = __ldg(prow + u + 1);
      if (k1 - k0 > kHubDeg) continue;
      for (int32_t k = k0 + lane; k < k1; k += 32) {
        const int32_t w = __ldg(pcol + k);
        const unsigned bit = 1u << (w & 31);
        if (atomicOr(visited + (w >> 5), bit) & bit) continue;
        dist[w] = level;
        small_append(w, nxt, qg, cap, &s_nn, prow, edges);
      }
    }
    for (int32_t h = 0; h < nh; ++h) {
      const int32_t u = heavy[h];
      const int32_t k0 = __ldg(prow + u), k1 = __ldg(prow + u + 1);
      if (k1 - k0 <= kHubDeg) continue;
      for (int32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int32_t w = __ldg(pcol + k);
        const unsigned bit = 1u << (w & 31);
        if (atomicOr(visited + (w >> 5), bit) & bit) continue;
        dist[w] = level;
        small_append(w, nxt, qg, cap, &s_nn, prow, edges);
      }
    }
    small_edges_flush(edges, &s_ne);
    __syncthreads();
    const int32_t nn = s_nn;
    const unsigned long long ne = s_ne;
    if (nn == 0 || nn > cap || ne > budget) {
      for (int32_t i = threadIdx.x; i < (nn < cap ? nn : cap); i += blockDim.x) qg[i] = nxt[i];
      if (threadIdx.x == 0) {
        ctr->nf = (unsigned long long)nn;
        ctr->mf = ne;
        ctr->level = (unsigned long long)level;
      }
      return;
    }
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
    nf = nn;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// Persistent cooperative levels for graphs without hubs (grids, meshes: out-degree
// <= kCoopMaxDeg) while the frontier is medium-sized: one launch runs level after
// level over all SMs with a grid barrier in between, instead of one launch and one
// host round trip per level.  The barrier's wait is bounded (by default 2^26 polls of
// 100 ns, about 7 s; gg_set_wait_limit sets another count): when it runs out, the
// kernel records an error, every block returns, and the call reports GG_ERR_TIMEOUT.  Queue counters rotate over three words so that the counter being
// zeroed is never the one being read or appended.
// ---------------------------------------------------------------------------------
static const int kCoopMaxDeg = 64;
static const int kCoopLo = 1024;   // the single-CTA kernel takes smaller frontiers
static const int kCoopThreads = 1024;
static const double kNearFarScale = 32.0;  // near-far band width = this x the mean weight

struct CoopCtl {
  unsigned long long cnt[3];
  unsigned bar[4];  // arrivals, generation, error, poll limit of the barrier's waits
  long long nf_out;
  int level_out;    // last completed level / round (relative for SSSP)
  int which_out;    // queue holding the remaining frontier: 0 = first, 1 = second
};

__device__ __forceinline__ bool coop_grid_sync(unsigned* bar, unsigned nblocks) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = bar + 1;
    volatile unsigned* verr = bar + 2;
    const unsigned gen = *vgen;
    const unsigned long long limit = bar[3];  // set by the control block's init kernel
    __threadfence();
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      bar[0] = 0;
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned long long polls = 0;
      while (*vgen == gen && *verr == 0) {
        if (++polls > limit) {
          atomicExch(bar + 2, 1u);
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *((volatile unsigned*)(bar + 2)) == 0;
}

__global__ void k_coop_init(CoopCtl* cc, long long nf0, unsigned polls) {
  cc->cnt[0] = 0;
  cc->cnt[1] = 0;
  cc->cnt[2] = (unsigned long long)nf0;
  cc->bar[0] = cc->bar[1] = cc->bar[2] = 0;
  cc->bar[3] = polls;
  cc->nf_out = 0;
  cc->level_out = 0;
  cc->which_out = 0;
}

// warp-aggregated append to a queue counted by *cnt (full warp must call)
__device__ __forceinline__ void coop_append(bool want, int32_t v, int32_t* q,
                                            unsigned long long* cnt) {
  const int lane = threadIdx.x & 31;
  const unsigned b = __ballot_sync(kFullG, want);
  if (!b) return;
  const int leader = __ffs(b) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(cnt, (unsigned long long)__popc(b));
  base = __shfl_sync(kFullG, base, leader);
  if (want) q[base + __popc(b & ((1u << lane) - 1u))] = v;
}

// BFS levels, thread per frontier vertex; exits when the frontier is empty, at most
// lo, or above hi
__global__ void __launch_bounds__(kCoopThreads, 1)
    k_bfs_coop(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol, int32_t* qa,
               int32_t* qb, unsigned* visited, int32_t* dist, CoopCtl* cc, int32_t level0,
               long long lo, long long hi) {
  const int lane = threadIdx.x & 31;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  int32_t* cur = qa;
  int32_t* nxt = qb;
  for (int st = 0;; ++st) {
    const int r = st % 3;
    const long long nf = (long long)*((volatile unsigned long long*)&cc->cnt[(r + 2) % 3]);
    if (nf == 0 || nf <= lo || nf > hi) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        cc->nf_out = nf;
        cc->level_out = level0 + st;
        cc->which_out = st & 1;
      }
      return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cc->cnt[(r + 1) % 3] = 0;
    const int32_t level = level0 + st + 1;
    for (int64_t i0 = gt - lane; i0 < nf; i0 += nt) {  // warp-uniform trip count
      const int64_t i = i0 + lane;
      int32_t k0 = 0, k1 = 0;
      if (i < nf) {
        const int32_t u = cur[i];
        k0 = __ldg(prow + u);
        k1 = __ldg(prow + u + 1);
      }
      int32_t dmax = k1 - k0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int32_t t = __shfl_xor_sync(kFullG, dmax, o);
        dmax = t > dmax ? t : dmax;
      }
      for (int32_t j = 0; j < dmax; ++j) {
        bool claim = false;
        int32_t w = 0;
        if (k0 + j < k1) {
          w = __ldg(pcol + k0 + j);
          const unsigned bit = 1u << (w & 31);
          if (!(__ldcg(visited + (w >> 5)) & bit)) claim = !(atomicOr(visited + (w >> 5), bit) & bit);
          if (claim) dist[w] = level;
        }
        coop_append(claim, w, nxt, &cc->cnt[r]);
      }
    }
    if (!coop_grid_sync(cc->bar, gridDim.x)) return;
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
  }
}

// BFS levels of hub-free graphs on one thread-block cluster: kClusterCtas CTAs (8 SMs)
// run level after level separated by the cluster barrier (barrier.cluster, a hardware
// barrier: no polling), which costs far less than a grid barrier over every SM.  It
// serves the long tail of small frontiers of high-diameter graphs (a 4096 x 4096 grid
// has 7439 levels of at most ~8000 vertices); it exits when the frontier is empty or
// larger than cap.  The frontier never leaves the cluster: every CTA keeps the
// vertices it claimed in its own shared memory, the CTAs read each other's queues and
// counts through distributed shared memory (mapa + ld.shared::cluster), and the
// barrier's release / acquire orders them -- a level costs the L2 round trips of its
// row pointers, columns and visited bits, not also a queue and counter in global
// memory and a fence.  A CTA's claims past kStageCap spill to qb (global counter
// cc->cnt[1]) and end the kernel after that level.  On exit the frontier is written
// to qa (CTA shares in rank order, then the spills).
static const int kClusterCtas = 8;
static const long long kClusterCap = 32768;
static const int kStageCap = 4096;  // per-CTA queue (kClusterCap / kClusterCtas)
static const int kSpillBit = 1 << 30;

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}
__device__ __forceinline__ uint32_t dsmem_addr(const void* p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ int32_t dsmem_ld(uint32_t a) {
  int32_t v;
  asm volatile("ld.shared::cluster.b32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}

// appends to the CTA's queue (one shared atomic per warp); claims past kStageCap go to
// the spill queue (one global atomic per warp) and mark the count with kSpillBit
__device__ __forceinline__ void stage_append(bool want, int32_t v, int32_t* sbuf, int* scnt,
                                             int32_t* spill, unsigned long long* nspill) {
  const int lane = threadIdx.x & 31;
  const unsigned b = __ballot_sync(kFullG, want);
  if (!b) return;
  const int leader = __ffs(b) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(scnt, __popc(b)) & (kSpillBit - 1);
  base = __shfl_sync(kFullG, base, leader);
  const int pos = base + __popc(b & ((1u << lane) - 1u));
  const bool fits = pos < kStageCap;
  if (want && fits) sbuf[pos] = v;
  const unsigned over = __ballot_sync(kFullG, want && !fits);
  if (!over) return;
  const int l2 = __ffs(over) - 1;
  unsigned long long gbase = 0;
  if (lane == l2) {
    gbase = atomicAdd(nspill, (unsigned long long)__popc(over));
    atomicOr(scnt, kSpillBit);
  }
  gbase = __shfl_sync(kFullG, gbase, l2);
  if (want && !fits) spill[gbase + __popc(over & ((1u << lane) - 1u))] = v;
}

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kCoopThreads, 1)
    k_bfs_cluster(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol, int32_t* qa,
                  int32_t* qb, unsigned* visited, int32_t* dist, CoopCtl* cc, int32_t level0,
                  long long cap) {
  __shared__ int32_t sq[2][kStageCap];
  __shared__ int s_cnt[2];
  __shared__ int s_pre[kClusterCtas + 1];
  __shared__ int s_spill;
  const int rank = blockIdx.x;  // the grid is one cluster
  const int lane = threadIdx.x & 31;
  const int64_t gt = (int64_t)rank * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)kClusterCtas * blockDim.x;
  {  // an even share of the starting frontier (at most kClusterCap) per CTA
    const long long nf0 = (long long)*((volatile unsigned long long*)&cc->cnt[2]);
    const long long lo = nf0 * rank / kClusterCtas, hi = nf0 * (rank + 1) / kClusterCtas;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) sq[0][i - lo] = qa[i];
    if (threadIdx.x == 0) {
      s_cnt[0] = (int)(hi - lo);
      s_cnt[1] = 0;
    }
  }
  cluster_barrier();
  for (int st = 0;; ++st) {
    const int p = st & 1;
    // every CTA's count of this level's frontier, through distributed shared memory
    if (threadIdx.x < kClusterCtas) s_pre[threadIdx.x + 1] = dsmem_ld(dsmem_addr(&s_cnt[p], threadIdx.x));
    __syncthreads();
    if (threadIdx.x == 0) {
      int sp = 0;
      s_pre[0] = 0;
      for (int c = 0; c < kClusterCtas; ++c) {
        const int v = s_pre[c + 1];
        sp |= v & kSpillBit;
        const int k = v & (kSpillBit - 1);
        s_pre[c + 1] = s_pre[c] + (k < kStageCap ? k : kStageCap);
      }
      s_spill = sp;
      s_cnt[p ^ 1] = 0;  // next level's queue (nobody reads it during this level)
    }
    __syncthreads();
    const long long nsp = s_spill ? (long long)*((volatile unsigned long long*)&cc->cnt[1]) : 0;
    const long long nf = (long long)s_pre[kClusterCtas] + nsp;
    if (nf == 0 || nf > cap || s_spill) {
      const int mine = s_pre[rank + 1] - s_pre[rank];
      for (int i = threadIdx.x; i < mine; i += blockDim.x) qa[s_pre[rank] + i] = sq[p][i];
      for (long long i = gt; i < nsp; i += nt) qa[s_pre[kClusterCtas] + i] = qb[i];
      if (rank == 0 && threadIdx.x == 0) {
        cc->nf_out = nf;
        cc->level_out = level0 + st;
        cc->which_out = 0;
      }
      cluster_barrier();  // no CTA leaves while another may still read its queue
      return;
    }
    const int32_t level = level0 + st + 1;
    int32_t* nxt = sq[p ^ 1];
    for (int64_t i0 = gt - lane; i0 < nf; i0 += nt) {
      const int64_t i = i0 + lane;
      int32_t k0 = 0, k1 = 0;
      if (i < nf) {
        int r = 0;
        while (r + 1 < kClusterCtas && s_pre[r + 1] <= i) ++r;
        const int32_t u = dsmem_ld(dsmem_addr(&sq[p][i - s_pre[r]], (uint32_t)r));
        k0 = __ldg(prow + u);
        k1 = __ldg(prow + u + 1);
      }
      int32_t dmax = k1 - k0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int32_t t = __shfl_xor_sync(kFullG, dmax, o);
        dmax = t > dmax ? t : dmax;
      }
      for (int32_t j = 0; j < dmax; ++j) {
        bool claim = false;
        int32_t w = 0;
        if (k0 + j < k1) {
          w = __ldg(pcol + k0 + j);
          const unsigned bit = 1u << (w & 31);
          // claimed by the atomic alone: one L2 round trip on this level's critical path
          claim = !(atomicOr(visited + (w >> 5), bit) & bit);
          if (claim) dist[w] = level;
        }
        stage_append(claim, w, nxt, &s_cnt[p ^ 1], qb, &cc->cnt[1]);
      }
    }
    cluster_barrier();
  }
}

// sum of out-degrees of a frontier queue (direction heuristic after the small kernel)
__global__ void k_queue_degree(const int32_t* __restrict__ prow, const int32_t* __restrict__ q,
                               int64_t nf, Counters* ctr) {
  unsigned long long d = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = q[i];
    d += (unsigned long long)(prow[u + 1] - prow[u]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(kFullG, d, o);
  if ((threadIdx.x & 31) == 0 && d) atomicAdd(&ctr->mf, d);
}

static const int kSmallCap = 8192;
static const int kSmallThreads = 1024;
static const size_t kSmallSmem = 3 * kSmallCap * sizeof(int32_t);

struct BfsScratch {
  unsigned* visited;
  unsigned* fb[2];
  int32_t* q[2];
  int32_t* hq;  // deferred frontier hubs (the first far list of near-far searches)
  int32_t* q2;  // the second far list
  int32_t* q3;  // the third far list
  int32_t* hoff;  // piece offsets of the deferred hubs (k_hub_offsets)
  Counters* ctr;
  CoopCtl* cc;
};

static int bfs_scratch(gg_ctx* ctx, int64_t n, BfsScratch* s) {
  const int64_t nw = (n + 31) / 32 + 1;
  const size_t bm = ((nw * sizeof(unsigned)) + 255) & ~(size_t)255;
  const size_t qb = (((n + 1) * sizeof(int32_t)) + 255) & ~(size_t)255;
  GG_CHECK(ensure_scratch(ctx, 3 * bm + 6 * qb + 512));
  char* p = static_cast<char*>(ctx->scratch);
  s->visited = (unsigned*)p;
  s->fb[0] = (unsigned*)(p + bm);
  s->fb[1] = (unsigned*)(p + 2 * bm);
  s->q[0] = (int32_t*)(p + 3 * bm);
  s->q[1] = (int32_t*)(p + 3 * bm + qb);
  s->hq = (int32_t*)(p + 3 * bm + 2 * qb);
  s->q2 = (int32_t*)(p + 3 * bm + 3 * qb);
  s->q3 = (int32_t*)(p + 3 * bm + 4 * qb);
  s->hoff = (int32_t*)(p + 3 * bm + 5 * qb);
  s->ctr = (Counters*)(p + 3 * bm + 6 * qb);
  s->cc = (CoopCtl*)(p + 3 * bm + 6 * qb + 256);
  GG_CUDA(cudaMemsetAsync(p, 0, 3 * bm, ctx->stream));
  return GG_OK;
}

// cooperative launch of a persistent level kernel, then its control block read back
static int coop_launch(gg_ctx* ctx, const void* fn, void** args, CoopCtl* cc, CoopCtl* h) {
  GG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(ctx->num_sms), dim3(kCoopThreads), args, 0,
                                      ctx->stream));
  GG_CUDA(cudaMemcpyAsync(h, cc, sizeof(CoopCtl), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (h->bar[2]) return set_error(GG_ERR_TIMEOUT, "grid barrier wait ran out");
  return GG_OK;
}

// Runs the BFS from source s (0-based) over the edges selected by `which` (0: odd
// values, 1: all stored); writes level(v) into dist for every reached v.
static int bfs_run(gg_ctx* ctx, gg_mat* A, int32_t s, int which, int32_t* dist,
                   int64_t* levels_out) {
  GG_CHECK(ensure_push(ctx, A, which));
  GraphAux* g = A->aux;
  const bool odd_only = (which == 0 && !g->all_odd);
  PushCSR& P = g->push[(which == 0 && g->all_odd) ? 1 : which];
  const int64_t n = A->m;
  BfsScratch sc;
  GG_CHECK(bfs_scratch(ctx, n, &sc));
  GG_CUDA(cudaFuncSetAttribute(k_bfs_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kSmallSmem));
  k_bfs_init<<<1, 1, 0, ctx->stream>>>(s, sc.visited, dist, sc.q[0]);
  GG_CUDA(cudaGetLastError());
  Counters* h = reinterpret_cast<Counters*>(ctx->h_flags);
  int64_t nf = 1, level = 0, mf = 0, explored = 0;
  int cur = 0;
  bool frontier_is_bitmap = false, pull = false;
  const int64_t total_edges = P.nnz;
  // hub-free graphs (grids, meshes) run medium frontiers in the persistent kernel
  const bool coop_ok = P.max_deg <= kCoopMaxDeg && n >= (1 << 16);
  const int32_t small_cap = coop_ok ? kCoopLo : kSmallCap;
  const long long coop_hi = n / 24 > kCoopLo ? n / 24 : kCoopLo;
  CoopCtl* hc = reinterpret_cast<CoopCtl*>(ctx->h_flags);
  while (nf > 0) {
    if (coop_ok && !pull && nf <= kClusterCap) {
      // small and medium frontiers of hub-free graphs: one cluster, cluster barriers
      k_coop_init<<<1, 1, 0, ctx->stream>>>(sc.cc, nf, barrier_polls(ctx));
      k_bfs_cluster<<<kClusterCtas, kCoopThreads, 0, ctx->stream>>>(
          P.rowptr, P.colval, sc.q[cur], sc.q[cur ^ 1], sc.visited, dist, sc.cc, (int32_t)level,
          kClusterCap);
      GG_CUDA(cudaGetLastError());
      GG_CUDA(cudaMemcpyAsync(hc, sc.cc, sizeof(CoopCtl), cudaMemcpyDeviceToHost, ctx->stream));
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      nf = hc->nf_out;
      level = hc->level_out;
      if (hc->which_out) cur ^= 1;
      if (nf == 0) break;
      GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
      k_queue_degree<<<gridsz(ctx, nf), 256, 0, ctx->stream>>>(P.rowptr, sc.q[cur], nf, sc.ctr);
      GG_CUDA(cudaMemcpyAsync(ctx->h_flags, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost,
                              ctx->stream));
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      mf = (int64_t)reinterpret_cast<Counters*>(ctx->h_flags)->mf;
      hc = reinterpret_cast<CoopCtl*>(ctx->h_flags);
      if (nf <= coop_hi) {
        // larger frontier: the grid-wide persistent kernel takes it from here
        k_coop_init<<<1, 1, 0, ctx->stream>>>(sc.cc, nf, barrier_polls(ctx));
        int32_t* qa = sc.q[cur];
        int32_t* qb = sc.q[cur ^ 1];
        int32_t lv0 = (int32_t)level;
        long long lo = kClusterCap / 2, hi = coop_hi;
        void* args[] = {&P.rowptr, &P.colval, &qa, &qb, &sc.visited, &dist, &sc.cc, &lv0, &lo, &hi};
        GG_CHECK(coop_launch(ctx, (const void*)k_bfs_coop, args, sc.cc, hc));
        nf = hc->nf_out;
        level = hc->level_out;
        if (hc->which_out) cur ^= 1;
        if (nf == 0) break;
        if (nf <= kClusterCap) continue;
        GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
        k_queue_degree<<<gridsz(ctx, nf), 256, 0, ctx->stream>>>(P.rowptr, sc.q[cur], nf, sc.ctr);
        GG_CUDA(cudaMemcpyAsync(ctx->h_flags, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost,
                                ctx->stream));
        GG_CUDA(cudaStreamSynchronize(ctx->stream));
        mf = (int64_t)reinterpret_cast<Counters*>(ctx->h_flags)->mf;
      }
      // frontier above the persistent kernels' range: push / pull levels below
    }
    if (coop_ok && !pull && nf > small_cap && nf <= coop_hi) {
      k_coop_init<<<1, 1, 0, ctx->stream>>>(sc.cc, nf, barrier_polls(ctx));
      int32_t* qa = sc.q[cur];
      int32_t* qb = sc.q[cur ^ 1];
      int32_t lv0 = (int32_t)level;
      long long lo = kCoopLo / 2, hi = coop_hi;
      void* args[] = {&P.rowptr, &P.colval, &qa, &qb, &sc.visited, &dist, &sc.cc, &lv0, &lo, &hi};
      GG_CHECK(coop_launch(ctx, (const void*)k_bfs_coop, args, sc.cc, hc));
      nf = hc->nf_out;
      level = hc->level_out;
      if (hc->which_out) cur ^= 1;
      if (nf > 0) {
        GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
        k_queue_degree<<<gridsz(ctx, nf), 256, 0, ctx->stream>>>(P.rowptr, sc.q[cur], nf, sc.ctr);
        GG_CUDA(cudaMemcpyAsync(ctx->h_flags, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost,
                                ctx->stream));
        GG_CUDA(cudaStreamSynchronize(ctx->stream));
        mf = (int64_t)reinterpret_cast<Counters*>(ctx->h_flags)->mf;
      }
      continue;
    }
    if (!pull && nf <= small_cap && mf <= (int64_t)kSmallEdges) {
      k_bfs_small<<<1, kSmallThreads, kSmallSmem, ctx->stream>>>(
          P.rowptr, P.colval, sc.q[cur], (int32_t)nf, (int32_t)level, small_cap, sc.visited, dist,
          sc.ctr, kSmallEdges);
      GG_CUDA(cudaGetLastError());
      GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      nf = (int64_t)h->nf;
      level = (int64_t)h->level;
      if (nf == 0) break;
      // the frontier of `level` is in q[cur]; its out-degree sum (counted by the kernel)
      // feeds the heuristic and keeps heavy frontiers on the grid-wide kernels
      mf = (int64_t)h->mf;
      explored += mf;
      continue;
    }
    // direction heuristic (Beamer et al.): pull when the frontier's edges outweigh a
    // 1/14 share of the unexplored edges, push again once the frontier is small
    const int64_t unexplored = total_edges - explored > 0 ? total_edges - explored : 0;
    if (!pull && mf * 14 > unexplored) pull = true;
    else if (pull && nf * 24 < n) pull = false;
    ++level;
    GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
    if (pull) {
      if (!frontier_is_bitmap) {
        GG_CUDA(cudaMemsetAsync(sc.fb[cur], 0, ((n + 31) / 32) * sizeof(unsigned), ctx->stream));
        k_queue_to_bitmap<<<gridsz(ctx, nf), 256, 0, ctx->stream>>>(sc.q[cur], nf, sc.fb[cur]);
      }
      GG_CUDA(cudaMemsetAsync(sc.fb[cur ^ 1], 0, ((n + 31) / 32) * sizeof(unsigned), ctx->stream));
      if (odd_only)
        k_bfs_pull<true><<<gridsz(ctx, n), 256, 0, ctx->stream>>>(
            n, g->vrowptr, g->vcolval, g->vnz, A->dtype, sc.fb[cur], sc.visited, dist,
            (int32_t)level, sc.fb[cur ^ 1], sc.q[cur ^ 1], sc.ctr, P.rowptr);
      else
        k_bfs_pull<false><<<gridsz(ctx, n), 256, 0, ctx->stream>>>(
            n, g->vrowptr, g->vcolval, g->vnz, A->dtype, sc.fb[cur], sc.visited, dist,
            (int32_t)level, sc.fb[cur ^ 1], sc.q[cur ^ 1], sc.ctr, P.rowptr);
      frontier_is_bitmap = true;
    } else {
      const bool hubs = P.max_deg > kPushHub;
      k_bfs_push<<<gridsz(ctx, nf * 32), 256, 0, ctx->stream>>>(
          P.rowptr, P.colval, sc.q[cur], nf, (int32_t)level, sc.visited, dist, sc.q[cur ^ 1], sc.ctr,
          hubs ? sc.hq : nullptr);
      if (hubs) {
        k_hub_offsets<<<1, 1024, 0, ctx->stream>>>(P.rowptr, sc.hq, sc.ctr, sc.hoff);
        k_bfs_push_hub<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(
            P.rowptr, P.colval, sc.hq, (int32_t)level, sc.visited, dist, sc.q[cur ^ 1], sc.ctr,
            sc.ctr, sc.hoff);
      }
      frontier_is_bitmap = false;
    }
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    nf = (int64_t)h->nf;
    mf = (int64_t)h->mf;
    explored += mf;
    cur ^= 1;  // the queue of the new frontier is always written; its bitmap only by pull levels
  }
  if (levels_out) *levels_out = level;
  return GG_OK;
}

// parents: warp per reached vertex; rule 1 = first qualifying in-neighbour in
// storage order, rule 2 = largest qualifying column
__global__ void __launch_bounds__(256)
    k_bfs_parents(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cv,
                  const int32_t* __restrict__ lev, int32_t source, int rule, int32_t* parents) {
  const int lane = threadIdx.x & 31;
  for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n;
       v += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t lv = lev[v];
    if (lv == INT32_MAX) continue;  // unreached: left untouched (bfs.jl:176)
    if (v == source) {
      if (lane == 0) parents[v] = 0;
      continue;
    }
    const int32_t k0 = rp[v] - 1, k1 = rp[v + 1] - 1;
    int32_t best = 0;
    for (int32_t base = k0; base < k1; base += 32) {
      const int32_t k = base + lane;
      int32_t c = 0;
      if (k < k1) {
        const int32_t col = __ldg(cv + k);
        if (__ldg(lev + col - 1) == lv - 1) c = col;
      }
      if (rule == GG_PARENT_FIRST_IN_ROW) {
        const unsigned b = __ballot_sync(kFullG, c != 0);
        if (b) {
          best = __shfl_sync(kFullG, c, __ffs(b) - 1);
          break;
        }
      } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_xor_sync(kFullG, c, o));
        best = max(best, c);
      }
    }
    if (lane == 0) parents[v] = best;
  }
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// ---------------------------------------------------------------------------------
// SSSP kernels (non-negative weights)
// ---------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T atomic_min_t(T* p, T v);
template <> __device__ __forceinline__ int32_t atomic_min_t<int32_t>(int32_t* p, int32_t v) {
  return atomicMin(p, v);
}
template <> __device__ __forceinline__ int64_t atomic_min_t<int64_t>(int64_t* p, int64_t v) {
  return (int64_t)atomicMin((long long*)p, (long long)v);
}
// non-negative floats order like their bit patterns
template <> __device__ __forceinline__ float atomic_min_t<float>(float* p, float v) {
  return __int_as_float(atomicMin((int*)p, __float_as_int(v)));
}
template <> __device__ __forceinline__ double atomic_min_t<double>(double* p, double v) {
  return __longlong_as_double(atomicMin((long long*)p, __double_as_longlong(v)));
}

template <typename T> __device__ __forceinline__ T ld_cg(const T* p) { return __ldcg(p); }
// coherent-cached load (ld.global.ca): may return a value another SM has since lowered
template <typename T> __device__ __forceinline__ T ld_l1(const T* p) { return __ldca(p); }

// safe_add on non-negative, non-NaN operands (algebra.jl:47-48)
template <typename T> __device__ __forceinline__ T relax_add(T w, T d) {
  return (w == Lim<T>::max() || d == Lim<T>::max()) ? Lim<T>::max() : w_add(w, d);
}

// relax the out-edges of frontier vertices; improved targets join the next frontier
// once (bitmap inq); the frontier vertex's own bit in inq_cur is cleared
template <typename T>
__global__ void __launch_bounds__(256)
    k_sssp_push(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                const T* __restrict__ pw, const int32_t* __restrict__ q, int64_t nf, T* dist,
                unsigned* inq_cur, unsigned* inq_next, int32_t* qn, Counters* ctr, int32_t* hq) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nf;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t u = q[i];
    if (lane == 0) atomicAnd(inq_cur + (u >> 5), ~(1u << (u & 31)));
    const int32_t k0 = prow[u], k1 = prow[u + 1];
    if (hq && k1 - k0 > kPushHub) {  // left to k_sssp_push_hub
      if (lane == 0) hq[atomicAdd(&ctr->nh, 1ull)] = u;
      continue;
    }
    const T du = ld_cg(dist + u);
    for (int32_t base = k0; base < k1; base += 32) {
      const int32_t k = base + lane;
      bool add = false;
      int32_t w = 0;
      if (k < k1) {
        w = __ldg(pcol + k);
        const T cand = relax_add(__ldg(pw + k), du);
        if (cand < ld_cg(dist + w)) {
          const T old = atomic_min_t(dist + w, cand);
          if (cand < old) {
            const unsigned bit = 1u << (w & 31);
            add = !(atomicOr(inq_next + (w >> 5), bit) & bit);
          }
        }
      }
      warp_append(add, w, add ? prow[w + 1] - prow[w] : 0, qn, ctr);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_sssp_push_hub(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                    const T* __restrict__ pw, const int32_t* __restrict__ hq, T* dist,
                    unsigned* inq_next, int32_t* qn, Counters* ctr, const Counters* hctr,
                    const int32_t* __restrict__ hoff) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nh = (int64_t)*((volatile const unsigned long long*)&hctr->nh);
  if (nh == 0) return;
  const int64_t npieces = hoff[nh];
  int64_t h = 0;
  for (int64_t q = gw; q < npieces; q += nw) {
    h = hub_of(hoff, nh, q, h);
    const int32_t u = hq[h];
    const int32_t k0 = prow[u], k1 = prow[u + 1];
    const T du = ld_cg(dist + u);
    {
      const int64_t p = q - hoff[h];
      const int32_t kb = k0 + (int32_t)p * kPushPiece;
      const int32_t ke = kb + kPushPiece < k1 ? kb + kPushPiece : k1;
      for (int32_t base = kb; base < ke; base += 32) {
        const int32_t k = base + lane;
        bool add = false;
        int32_t w = 0;
        if (k < ke) {
          w = __ldg(pcol + k);
          const T cand = relax_add(__ldg(pw + k), du);
          if (cand < ld_cg(dist + w)) {
            const T old = atomic_min_t(dist + w, cand);
            if (cand < old) {
              const unsigned bit = 1u << (w & 31);
              add = !(atomicOr(inq_next + (w >> 5), bit) & bit);
            }
          }
        }
        warp_append(add, w, add ? prow[w + 1] - prow[w] : 0, qn, ctr);
      }
    }
  }
}

// single-CTA rounds while the frontier is small (mirror of k_bfs_small)
template <typename T>
__global__ void __launch_bounds__(1024)
    k_sssp_small(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                 const T* __restrict__ pw, int32_t* qg, int32_t nf0, int32_t cap, T* dist,
                 unsigned* inq_a, unsigned* inq_b, Counters* ctr, int64_t max_rounds,
                 unsigned long long budget) {
  extern __shared__ int32_t smem[];
  int32_t* cur = smem;
  int32_t* nxt = smem + cap;
  int32_t* heavy = smem + 2 * cap;
  __shared__ int32_t s_nn, s_nh;
  __shared__ unsigned long long s_ne;
  unsigned long long edges = 0;  // out-degrees this thread appended in the current level
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) s_ne = 0;
  for (int32_t i = threadIdx.x; i < nf0; i += blockDim.x) cur[i] = qg[i];
  int32_t nf = nf0;
  unsigned* ic = inq_a;
  unsigned* in = inq_b;
  unsigned long long rounds = 0;
  __syncthreads();
  small_edges(cur, nf0, prow, &s_ne);
  __syncthreads();
  if (s_ne > budget) {  // the starting frontier is already too heavy for one CTA
    if (threadIdx.x == 0) {
      ctr->nf = (unsigned long long)nf0;
      ctr->mf = s_ne;
      ctr->level = 0;
      ctr->status = 0;  // its membership bits are still in inq_a
    }
    return;
  }
  __syncthreads();
  for (;;) {
    ++rounds;
    if (threadIdx.x == 0) {
      s_nn = 0;
      s_nh = 0;
      s_ne = 0;
    }
    __syncthreads();
    for (int32_t i0 = threadIdx.x; i0 < nf; i0 += blockDim.x * kBatch) {
      int32_t k0[kBatch], k1[kBatch];
      T du[kBatch];
#pragma unroll
      for (int b = 0; b < kBatch; ++b) {
        const int32_t i = i0 + b * (int32_t)blockDim.x;
        k0[b] = 0;
        k1[b] = 0;
        du[b] = Lim<T>::max();
        if (i < nf) {
          const int32_t u = cur[i];
          atomicAnd(ic + (u >> 5), ~(1u << (u & 31)));
          k0[b] = __ldg(prow + u);
          k1[b] = __ldg(prow + u + 1);
          if (k1[b] - k0[b] > kLightDeg) {
            heavy[atomicAdd(&s_nh, 1)] = u;
            k1[b] = k0[b];
          } else {
            du[b] = ld_cg(dist + u);
          }
        }
      }
      int32_t w[kBatch][kLightDeg];
      T cand[kBatch][kLightDeg];
#pragma unroll
      for (int b = 0; b < kBatch; ++b)
#pragma unroll
        for (int j = 0; j < kLightDeg; ++j) {
          const bool ok = k0[b] + j < k1[b];
          w[b][j] = ok ? __ldg(pcol + k0[b] + j) : -1;
          cand[b][j] = ok ? relax_add(__ldg(pw + k0[b] + j), du[b]) : Lim<T>::max();
        }
#pragma unroll
      for (int b = 0; b < kBatch; ++b)
#pragma unroll
        for (int j = 0; j < kLightDeg; ++j)
          if (w[b][j] >= 0 && !(cand[b][j] < atomic_min_t(dist + w[b][j], cand[b][j]))) w[b][j] = -1;
#pragma unroll
      for (int b = 0; b < kBatch; ++b)
#pragma unroll
        for (int j = 0; j < kLightDeg; ++j)
          if (w[b][j] >= 0) {
            const unsigned bit = 1u << (w[b][j] & 31);
            if (!(atomicOr(in + (w[b][j] >> 5), bit) & bit)) small_append(w[b][j], nxt, qg, cap, &s_nn, prow, edges);
          }
    }
    __syncthreads();
    const int32_t nh = s_nh;
    for (int32_t h = warp; h < nh; h += nwarps) {
      const int32_t u = heavy[h];
      const T du = ld_cg(dist + u);
      const int32_t k0 = __ldg(prow + u), k1 = __ldg(prow + u + 1);
      if (k1 - k0 > kHubDeg) continue;
      for (int32_t k = k0 + lane; k < k1; k += 32) {
        const int32_t w = __ldg(pcol + k);
        const T cand = relax_add(__ldg(pw + k), du);
        if (!(cand < ld_cg(dist + w))) continue;
        if (!(cand < atomic_min_t(dist + w, cand))) continue;
        const unsigned bit = 1u << (w & 31);
        if (atomicOr(in + (w >> 5), bit) & bit) continue;
        small_append(w, nxt, qg, cap, &s_nn, prow, edges);
      }
    }
    for (int32_t h = 0; h < nh; ++h) {
      const int32_t u = heavy[h];
      const int32_t k0 = __ldg(prow + u), k1 = __ldg(prow + u + 1);
      if (k1 - k0 <= kHubDeg) continue;
      const T du = ld_cg(dist + u);
      for (int32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int32_t w = __ldg(pcol + k);
        const T cand = relax_add(__ldg(pw + k), du);
        if (!(cand < ld_cg(dist + w))) continue;
        if (!(cand < atomic_min_t(dist + w, cand))) continue;
        const unsigned bit = 1u << (w & 31);
        if (atomicOr(in + (w >> 5), bit) & bit) continue;
        small_append(w, nxt, qg, cap, &s_nn, prow, edges);
      }
    }
    small_edges_flush(edges, &s_ne);
    __syncthreads();
    const int32_t nn = s_nn;
    const unsigned long long ne = s_ne;
    if (nn == 0 || nn > cap || ne > budget || (max_rounds > 0 && (int64_t)rounds >= max_rounds)) {
      if (nn > cap)
        for (int32_t i = threadIdx.x; i < cap; i += blockDim.x) qg[i] = nxt[i];
      else
        for (int32_t i = threadIdx.x; i < nn; i += blockDim.x) qg[i] = nxt[i];
      if (threadIdx.x == 0) {
        ctr->nf = (unsigned long long)nn;
        ctr->mf = ne;
        ctr->level = rounds;
        ctr->status = (in == inq_b) ? 1ull : 0ull;  // which bitmap holds the frontier bits
      }
      return;
    }
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
    unsigned* tb = ic;
    ic = in;
    in = tb;
    nf = nn;
    __syncthreads();
  }
}

// frontier = every vertex whose start distance is finite
template <typename T>
__global__ void k_sssp_seed(int64_t n, const T* dist, unsigned* inq, int32_t* q, Counters* ctr) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t v = base + threadIdx.x;
    const bool fin = v < n && dist[v] != Lim<T>::max();
    const unsigned bal = __ballot_sync(kFullG, fin);
    if ((threadIdx.x & 31) == 0 && bal) inq[v >> 5] = bal;
    warp_append(fin, (int32_t)v, 0, q, ctr);
  }
}

template <typename T>
__global__ void k_fill_t(T* p, int64_t n, T v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

template <typename T>
__global__ void k_set_source(T* dist, T* next, int64_t s) {
  dist[s] = T(0);
  if (next) next[s] = T(0);
}

// Jacobi helpers for the fallback path
template <typename T>
__global__ void k_changed_copy(int64_t n, const T* next, T* dist, unsigned* flag) {
  unsigned ch = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T a = next[i], b = dist[i];
    if (a < b) ch = 1;
    dist[i] = a;
  }
  if (ch) atomicOr(flag, 1u);
}

// Bellman-Ford rounds (push, atomic min, membership bitmaps), thread per frontier vertex
template <typename T>
__global__ void __launch_bounds__(kCoopThreads, 1)
    k_sssp_coop(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                const T* __restrict__ pw, int32_t* qa, int32_t* qb, T* dist, unsigned* inq_a,
                unsigned* inq_b, CoopCtl* cc, long long lo, long long hi, long long max_rounds) {
  const int lane = threadIdx.x & 31;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  int32_t* cur = qa;
  int32_t* nxt = qb;
  unsigned* icur = inq_a;
  unsigned* inxt = inq_b;
  for (int st = 0;; ++st) {
    const int r = st % 3;
    const long long nf = (long long)*((volatile unsigned long long*)&cc->cnt[(r + 2) % 3]);
    if (nf == 0 || nf <= lo || nf > hi || st >= max_rounds) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        cc->nf_out = nf;
        cc->level_out = st;
        cc->which_out = st & 1;
      }
      return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cc->cnt[(r + 1) % 3] = 0;
    for (int64_t i0 = gt - lane; i0 < nf; i0 += nt) {
      const int64_t i = i0 + lane;
      int32_t k0 = 0, k1 = 0;
      T du = T(0);
      if (i < nf) {
        const int32_t u = cur[i];
        atomicAnd(icur + (u >> 5), ~(1u << (u & 31)));
        k0 = __ldg(prow + u);
        k1 = __ldg(prow + u + 1);
        du = ld_cg(dist + u);
      }
      int32_t dmax = k1 - k0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int32_t t = __shfl_xor_sync(kFullG, dmax, o);
        dmax = t > dmax ? t : dmax;
      }
      for (int32_t j = 0; j < dmax; ++j) {
        bool add = false;
        int32_t w = 0;
        if (k0 + j < k1) {
          w = __ldg(pcol + k0 + j);
          const T cand = relax_add(__ldg(pw + k0 + j), du);
          if (cand < ld_cg(dist + w)) {
            const T old = atomic_min_t(dist + w, cand);
            if (cand < old) {
              const unsigned bit = 1u << (w & 31);
              add = !(atomicOr(inxt + (w >> 5), bit) & bit);
            }
          }
        }
        coop_append(add, w, nxt, &cc->cnt[r]);
      }
    }
    if (!coop_grid_sync(cc->bar, gridDim.x)) return;
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
    unsigned* tb = icur;
    icur = inxt;
    inxt = tb;
  }
}

// Whole shortest-path search for hub-free graphs in one persistent cooperative
// launch, near-far ordered: only vertices whose tentative distance is below the
// threshold thr are relaxed ("near"); improved vertices at or above it wait in the far
// list; when the near frontier empties, thr grows by delta and the far list is split.
// On high-diameter graphs with spread weights this avoids most of the repeated
// relaxations of plain rounds.  The fixpoint is the same (min over paths of the
// left-folded sums; every improved vertex is relaxed again eventually).  Grid
// barriers are bounded (coop_grid_sync); the number of steps is bounded by max_steps.
struct NfCtl {
  unsigned long long cnt[3];  // near queue lengths, rotating as in CoopCtl
  unsigned long long fcnt[3];  // far list lengths (three lists in rotation)
  unsigned bar[4];
  long long steps_out;
  int status;  // 1 finished, 2 step budget exhausted
};

__global__ void k_nf_init(NfCtl* cc, long long nf0, unsigned polls) {
  cc->cnt[0] = 0;
  cc->cnt[1] = 0;
  cc->cnt[2] = (unsigned long long)nf0;
  cc->fcnt[0] = cc->fcnt[1] = cc->fcnt[2] = 0;
  cc->bar[0] = cc->bar[1] = cc->bar[2] = 0;
  cc->bar[3] = polls;  // poll limit of the barrier's waits
  cc->steps_out = 0;
  cc->status = 0;
}

template <typename T>
__global__ void __launch_bounds__(kCoopThreads, 1)
    k_sssp_nearfar(const int32_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                   const T* __restrict__ pw, int32_t* qa, int32_t* qb, int32_t* fa, int32_t* fb,
                   int32_t* fz, T* dist, unsigned* inq_a, unsigned* inq_b, unsigned* infar,
                   NfCtl* cc, T delta, long long max_steps) {
  const int lane = threadIdx.x & 31;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  int32_t* cur = qa;
  int32_t* nxt = qb;
  unsigned* icur = inq_a;
  unsigned* inxt = inq_b;
  // three far lists in rotation: steps append to list fc; a band change reads list fc
  // and writes the remainder to list fc + 1; every step zeroes the counter of list
  // fc + 2, which nobody touches before it is next written
  int32_t* const fl[3] = {fa, fb, fz};
  int fc = 0;
  T thr = delta;
  for (long long st = 0;; ++st) {
    const int r = (int)(st % 3);
    const long long nf = (long long)*((volatile unsigned long long*)&cc->cnt[(r + 2) % 3]);
    if (st >= max_steps) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        cc->steps_out = st;
        cc->status = 2;
      }
      return;
    }
    if (nf == 0) {
      const long long nfar = (long long)*((volatile unsigned long long*)&cc->fcnt[fc]);
      const int fn = fc == 2 ? 0 : fc + 1;
      if (nfar == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          cc->steps_out = st;
          cc->status = 1;
        }
        return;
      }
      // next distance band: far vertices below the new threshold become the next
      // frontier (counted and marked like a normal step's output), the others move to
      // the other far list
      thr = thr > Lim<T>::max() - delta ? Lim<T>::max() : w_add(thr, delta);
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        cc->cnt[(r + 1) % 3] = 0;
        cc->fcnt[(fc + 2) % 3] = 0;
      }
      for (int64_t i0 = gt - lane; i0 < nfar; i0 += nt) {
        const int64_t i = i0 + lane;
        bool to_near = false, to_far = false;
        int32_t v = 0;
        if (i < nfar) {
          v = fl[fc][i];
          if (ld_cg(dist + v) < thr) {
            atomicAnd(infar + (v >> 5), ~(1u << (v & 31)));
            const unsigned bit = 1u << (v & 31);
            to_near = !(atomicOr(inxt + (v >> 5), bit) & bit);
          } else {
            to_far = true;
          }
        }
        coop_append(to_near, v, nxt, &cc->cnt[r]);
        coop_append(to_far, v, fl[fn], &cc->fcnt[fn]);
      }
      if (!coop_grid_sync(cc->bar, gridDim.x)) return;
      int32_t* t = cur;
      cur = nxt;
      nxt = t;
      unsigned* tb = icur;
      icur = inxt;
      inxt = tb;
      fc = fn;
      continue;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      cc->cnt[(r + 1) % 3] = 0;
      cc->fcnt[(fc + 2) % 3] = 0;
    }
    for (int64_t i0 = gt - lane; i0 < nf; i0 += nt) {
      const int64_t i = i0 + lane;
      int32_t k0 = 0, k1 = 0;
      T du = T(0);
      if (i < nf) {
        const int32_t u = cur[i];
        atomicAnd(icur + (u >> 5), ~(1u << (u & 31)));
        k0 = __ldg(prow + u);
        k1 = __ldg(prow + u + 1);
        du = ld_cg(dist + u);
      }
      int32_t dmax = k1 - k0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int32_t t = __shfl_xor_sync(kFullG, dmax, o);
        dmax = t > dmax ? t : dmax;
      }
      for (int32_t j = 0; j < dmax; ++j) {
        bool near_add = false, far_add = false;
        int32_t w = 0;
        if (k0 + j < k1) {
          w = __ldg(pcol + k0 + j);
          const T cand = relax_add(__ldg(pw + k0 + j), du);
          if (cand < ld_cg(dist + w)) {
            const T old = atomic_min_t(dist + w, cand);
            if (cand < old) {
              const unsigned bit = 1u << (w & 31);
              if (cand < thr) near_add = !(atomicOr(inxt + (w >> 5), bit) & bit);
              else far_add = !(atomicOr(infar + (w >> 5), bit) & bit);
            }
          }
        }
        coop_append(near_add, w, nxt, &cc->cnt[r]);
        coop_append(far_add, w, fl[fc], &cc->fcnt[fc]);
      }
    }
    if (!coop_grid_sync(cc->bar, gridDim.x)) return;
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
    unsigned* tb = icur;
    icur = inxt;
    inxt = tb;
  }
}

template <typename T>
__global__ void k_sum_weights(const T* __restrict__ w, int64_t nnz, double* out) {
  double s = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x)
    s += (double)w[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFullG, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// ---------------------------------------------------------------------------------
// pull rounds for large frontiers: every vertex takes the minimum over its in-edges
// from vertices that changed in the previous round (membership bitmap chg), in place.
// Only v's own lane writes dist[v], so no atomics; the new membership bitmap is
// written word by word from a ballot.  Rows with more than kHubDegB in-edges are
// skipped and relaxed in pieces with atomic min by k_sssp_pull_hub.
// ---------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T view_weight(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<T>(static_cast<const uint8_t*>(nz)[k]);
    case GG_INT32: return static_cast<T>(static_cast<const int32_t*>(nz)[k]);
    case GG_INT64: return static_cast<T>(static_cast<const int64_t*>(nz)[k]);
    case GG_FLOAT32: return static_cast<T>(static_cast<const float*>(nz)[k]);
  }
  return static_cast<T>(static_cast<const double*>(nz)[k]);
}

template <typename T>
__device__ __forceinline__ T warp_min_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T t = __shfl_xor_sync(kFullG, v, o);
    v = t < v ? t : v;
  }
  return v;
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_sssp_pull(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cv,
                const void* nz, int tv, const unsigned* __restrict__ chg, T* dist,
                unsigned* chg_next, int32_t* qn, Counters* ctr, const int32_t* __restrict__ prow) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t v = base + threadIdx.x;
    int64_t k0 = 0, k1 = 0;
    if (v < n) {
      k0 = (int64_t)rp[v] - 1;
      k1 = (int64_t)rp[v + 1] - 1;
    }
    const bool hub = k1 - k0 > kHubDegB;  // relaxed by k_sssp_pull_hub
    T best = Lim<T>::max();
    if (v < n && !hub && k1 - k0 <= 32) {
      // 8 in-edges at a time: their columns, membership bits and (weight, distance)
      // pairs are each loaded together, so a row costs ceil(deg / 8) load chains
      for (int64_t kb = k0; kb < k1; kb += 8) {
        int32_t u[8];
        bool on[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) u[t] = kb + t < k1 ? __ldg(cv + kb + t) - 1 : -1;
#pragma unroll
        for (int t = 0; t < 8; ++t) on[t] = u[t] >= 0 && bit_of(chg, u[t]);
        T c[8];
#pragma unroll
        for (int t = 0; t < 8; ++t)
          c[t] = on[t] ? relax_add(view_weight<T>(nz, tv, kb + t), ld_cg(dist + u[t])) : Lim<T>::max();
#pragma unroll
        for (int t = 0; t < 8; ++t) best = c[t] < best ? c[t] : best;
      }
    }
    // rows of 33..kHubDegB in-edges are left to k_sssp_pull_mid (a warp each, spread
    // over the grid): done here by the vertex's own warp, R-MAT's long rows (low vertex
    // ids) kept a few SMs busy long after the others had finished
    bool changed = false;
    if (v < n && !hub && k1 - k0 <= 32 && best < dist[v]) {
      dist[v] = best;
      changed = true;
    }
    const unsigned word = __ballot_sync(kFullG, changed);
    if (lane == 0 && base + threadIdx.x - lane < n) chg_next[v >> 5] = word;
    warp_append(changed, (int32_t)v, changed ? prow[v + 1] - prow[v] : 0, qn, ctr);
  }
}

// rows of 33..kHubDegB in-edges of a pull round (the hub plan's mid list, longest
// first): a warp takes 32 of them, scans each with the whole warp (128 in-edges per
// step, loads grouped), keeps row j's minimum in lane j, then lowers the distances
// (each row has this one writer) and appends the changed rows in one go
template <typename T>
__global__ void __launch_bounds__(256)
    k_sssp_pull_mid(const int32_t* __restrict__ rp, const int32_t* __restrict__ cv, const void* nz,
                    int tv, const unsigned* __restrict__ chg, T* dist, unsigned* chg_next,
                    int32_t* qn, Counters* ctr, const int32_t* __restrict__ prow,
                    const int32_t* __restrict__ mid, int64_t nmid) {
  const int lane = threadIdx.x & 31;
  // warps numbered block-major: the longest groups go to different SMs
  const int64_t gw = (int64_t)(threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g0 = gw * 32; g0 < nmid; g0 += nw * 32) {
    const int cnt = nmid - g0 < 32 ? (int)(nmid - g0) : 32;
    T mine = Lim<T>::max();
    int32_t myv = -1;
    // the group's row ids and row bounds, loaded by the lanes at once (row j in lane j),
    // so each row's scan starts without waiting on its own id and row pointers
    int32_t vj = -1;
    int64_t k0j = 0, k1j = 0;
    if (lane < cnt) {
      vj = mid[g0 + lane];
      k0j = (int64_t)rp[vj] - 1;
      k1j = (int64_t)rp[vj + 1] - 1;
    }
    // groups whose longest row (the first: the list is sorted) has at most 128 entries:
    // 8 lanes per row, 4 rows at once, 32 entries per step
    const int64_t len0 = __shfl_sync(0xffffffffu, k1j - k0j, 0);
    if (len0 <= 128) {
      const int sub = lane >> 3, sl = lane & 7;
      for (int j0 = 0; j0 < cnt; j0 += 4) {
        const int r = j0 + sub;  // this sub-warp's row of the group
        const int64_t k0 = __shfl_sync(0xffffffffu, k0j, r & 31);
        const int64_t k1s = __shfl_sync(0xffffffffu, k1j, r & 31);
        const int64_t k1 = r < cnt ? k1s : k0;
        T b = Lim<T>::max();
        for (int64_t kb = k0; kb < k1; kb += 32) {
          int32_t u[4];
          bool on[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const int64_t k = kb + t * 8 + sl;
            u[t] = k < k1 ? __ldg(cv + k) - 1 : -1;
          }
#pragma unroll
          for (int t = 0; t < 4; ++t) on[t] = u[t] >= 0 && bit_of(chg, u[t]);
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const T c = on[t] ? relax_add(view_weight<T>(nz, tv, kb + t * 8 + sl), ld_cg(dist + u[t]))
                              : Lim<T>::max();
            b = c < b ? c : b;
          }
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
          const T t = __shfl_xor_sync(0xffffffffu, b, o);
          b = t < b ? t : b;
        }
        // lane j0 + q takes the minimum of sub-warp q (rows j0 .. j0 + 3)
        const T got = __shfl_sync(0xffffffffu, b, ((lane - j0) & 3) * 8);
        if (lane >= j0 && lane < j0 + 4 && lane < cnt) {
          mine = got;
          myv = vj;
        }
      }
    }
    for (int j = 0; j < cnt && len0 > 128; ++j) {
      const int32_t v = __shfl_sync(0xffffffffu, vj, j);
      const int64_t k0 = __shfl_sync(0xffffffffu, k0j, j), k1 = __shfl_sync(0xffffffffu, k1j, j);
      T b = Lim<T>::max();
      for (int64_t kb = k0; kb < k1; kb += 128) {
        int32_t u[4];
        bool on[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int64_t k = kb + t * 32 + lane;
          u[t] = k < k1 ? __ldg(cv + k) - 1 : -1;
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) on[t] = u[t] >= 0 && bit_of(chg, u[t]);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const T c = on[t] ? relax_add(view_weight<T>(nz, tv, kb + t * 32 + lane), ld_cg(dist + u[t]))
                            : Lim<T>::max();
          b = c < b ? c : b;
        }
      }
      b = warp_min_t(b);
      if (lane == j) {
        mine = b;
        myv = v;
      }
    }
    bool changed = false;
    if (myv >= 0 && mine < dist[myv]) {
      dist[myv] = mine;
      changed = true;
      atomicOr(chg_next + (myv >> 5), 1u << (myv & 31));
    }
    warp_append(changed, myv, changed ? prow[myv + 1] - prow[myv] : 0, qn, ctr);
  }
}

// hub rows of the pull round: one warp per piece of the matrix's hub plan (rows of
// more than kHubDegB entries cut into kHubPieceB), atomic min into the hub
template <typename T>
__global__ void __launch_bounds__(256)
    k_sssp_pull_hub(const int32_t* __restrict__ cv, const void* nz, int tv,
                    const unsigned* __restrict__ chg, T* dist, unsigned* chg_next, int32_t* qn,
                    Counters* ctr, const int32_t* __restrict__ prow,
                    const int4* __restrict__ pieces, int64_t npiece,
                    const int32_t* __restrict__ hubs) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < npiece;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int4 pc = pieces[i];  // hub index, first entry, end entry (0-based)
    const int32_t v = hubs[pc.x];
    T b = Lim<T>::max();
    for (int64_t k = pc.y + lane; k < pc.z; k += 32) {
      const int32_t u = __ldg(cv + k) - 1;
      if (bit_of(chg, u)) {
        const T c = relax_add(view_weight<T>(nz, tv, k), ld_cg(dist + u));
        b = c < b ? c : b;
      }
    }
    b = warp_min_t(b);
    if (lane == 0 && b < ld_cg(dist + v) && b < atomic_min_t(dist + v, b)) {
      const unsigned bit = 1u << (v & 31);
      if (!(atomicOr(chg_next + (v >> 5), bit) & bit)) {
        const unsigned long long pos = atomicAdd(&ctr->nf, 1ull);
        atomicAdd(&ctr->mf, (unsigned long long)(prow[v + 1] - prow[v]));
        qn[pos] = v;
      }
    }
  }
}

// ---------------------------------------------------------------------------------
// Pull round over the SELL-32 copy of A_T (rows sorted by length, slice-column-major):
// one warp per work item of the copy's plan (a chunk of <= 128 columns of a slice, or
// a group of narrow slices), lane = stored row, so every column / weight load of a
// warp is one 128-byte line.  Each row takes the minimum of w + dist[u] over all its
// in-edges of the item (an in-edge whose source did not change cannot improve it, so
// no membership test is made) and lowers dist[v] with an atomic min (the chunks of a
// long row race only through that min).  Improved vertices join the next frontier
// once (bitmap inq_next) with their out-degrees counted.  Distances are gathered
// through L1 (a value lowered by another SM may be seen late: any distance read is an
// upper bound of the fixpoint, and a vertex lowered in this round joins the next
// frontier, so any order reaches the same fixpoint) and lowered in place.
// ---------------------------------------------------------------------------------
static const int kPullSellThreads = 512;
// a round pulls when the frontier's out-edges exceed nnz / kPullSellDiv
#ifndef GG_PULL_SELL_DIV
#define GG_PULL_SELL_DIV 16
#endif
static const int64_t kPullSellDiv = GG_PULL_SELL_DIV;

template <typename T>
__device__ __forceinline__ void pull_lower(int64_t srow, int64_t m, const int32_t* __restrict__ perm,
                                           T cand, T* dist, unsigned* inq_next, int32_t* qn,
                                           Counters* ctr, const int32_t* __restrict__ prow) {
  bool improved = false;
  int32_t v = 0, deg = 0;
  if (srow < m && cand != Lim<T>::max()) {
    v = __ldg(perm + srow) - 1;
    if (cand < ld_cg(dist + v)) {
      const T old = atomic_min_t(dist + v, cand);
      if (cand < old) {
        const unsigned bit = 1u << (v & 31);
        improved = !(atomicOr(inq_next + (v >> 5), bit) & bit);
        if (improved) deg = __ldg(prow + v + 1) - __ldg(prow + v);
      }
    }
  }
  warp_append(improved, v, deg, qn, ctr);
}

template <typename T>
__global__ void __launch_bounds__(kPullSellThreads)
    k_sssp_pull_sell(const int32_t* __restrict__ colval, const void* __restrict__ nz, int tv,
                     const int32_t* __restrict__ perm, int64_t m, const int4* __restrict__ pitems,
                     int64_t nitems, T* dist, unsigned* inq_next, int32_t* qn, Counters* ctr,
                     const int32_t* __restrict__ prow) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int4 dn = gw < nitems ? __ldg(pitems + gw) : make_int4(0, 0, 0, -1);
  for (int64_t it = gw; it < nitems; it += nw) {
    const int4 d = dn;  // first position, first stored row, columns (or -slices), partial
    if (it + nw < nitems) dn = __ldg(pitems + it + nw);
    if (d.z < 0) {
      // group of -d.z narrow slices (widths in 4-bit fields of d.w), <= 8 columns in all
      const int ns = -d.z;
      const uint32_t widths = (uint32_t)d.w;
      int total = 0;
      for (int t = 0; t < ns; ++t) total += (widths >> (4 * t)) & 15u;
      T c[kNarrowCols];
#pragma unroll
      for (int u = 0; u < kNarrowCols; ++u) {
        c[u] = Lim<T>::max();
        if (u < total) {
          const int32_t col = __ldg(colval + d.x + u * 32 + lane);
          if (col > 0)
            c[u] = relax_add(view_weight<T>(nz, tv, (int64_t)d.x + u * 32 + lane), ld_l1(dist + (col - 1)));
        }
      }
      int u0 = 0;
      for (int t = 0; t < ns; ++t) {
        const int w = (int)((widths >> (4 * t)) & 15u);
        T best = Lim<T>::max();
#pragma unroll
        for (int u = 0; u < kNarrowCols; ++u)
          if (u >= u0 && u < u0 + w && c[u] < best) best = c[u];
        u0 += w;
        pull_lower(d.y + t * 32 + lane, m, perm, best, dist, inq_next, qn, ctr, prow);
      }
      continue;
    }
    const int64_t srow = (int64_t)d.y + lane;
    T best = Lim<T>::max();
    if (srow < m) {
      // the next 8 columns / weights are loaded (streamed past L1) while the current
      // 8 distances are gathered
      int32_t col[8];
      T w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int64_t pos = (int64_t)d.x + lane + (int64_t)u * 32;
        col[u] = u < d.z ? __ldcs(colval + pos) : -1;
        w[u] = u < d.z ? view_weight<T>(nz, tv, pos) : Lim<T>::max();
      }
      for (int32_t j = 0; j < d.z; j += 8) {
        int32_t cn[8];
        T wn[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int64_t pos = (int64_t)d.x + lane + (int64_t)(j + 8 + u) * 32;
          cn[u] = j + 8 + u < d.z ? __ldcs(colval + pos) : -1;
          wn[u] = j + 8 + u < d.z ? view_weight<T>(nz, tv, pos) : Lim<T>::max();
        }
        T dv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) dv[u] = col[u] > 0 ? ld_l1(dist + (col[u] - 1)) : Lim<T>::max();
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const T cand = relax_add(w[u], dv[u]);
          best = cand < best ? cand : best;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          col[u] = cn[u];
          w[u] = wn[u];
        }
      }
    }
    pull_lower(srow, m, perm, best, dist, inq_next, qn, ctr, prow);
  }
}

// the SELL-32 copy (rows sorted by length) and its work plan, built on first use
static int ensure_pull_sell(gg_ctx* ctx, gg_mat* A) {
  GraphAux* g = A->aux;
  if (g->pull_sell) return GG_OK;
  gg_mat* S = nullptr;
  GG_CHECK(gg_sell_create(ctx, A, 32, A->m, &S));
  int rc = build_sell_plan(ctx, S);
  if (rc != GG_OK) {
    gg_mat_destroy(S);
    return rc;
  }
  g->pull_sell = S;
  return GG_OK;
}

// The SELL-32 copy (rows sorted by length, with its work items) of the shortest-path
// pull rounds, built on first use; nullptr for SELL handles and CSR handles of fewer
// than 65536 rows.
int pull_sell_copy(gg_ctx* ctx, gg_mat* A, const gg_mat** out) {
  *out = nullptr;
  if (A->format != GG_FMT_CSR || A->m < (1 << 16) || !A->aux) return GG_OK;
  GG_CHECK(ensure_pull_sell(ctx, A));
  *out = A->aux->pull_sell;
  return GG_OK;
}

// Builds, ahead of any concurrent use, every analysis a shortest-path search of A may
// build on first use: the out-edge view with weights, the hub plan and (large CSR
// handles) the SELL-32 copy of the pull rounds.  The serving loop calls it when a
// graph is added, so concurrent searches only read these structures.
int sssp_prepare(gg_ctx* ctx, gg_mat* A) {
  GG_CHECK(ensure_push(ctx, A, 2));
  GraphAux* g = A->aux;
  if (g->max_in_deg < 0) {
    GG_CUDA(cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream));
    k_max_deg<<<gridsz(ctx, A->m), 256, 0, ctx->stream>>>(A->m, g->vrowptr, ctx->d_flags);
    GG_CUDA(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    g->max_in_deg = ctx->h_flags[0];
  }
  if (g->max_in_deg > 32) GG_CHECK(build_hub_plan(ctx, A, g->vrowptr, A->m));
  if (A->format == GG_FMT_CSR && A->m >= (1 << 16)) GG_CHECK(ensure_pull_sell(ctx, A));
  return GG_OK;
}

template <typename T>
static int sssp_fixpoint(gg_ctx* ctx, gg_mat* A, T* d, int64_t* rounds_out) {
  GG_CHECK(ensure_push(ctx, A, 2));
  GraphAux* g = A->aux;
  PushCSR& P = g->push[2];
  const int64_t n = A->m;
  BfsScratch sc;  // visited -> unused; fb[0], fb[1] are the two membership bitmaps
  GG_CHECK(bfs_scratch(ctx, n, &sc));
  GG_CUDA(cudaFuncSetAttribute(k_sssp_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kSmallSmem));
  Counters* h = reinterpret_cast<Counters*>(ctx->h_flags);
  GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
  k_sssp_seed<T><<<gridsz(ctx, n), 256, 0, ctx->stream>>>(n, d, sc.fb[0], sc.q[0], sc.ctr);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  int64_t nf = (int64_t)h->nf, rounds = 0, mf = 0;
  int cur = 0;
  const int64_t max_rounds = n + 1;  // Bellman-Ford bound for non-negative weights
  if (g->max_in_deg < 0) {
    GG_CUDA(cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream));
    k_max_deg<<<gridsz(ctx, n), 256, 0, ctx->stream>>>(n, g->vrowptr, ctx->d_flags);
    GG_CUDA(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    g->max_in_deg = ctx->h_flags[0];
  }
  // rows with more than kHubDegB in-edges: relaxed in pieces during pull rounds
  const HubPlan* hp = nullptr;
  if (g->max_in_deg > 32) {  // rows the pull kernel's thread-per-vertex path leaves out
    GG_CHECK(build_hub_plan(ctx, A, g->vrowptr, n));
    hp = A->hubplan;
  }
  const bool coop_ok = P.max_deg <= kCoopMaxDeg && n >= (1 << 16);
  if (coop_ok && nf > 0) {
    // hub-free graph: the whole search in one near-far ordered persistent launch
    if (g->avg_w < 0) {
      double* dsum = nullptr;
      GG_CUDA(cudaMallocAsync((void**)&dsum, sizeof(double), ctx->stream));
      GG_CUDA(cudaMemsetAsync(dsum, 0, sizeof(double), ctx->stream));
      k_sum_weights<T><<<gridsz(ctx, P.nnz), 256, 0, ctx->stream>>>(static_cast<const T*>(P.w), P.nnz,
                                                                    dsum);
      double hs = 0.0;
      GG_CUDA(cudaMemcpyAsync(&hs, dsum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      cudaFree(dsum);
      g->avg_w = P.nnz > 0 ? hs / (double)P.nnz : 1.0;
    }
    double dd = g->avg_w * kNearFarScale;
    if (!(dd > 0.0)) dd = 1.0;
    T delta = static_cast<T>(dd);
    if (!(delta > T(0))) delta = T(1);
    NfCtl* ncc = reinterpret_cast<NfCtl*>(sc.cc);
    k_nf_init<<<1, 1, 0, ctx->stream>>>(ncc, nf, barrier_polls(ctx));
    int32_t* qa = sc.q[cur];
    int32_t* qb = sc.q[cur ^ 1];
    unsigned* ia = sc.fb[cur];
    unsigned* ib = sc.fb[cur ^ 1];
    const T* pw = static_cast<const T*>(P.w);
    long long max_steps = 8 * (long long)n + 1024;
    void* args[] = {&P.rowptr, &P.colval, &pw, &qa, &qb, &sc.hq, &sc.q2, &sc.q3, &d, &ia, &ib,
                    &sc.visited, &ncc, &delta, &max_steps};
    GG_CUDA(cudaLaunchCooperativeKernel((const void*)k_sssp_nearfar<T>, dim3(ctx->num_sms),
                                        dim3(kCoopThreads), args, 0, ctx->stream));
    NfCtl hn;
    GG_CUDA(cudaMemcpyAsync(&hn, ncc, sizeof(NfCtl), cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hn.bar[2]) return set_error(GG_ERR_TIMEOUT, "grid barrier wait ran out");
    if (hn.status != 1) return set_error(GG_ERR_NOT_CONVERGED, "shortest_path did not converge");
    if (rounds_out) *rounds_out += hn.steps_out;
    return GG_OK;
  }
  const int32_t small_cap = coop_ok ? kCoopLo : kSmallCap;
  const long long coop_hi = n / 8 > kCoopLo ? n / 8 : kCoopLo;
  // large CSR handles pull over a SELL-32 copy (built at the first pull round)
  const bool sell_pull = A->format == GG_FMT_CSR && n >= (1 << 16);
  while (nf > 0) {
    if (rounds > max_rounds) return set_error(GG_ERR_NOT_CONVERGED, "shortest_path did not converge");
    if (coop_ok && nf > small_cap && nf <= coop_hi && mf * 8 <= P.nnz) {
      k_coop_init<<<1, 1, 0, ctx->stream>>>(sc.cc, nf, barrier_polls(ctx));
      int32_t* qa = sc.q[cur];
      int32_t* qb = sc.q[cur ^ 1];
      unsigned* ia = sc.fb[cur];
      unsigned* ib = sc.fb[cur ^ 1];
      const T* pw = static_cast<const T*>(P.w);
      long long lo = kCoopLo / 2, hi = coop_hi, mr = max_rounds - rounds + 1;
      void* args[] = {&P.rowptr, &P.colval, &pw, &qa, &qb, &d, &ia, &ib, &sc.cc, &lo, &hi, &mr};
      CoopCtl* hc = reinterpret_cast<CoopCtl*>(ctx->h_flags);
      GG_CHECK(coop_launch(ctx, (const void*)k_sssp_coop<T>, args, sc.cc, hc));
      nf = hc->nf_out;
      rounds += hc->level_out;
      if (hc->which_out) cur ^= 1;
      mf = 0;
      if (nf > 0) {
        GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
        k_queue_degree<<<gridsz(ctx, nf), 256, 0, ctx->stream>>>(P.rowptr, sc.q[cur], nf, sc.ctr);
        GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
        GG_CUDA(cudaStreamSynchronize(ctx->stream));
        mf = (int64_t)h->mf;
      }
      continue;
    }
    if (nf <= small_cap && mf <= (int64_t)kSmallEdges) {
      GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
      k_sssp_small<T><<<1, kSmallThreads, kSmallSmem, ctx->stream>>>(
          P.rowptr, P.colval, static_cast<const T*>(P.w), sc.q[cur], (int32_t)nf, small_cap, d,
          sc.fb[cur], sc.fb[cur ^ 1], sc.ctr, max_rounds - rounds, kSmallEdges);
      GG_CUDA(cudaGetLastError());
      GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      nf = (int64_t)h->nf;
      rounds += (int64_t)h->level;
      // the remaining frontier is in q[cur]; its membership bits are in fb[cur] when
      // status == 0, else in fb[cur ^ 1] -- then swap roles so bits and queue agree
      // out-edges of the remaining frontier (counted by the kernel), for the direction
      // choice; a frontier above kSmallEdges goes to the grid-wide rounds
      mf = nf > 0 ? (int64_t)h->mf : 0;
      if (nf > 0 && h->status == 1) {
        cur ^= 1;
        GG_CUDA(cudaMemcpyAsync(sc.q[cur], sc.q[cur ^ 1], nf * sizeof(int32_t),
                                cudaMemcpyDeviceToDevice, ctx->stream));
      }
      continue;
    }
    ++rounds;
    GG_CUDA(cudaMemsetAsync(sc.ctr, 0, sizeof(Counters), ctx->stream));
    if (sell_pull && mf * kPullSellDiv > P.nnz) {
      // large frontier: pull round over the SELL-32 copy, every in-edge
      GG_CHECK(ensure_pull_sell(ctx, A));
      const gg_mat* S = g->pull_sell;
      const SellPlan* SP = S->sellplan;
      if (SP->npitems > 0)
        k_sssp_pull_sell<T><<<ctx->num_sms * (2048 / kPullSellThreads), kPullSellThreads, 0,
                              ctx->stream>>>(S->colval, S->nzval, S->dtype, S->perm, S->m,
                                             SP->pitems, SP->npitems, d, sc.fb[cur ^ 1],
                                             sc.q[cur ^ 1], sc.ctr, P.rowptr);
      // the consumed membership bitmap becomes the next round's target: clear it
      GG_CUDA(cudaMemsetAsync(sc.fb[cur], 0, ((n + 31) / 32) * sizeof(unsigned), ctx->stream));
      GG_CUDA(cudaGetLastError());
      GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      nf = (int64_t)h->nf;
      mf = (int64_t)h->mf;
      cur ^= 1;
      continue;
    }
    if (!sell_pull && mf * 4 > P.nnz) {
      // large frontier: pull round (no atomics on the common path)
      k_sssp_pull<T><<<gridsz(ctx, n), 256, 0, ctx->stream>>>(
          n, g->vrowptr, g->vcolval, g->vnz, A->dtype, sc.fb[cur], d, sc.fb[cur ^ 1], sc.q[cur ^ 1],
          sc.ctr, P.rowptr);
      if (hp && hp->nmid > 0)
        k_sssp_pull_mid<T><<<gridsz(ctx, hp->nmid), 256, 0, ctx->stream>>>(
            g->vrowptr, g->vcolval, g->vnz, A->dtype, sc.fb[cur], d, sc.fb[cur ^ 1], sc.q[cur ^ 1],
            sc.ctr, P.rowptr, hp->mid, hp->nmid);
      if (hp && hp->npiece > 0)
        k_sssp_pull_hub<T><<<gridsz(ctx, hp->npiece * 32), 256, 0, ctx->stream>>>(
            g->vcolval, g->vnz, A->dtype, sc.fb[cur], d, sc.fb[cur ^ 1], sc.q[cur ^ 1], sc.ctr,
            P.rowptr, hp->pieces, hp->npiece, hp->hubs);
      // the consumed membership bitmap becomes the next round's target: clear it
      GG_CUDA(cudaMemsetAsync(sc.fb[cur], 0, ((n + 31) / 32) * sizeof(unsigned), ctx->stream));
      GG_CUDA(cudaGetLastError());
      GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      nf = (int64_t)h->nf;
      mf = (int64_t)h->mf;
      cur ^= 1;
      continue;
    }
    const bool hubs = P.max_deg > kPushHub;
    k_sssp_push<T><<<gridsz(ctx, nf * 32), 256, 0, ctx->stream>>>(
        P.rowptr, P.colval, static_cast<const T*>(P.w), sc.q[cur], nf, d, sc.fb[cur],
        sc.fb[cur ^ 1], sc.q[cur ^ 1], sc.ctr, hubs ? sc.hq : nullptr);
    if (hubs) {
      k_hub_offsets<<<1, 1024, 0, ctx->stream>>>(P.rowptr, sc.hq, sc.ctr, sc.hoff);
      k_sssp_push_hub<T><<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(
          P.rowptr, P.colval, static_cast<const T*>(P.w), sc.hq, d, sc.fb[cur ^ 1], sc.q[cur ^ 1],
          sc.ctr, sc.ctr, sc.hoff);
    }
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(h, sc.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    nf = (int64_t)h->nf;
    mf = (int64_t)h->mf;
    cur ^= 1;
  }
  if (rounds_out) *rounds_out += rounds;
  return GG_OK;
}

// Jacobi rounds of the reference (shortest_path.jl:61-80) with the generic min-plus
// SpMV; used for negative / NaN weights.  Stops when a round changes nothing.
template <typename T>
static int sssp_jacobi(gg_ctx* ctx, gg_mat* A, T* dist, T* next, int td, int64_t* rounds_out) {
  const int64_t n = A->m;
  int tc = 0;
  GG_CHECK(check_semiring(A->dtype, td, td, GG_OP_SAFE_ADD, GG_OP_MIN, GG_OP_MIN, &tc));
  for (int64_t r = 0; r <= n + 1; ++r) {
    GG_CHECK(spmv_dispatch(ctx, A, tc, GG_OP_SAFE_ADD, GG_OP_MIN, GG_OP_MIN, next, td, dist, td,
                           nullptr, 0, 0, 0));
    GG_CUDA(cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream));
    k_changed_copy<T><<<gridsz(ctx, n), 256, 0, ctx->stream>>>(n, next, dist, ctx->d_flags);
    GG_CUDA(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (rounds_out) *rounds_out += 1;
    if (!ctx->h_flags[0]) return GG_OK;
  }
  return set_error(GG_ERR_NOT_CONVERGED, "shortest_path did not converge (negative cycle?)");
}

template <typename T>
static int sssp_column(gg_ctx* ctx, gg_mat* A, int64_t s, T* dist, T* next, int td, bool caller,
                       int64_t* rounds_out) {
  const int64_t n = A->m;
  GraphAux* g = A->aux;
  if (!caller) {
    k_fill_t<T><<<gridsz(ctx, n), 256, 0, ctx->stream>>>(dist, n, Lim<T>::max());
    if (next) k_fill_t<T><<<gridsz(ctx, n), 256, 0, ctx->stream>>>(next, n, Lim<T>::max());
  }
  k_set_source<T><<<1, 1, 0, ctx->stream>>>(dist, next, s);
  GG_CUDA(cudaGetLastError());
  if (!g->nonneg) {
    T* nx = next;
    if (!nx) {
      GG_CUDA(cudaMalloc((void**)&nx, n * sizeof(T)));
      GG_CUDA(cudaMemcpyAsync(nx, dist, n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    int rc = sssp_jacobi<T>(ctx, A, dist, nx, td, rounds_out);
    if (!next) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(nx);
    }
    return rc;
  }
  T* start = dist;
  if (caller && next) {
    // first Jacobi round exactly as the reference: next = min(next, F(dist))
    int tc = 0;
    GG_CHECK(check_semiring(A->dtype, td, td, GG_OP_SAFE_ADD, GG_OP_MIN, GG_OP_MIN, &tc));
    GG_CHECK(spmv_dispatch(ctx, A, tc, GG_OP_SAFE_ADD, GG_OP_MIN, GG_OP_MIN, next, td, dist, td,
                           nullptr, 0, 0, 0));
    start = next;
  }
  GG_CHECK(sssp_fixpoint<T>(ctx, A, start, rounds_out));
  if (start != dist)
    GG_CUDA(cudaMemcpyAsync(dist, start, n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
  if (next && start != next)
    GG_CUDA(cudaMemcpyAsync(next, dist, n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
  return GG_OK;
}

static int check_graph(const gg_mat* A) {
  if (A->m != A->n) return set_error(GG_ERR_DIMENSION, "A_T must be square (got %lld x %lld)",
                                     (long long)A->m, (long long)A->n);
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_bfs_levels(gg_ctx* ctx, const gg_mat* A_T, int64_t source, int32_t* dist, int64_t n,
                  int64_t* levels_out) {
  if (!ctx || !A_T || !dist) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  GG_CHECK(check_graph(A_T));
  if (n != A_T->m) return set_error(GG_ERR_DIMENSION, "dist length must equal size(A_T, 1)");
  if (source < 1 || source > A_T->m) return set_error(GG_ERR_BOUNDS, "source %lld out of 1:%lld",
                                                      (long long)source, (long long)A_T->m);
  if (dtype_is_float(A_T->dtype))
    return set_error(GG_ERR_UNSUPPORTED, "GPUGraphs_band has no method for floating-point matrices");
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_mat* A = const_cast<gg_mat*>(A_T);
  return bfs_run(ctx, A, (int32_t)(source - 1), 0, dist, levels_out);
}

int gg_bfs_parents(gg_ctx* ctx, const gg_mat* A_T, int64_t source, int32_t* parents, int64_t n,
                   int rule, int64_t* levels_out) {
  if (!ctx || !A_T || !parents) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  GG_CHECK(check_graph(A_T));
  if (n != A_T->m) return set_error(GG_ERR_DIMENSION, "parents length must equal size(A_T, 1)");
  if (source < 1 || source > A_T->m) return set_error(GG_ERR_BOUNDS, "source %lld out of 1:%lld",
                                                      (long long)source, (long long)A_T->m);
  if (rule == GG_PARENT_FORMAT_DEFAULT)
    rule = A_T->format == GG_FMT_CSR ? GG_PARENT_FIRST_IN_ROW : GG_PARENT_MAX_INDEX;
  if (rule != GG_PARENT_FIRST_IN_ROW && rule != GG_PARENT_MAX_INDEX)
    return set_error(GG_ERR_ARGUMENT, "unknown parent rule %d", rule);
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_mat* A = const_cast<gg_mat*>(A_T);
  int32_t* lev = nullptr;
  GG_CUDA(cudaMallocAsync((void**)&lev, n * sizeof(int32_t), ctx->stream));
  k_fill_i32<<<gridsz(ctx, n), 256, 0, ctx->stream>>>(lev, n, INT32_MAX);
  int rc = bfs_run(ctx, A, (int32_t)(source - 1), 1, lev, levels_out);
  if (rc == GG_OK) {
    GraphAux* g = A->aux;
    k_bfs_parents<<<gridsz(ctx, n * 32), 256, 0, ctx->stream>>>(
        n, g->vrowptr, g->vcolval, lev, (int32_t)(source - 1), rule, parents);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_error(e, "k_bfs_parents");
  }
  cudaFreeAsync(lev, ctx->stream);
  return rc;
}

int gg_sssp(gg_ctx* ctx, const gg_mat* A_T, const int64_t* sources, int64_t nsources, void* dist,
            void* next, int dist_dtype, int64_t ld, int64_t* rounds_out) {
  if (!ctx || !A_T || !dist || (nsources > 0 && !sources))
    return set_error(GG_ERR_ARGUMENT, "NULL argument");
  GG_CHECK(check_graph(A_T));
  const int64_t n = A_T->m;
  if (ld < n) return set_error(GG_ERR_DIMENSION, "leading dimension of dist must be >= n");
  if (dist_dtype != dist_type_of(A_T->dtype))
    return set_error(GG_ERR_TYPE, "dist element type must be Int32 for Bool matrices, else eltype(A_T)");
  for (int64_t q = 0; q < nsources; ++q)
    if (sources[q] < 1 || sources[q] > n)
      return set_error(GG_ERR_BOUNDS, "source %lld out of 1:%lld", (long long)sources[q], (long long)n);
  if (rounds_out) *rounds_out = 0;
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_mat* A = const_cast<gg_mat*>(A_T);
  GG_CHECK(ensure_aux(ctx, A));
  const bool caller = next != nullptr;
  // several sources from the standard start: one batched pass (the reference's
  // min-plus SpMM formulation, shortest_path.jl:88-161)
  if (!caller && nsources > 1 && A->aux->nonneg)
    return gg_sssp_batch(ctx, A_T, sources, nsources, dist, dist_dtype, ld, rounds_out);
  const int esz = dtype_size(dist_dtype);
  for (int64_t q = 0; q < nsources; ++q) {
    char* dcol = static_cast<char*>(dist) + q * ld * esz;
    char* ncol = next ? static_cast<char*>(next) + q * ld * esz : nullptr;
    int rc = GG_OK;
    switch (dist_dtype) {
      case GG_INT32:
        rc = sssp_column<int32_t>(ctx, A, sources[q] - 1, (int32_t*)dcol, (int32_t*)ncol, dist_dtype, caller, rounds_out);
        break;
      case GG_INT64:
        rc = sssp_column<int64_t>(ctx, A, sources[q] - 1, (int64_t*)dcol, (int64_t*)ncol, dist_dtype, caller, rounds_out);
        break;
      case GG_FLOAT32:
        rc = sssp_column<float>(ctx, A, sources[q] - 1, (float*)dcol, (float*)ncol, dist_dtype, caller, rounds_out);
        break;
      case GG_FLOAT64:
        rc = sssp_column<double>(ctx, A, sources[q] - 1, (double*)dcol, (double*)ncol, dist_dtype, caller, rounds_out);
        break;
      default:
        rc = set_error(GG_ERR_TYPE, "unsupported distance type");
    }
    if (rc) return rc;
  }
  return GG_OK;
}

}  // extern "C"
