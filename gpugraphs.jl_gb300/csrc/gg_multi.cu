// gg_multi.cu -- many independent graphs processed by single launches.
//
// A gg_multigraph holds G square CSR graphs concatenated into one block-diagonal
// structure: each graph keeps its own 1-based Int32 column ids, and 64-bit offsets
// locate its rows and entries (the total entry count may exceed Int32).  Vertex v of
// graph g has the global id row_off[g] + v - 1.
//  * gg_multigraph_spmv: y = A_g x_g (plus-times Float32) for every graph in one
//    kernel launch, 8 lanes per row.
//  * gg_multigraph_bfs: one BFS per graph (one source each) in ONE persistent
//    cooperative launch: all graphs advance level by level together, separated by a
//    grid barrier; frontiers are global queues of global vertex ids.  The barrier's
//    wait is bounded: on timeout it records an error, every block returns, and the
//    call reports GG_ERR_TIMEOUT.  The launch (with its resets) is captured once in
//    a CUDA graph and replayed by later calls.
//  * gg_multigraph_sssp: one single-source shortest-path search per graph in one
//    persistent cooperative launch (frontier Bellman-Ford, atomic min, bounded grid
//    barrier), captured in a CUDA graph the same way.
// Levels follow bfs_distances (src/algorithms/bfs.jl:1-73): edges with odd / true
// stored values (every stored entry of a floating-point graph, i.e. its Bool
// pattern), dist = hop level, typemax(Int32) when unreached.  Distances follow
// shortest_path (src/algorithms/shortest_path.jl:12-83) for non-negative weights.
// Both searches use the rows of A_T as out-edges, which equals the reference for
// symmetric graphs.
#include <algorithm>
#include <vector>

#include "gg_semiring.cuh"

struct gg_multigraph {
  int device = 0;
  int64_t ngraphs = 0;
  int64_t total_n = 0, total_nnz = 0;
  int dtype = GG_FLOAT32;
  int64_t* row_off = nullptr;  // [G+1] global vertex offsets (0-based)
  int64_t* rp64 = nullptr;     // [total_n+1] global 0-based entry offsets of each row
  int32_t* colval = nullptr;   // [total_nnz] global 0-based column (vertex) ids
  void* nzval = nullptr;       // [total_nnz]
  std::vector<int64_t> h_row_off;
  bool all_odd = true;
  // persistent BFS state
  unsigned* visited = nullptr;
  int32_t* q[2] = {nullptr, nullptr};
  unsigned long long* ctr = nullptr;  // [3] rotating queue counters
  unsigned* bar = nullptr;  // [8] barrier count, generation, error, levels, poll limit
  int64_t* d_src = nullptr;           // [G] global source ids
  int32_t* dist_bound = nullptr;      // dist pointer captured in the graph
  unsigned polls_set = 0;  // poll limit last written to bar[4] (0: none yet)
  cudaGraphExec_t gexec = nullptr;
  int grid = 0;
  // persistent shortest-path state (allocated on first use)
  unsigned* inq[2] = {nullptr, nullptr};
  void* sssp_dist_bound = nullptr;
  cudaGraphExec_t sssp_gexec = nullptr;
  int nonneg = -1;  // all stored values >= 0 (and not NaN)? -1: not yet checked
};

// the context's barrier poll limit into bar[4] (kept across launches: the captured
// graphs clear bar[0..3] only)
static int mg_set_polls(gg_ctx* ctx, gg_multigraph* M) {
  const unsigned p = gg::barrier_polls(ctx);
  if (M->polls_set != p) {
    GG_CUDA(cudaMemcpyAsync(M->bar + 4, &p, sizeof(unsigned), cudaMemcpyHostToDevice, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    M->polls_set = p;
  }
  return GG_OK;
}

namespace gg {

static const unsigned kFullM = 0xffffffffu;

__device__ __forceinline__ int graph_of(const int64_t* __restrict__ off, int64_t G, int64_t v) {
  int64_t lo = 0, hi = G - 1;  // largest g with off[g] <= v
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (off[mid] <= v) lo = mid; else hi = mid - 1;
  }
  return (int)lo;
}

// 8 lanes per row over all graphs' rows (global column ids: no per-row graph lookup)
__global__ void __launch_bounds__(256)
    k_mg_spmv(int64_t total_n, const int64_t* __restrict__ rp, const int32_t* __restrict__ colval,
              const float* __restrict__ nz, const float* __restrict__ x, float* __restrict__ y) {
  const int sub = threadIdx.x & 7;
  const unsigned gm = 0xffu << ((threadIdx.x & 31) & ~7);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3; r < total_n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 3) {
    float acc = 0.0f;
    const int64_t k1 = rp[r + 1];
    for (int64_t k = rp[r] + sub; k < k1; k += 8)
      acc = __fadd_rn(acc, __fmul_rn(ld_stream(nz + k), __ldg(x + ld_stream(colval + k))));
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(gm, acc, o, 8));
    if (sub == 0) y[r] = acc;
  }
}

__device__ __forceinline__ bool mg_odd(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<const uint8_t*>(nz)[k] & 1;
    case GG_INT32: return static_cast<const int32_t*>(nz)[k] & 1;
    case GG_INT64: return static_cast<const int64_t*>(nz)[k] & 1;
  }
  return false;
}

// grid-wide barrier for a cooperative launch; the wait gives up after bar[4] polls
// (the context's limit, gg_set_wait_limit) and records an error so that every block
// can return.  bar: arrivals, generation, error, levels / rounds done, poll limit.
__device__ __forceinline__ bool mg_grid_sync(unsigned* bar, unsigned nblocks) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = bar + 1;
    volatile unsigned* verr = bar + 2;
    const unsigned gen = *vgen;
    const unsigned long long limit = bar[4];  // written by the host before each launch
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

__global__ void k_mg_bfs_init(int64_t G, const int64_t* src, unsigned* visited, int32_t* dist,
                              int32_t* q, unsigned long long* ctr) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < G;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = src[g];
    atomicOr(visited + (v >> 5), 1u << (v & 31));
    dist[v] = 0;
    q[g] = (int32_t)v;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctr[0] = (unsigned long long)G;  // queue size of level 0
    ctr[1] = 0;
    ctr[2] = 0;
  }
}

// all graphs' BFS levels in one persistent launch (warp per frontier vertex)
__global__ void __launch_bounds__(256)
    k_mg_bfs(int64_t G, const int64_t* __restrict__ row_off, const int64_t* __restrict__ rp,
             const int32_t* __restrict__ colval, const void* nz, int tv, int odd_only,
             unsigned* visited, int32_t* dist, int32_t* qa, int32_t* qb,
             unsigned long long* ctr, unsigned* bar) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int32_t* cur = qa;
  int32_t* nxt = qb;
  for (int32_t level = 1;; ++level) {
    const int r = level % 3;
    const int64_t nf = (int64_t)*((volatile unsigned long long*)(ctr + (r + 2) % 3));
    if (nf == 0) {
      if (blockIdx.x == 0 && threadIdx.x == 0) bar[3] = (unsigned)(level - 1);
      return;
    }
    // counter for this level's appends was zeroed two levels ago; zero the next one
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[(r + 1) % 3] = 0;
    for (int64_t i = gw; i < nf; i += nw) {
      const int64_t v = cur[i];
      const int64_t k0 = rp[v], k1 = rp[v + 1];
      for (int64_t kb = k0; kb < k1; kb += 32) {
        const int64_t k = kb + lane;
        bool claim = false;
        int64_t w = 0;
        if (k < k1 && (!odd_only || mg_odd(nz, tv, k))) {
          w = __ldg(colval + k);
          const unsigned bit = 1u << (w & 31);
          if (!(__ldcg(visited + (w >> 5)) & bit))
            claim = !(atomicOr(visited + (w >> 5), bit) & bit);
          if (claim) dist[w] = level;
        }
        const unsigned b = __ballot_sync(kFullM, claim);
        if (b) {
          const int leader = __ffs(b) - 1;
          unsigned long long pos = 0;
          if (lane == leader) pos = atomicAdd(ctr + r, (unsigned long long)__popc(b));
          pos = __shfl_sync(kFullM, pos, leader);
          if (claim) nxt[pos + __popc(b & ((1u << lane) - 1u))] = (int32_t)w;
        }
      }
    }
    if (!mg_grid_sync(bar, gridDim.x)) return;
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
  }
}

template <typename T> __device__ __forceinline__ T mg_atomic_min(T* p, T v);
template <> __device__ __forceinline__ int32_t mg_atomic_min<int32_t>(int32_t* p, int32_t v) {
  return atomicMin(p, v);
}
template <> __device__ __forceinline__ int64_t mg_atomic_min<int64_t>(int64_t* p, int64_t v) {
  return (int64_t)atomicMin((long long*)p, (long long)v);
}
// distances are non-negative and never -0.0 (+0.0 + w), so floats order like their bits
template <> __device__ __forceinline__ float mg_atomic_min<float>(float* p, float v) {
  return __int_as_float(atomicMin((int*)p, __float_as_int(v)));
}
template <> __device__ __forceinline__ double mg_atomic_min<double>(double* p, double v) {
  return __longlong_as_double(atomicMin((long long*)p, __double_as_longlong(v)));
}

template <typename T>
__device__ __forceinline__ T mg_weight(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<T>(static_cast<const uint8_t*>(nz)[k]);
    case GG_INT32: return static_cast<T>(static_cast<const int32_t*>(nz)[k]);
    case GG_INT64: return static_cast<T>(static_cast<const int64_t*>(nz)[k]);
    case GG_FLOAT32: return static_cast<T>(static_cast<const float*>(nz)[k]);
  }
  return static_cast<T>(static_cast<const double*>(nz)[k]);
}

template <typename T>
__global__ void k_mg_fill_t(T* d, int64_t n, T v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = v;
}

template <typename T>
__global__ void k_mg_sssp_seed(int64_t G, const int64_t* src, T* dist, unsigned* inq, int32_t* q,
                               unsigned long long* ctr) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < G;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = src[g];
    dist[v] = T(0);
    atomicOr(inq + (v >> 5), 1u << (v & 31));
    q[g] = (int32_t)v;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctr[0] = (unsigned long long)G;
    ctr[1] = 0;
    ctr[2] = 0;
  }
}

// all graphs' Bellman-Ford rounds in one persistent launch (warp per frontier
// vertex, push over its row); inq_cur / inq_next mark queued vertices
template <typename T>
__global__ void __launch_bounds__(256)
    k_mg_sssp(int64_t G, const int64_t* __restrict__ row_off, const int64_t* __restrict__ rp,
              const int32_t* __restrict__ colval, const void* nz, int tv, T* dist, unsigned* inq_a,
              unsigned* inq_b, int32_t* qa, int32_t* qb, unsigned long long* ctr, unsigned* bar,
              int64_t max_rounds) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int32_t* cur = qa;
  int32_t* nxt = qb;
  unsigned* icur = inq_a;
  unsigned* inxt = inq_b;
  for (int64_t round = 1;; ++round) {
    const int r = (int)(round % 3);
    const int64_t nf = (int64_t)*((volatile unsigned long long*)(ctr + (r + 2) % 3));
    if (nf == 0 || round > max_rounds) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        bar[3] = (unsigned)(round - 1);
        if (nf != 0) atomicExch(bar + 2, 2u);  // still improving after max_rounds
      }
      return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[(r + 1) % 3] = 0;
    for (int64_t i = gw; i < nf; i += nw) {
      const int64_t u = cur[i];
      if (lane == 0) atomicAnd(icur + (u >> 5), ~(1u << (u & 31)));
      const T du = __ldcg(dist + u);
      const int64_t k0 = rp[u], k1 = rp[u + 1];
      for (int64_t kb = k0; kb < k1; kb += 32) {
        const int64_t k = kb + lane;
        bool add = false;
        int64_t v = 0;
        if (k < k1) {
          v = __ldg(colval + k);
          const T w = mg_weight<T>(nz, tv, k);
          const T cand = (w == Lim<T>::max() || du == Lim<T>::max()) ? Lim<T>::max() : w_add(w, du);
          if (cand < __ldcg(dist + v)) {
            const T old = mg_atomic_min<T>(dist + v, cand);
            if (cand < old) {
              const unsigned bit = 1u << (v & 31);
              add = !(atomicOr(inxt + (v >> 5), bit) & bit);
            }
          }
        }
        const unsigned b = __ballot_sync(kFullM, add);
        if (b) {
          const int leader = __ffs(b) - 1;
          unsigned long long pos = 0;
          if (lane == leader) pos = atomicAdd(ctr + r, (unsigned long long)__popc(b));
          pos = __shfl_sync(kFullM, pos, leader);
          if (add) nxt[pos + __popc(b & ((1u << lane) - 1u))] = (int32_t)v;
        }
      }
    }
    if (!mg_grid_sync(bar, gridDim.x)) return;
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
    unsigned* tb = icur;
    icur = inxt;
    inxt = tb;
  }
}

__global__ void k_mg_nonneg(const void* nz, int tv, int64_t nnz, unsigned* bad) {
  unsigned b = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x) {
    switch (tv) {
      case GG_INT32: b |= static_cast<const int32_t*>(nz)[k] < 0; break;
      case GG_INT64: b |= static_cast<const int64_t*>(nz)[k] < 0; break;
      case GG_FLOAT32: { const float w = static_cast<const float*>(nz)[k]; b |= !(w >= 0.0f); break; }
      case GG_FLOAT64: { const double w = static_cast<const double*>(nz)[k]; b |= !(w >= 0.0); break; }
      default: break;
    }
  }
  if (__syncthreads_or(b) && threadIdx.x == 0) atomicOr(bad, 1u);
}

__global__ void k_mg_fill(int32_t* d, int64_t n, int32_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = v;
}

// global 0-based column ids: colval_g (1-based within graph g) + row_off[g] - 1
__global__ void k_mg_cols(int64_t nnz, const int32_t* __restrict__ cv, int32_t base, int32_t* out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = cv[k] - 1 + base;
}

// global entry offsets of each row: rp64[row_off[g] + v] = nnz_off[g] + rowptr_g[v] - 1
__global__ void k_mg_rp(int64_t n, const int32_t* rp_local, int64_t row_base, int64_t nnz_base,
                        int64_t* rp64) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n;
       v += (int64_t)gridDim.x * blockDim.x)
    rp64[row_base + v] = nnz_base + (int64_t)rp_local[v] - 1;
}

static int mg_grid(int num_sms, int64_t work) {
  int64_t g = (work + 255) / 256;
  const int64_t cap = (int64_t)num_sms * 8;
  return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_multigraph_create(gg_ctx* ctx, const gg_mat* const* graphs, int64_t ngraphs,
                         gg_multigraph** out) {
  if (!ctx || !graphs || !out || ngraphs < 1) return set_error(GG_ERR_ARGUMENT, "bad arguments");
  *out = nullptr;
  GG_CUDA(cudaSetDevice(ctx->device));
  const int dt = graphs[0]->dtype;
  std::vector<int64_t> off(ngraphs + 1, 0), noff(ngraphs + 1, 0);
  for (int64_t g = 0; g < ngraphs; ++g) {
    const gg_mat* A = graphs[g];
    if (!A || A->format != GG_FMT_CSR) return set_error(GG_ERR_ARGUMENT, "graph %lld is not a CSR handle", (long long)g);
    if (A->m != A->n) return set_error(GG_ERR_DIMENSION, "graph %lld is not square", (long long)g);
    if (A->dtype != dt) return set_error(GG_ERR_TYPE, "all graphs must share one element type");
    off[g + 1] = off[g] + A->m;
    noff[g + 1] = noff[g] + A->nnz;
  }
  if (off[ngraphs] >= INT32_MAX) return set_error(GG_ERR_ARGUMENT, "more than 2^31 vertices in total");
  gg_multigraph* M = new gg_multigraph();
  M->device = ctx->device;
  M->ngraphs = ngraphs;
  M->total_n = off[ngraphs];
  M->total_nnz = noff[ngraphs];
  M->dtype = dt;
  M->h_row_off = off;
  const size_t esz = dtype_size(dt);
  cudaError_t e = cudaMalloc((void**)&M->row_off, (ngraphs + 1) * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->rp64, (M->total_n + 1) * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->colval, (M->total_nnz + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&M->nzval, (M->total_nnz + 1) * esz);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(M->row_off, off.data(), (ngraphs + 1) * sizeof(int64_t),
                        cudaMemcpyHostToDevice, ctx->stream);
  for (int64_t g = 0; g < ngraphs && e == cudaSuccess; ++g) {
    const gg_mat* A = graphs[g];
    k_mg_rp<<<mg_grid(ctx->num_sms, A->m + 1), 256, 0, ctx->stream>>>(A->m, A->rowptr, off[g], noff[g],
                                                                       M->rp64);
    e = cudaGetLastError();
    if (e == cudaSuccess && A->nnz > 0) {
      k_mg_cols<<<mg_grid(ctx->num_sms, A->nnz), 256, 0, ctx->stream>>>(A->nnz, A->colval,
                                                                        (int32_t)off[g], M->colval + noff[g]);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && A->nnz > 0)
      e = cudaMemcpyAsync(static_cast<char*>(M->nzval) + noff[g] * esz, A->nzval, A->nnz * esz,
                          cudaMemcpyDeviceToDevice, ctx->stream);
  }
  // BFS state
  const int64_t nw = M->total_n / 32 + 2;
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->visited, nw * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->q[0], (M->total_n + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->q[1], (M->total_n + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->ctr, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->bar, 8 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(M->bar, 0, 8 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->d_src, ngraphs * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    gg_multigraph_destroy(M);
    return cuda_error(e, "gg_multigraph_create");
  }
  // edge activity for the levels semiring: odd / true values only
  if (dt == GG_BOOL || dt == GG_INT32 || dt == GG_INT64) {
    M->all_odd = true;  // checked lazily by the kernel's odd_only flag below
  }
  *out = M;
  return GG_OK;
}

int gg_multigraph_destroy(gg_multigraph* M) {
  if (!M) return GG_OK;
  cudaSetDevice(M->device);
  if (M->gexec) cudaGraphExecDestroy(M->gexec);
  if (M->sssp_gexec) cudaGraphExecDestroy(M->sssp_gexec);
  cudaFree(M->inq[0]);
  cudaFree(M->inq[1]);
  cudaFree(M->row_off);
  cudaFree(M->rp64);
  cudaFree(M->colval);
  cudaFree(M->nzval);
  cudaFree(M->visited);
  cudaFree(M->q[0]);
  cudaFree(M->q[1]);
  cudaFree(M->ctr);
  cudaFree(M->bar);
  cudaFree(M->d_src);
  delete M;
  return GG_OK;
}

int gg_multigraph_info(const gg_multigraph* M, int64_t* ngraphs, int64_t* total_n,
                       int64_t* total_nnz, int64_t* row_offsets) {
  if (!M) return set_error(GG_ERR_ARGUMENT, "NULL multigraph");
  if (ngraphs) *ngraphs = M->ngraphs;
  if (total_n) *total_n = M->total_n;
  if (total_nnz) *total_nnz = M->total_nnz;
  if (row_offsets)
    for (int64_t g = 0; g <= M->ngraphs; ++g) row_offsets[g] = M->h_row_off[g];
  return GG_OK;
}

int gg_multigraph_spmv(gg_ctx* ctx, const gg_multigraph* M, const float* x, float* y) {
  if (!ctx || !M || !x || !y) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (M->dtype != GG_FLOAT32) return set_error(GG_ERR_TYPE, "multigraph SpMV needs Float32 values");
  GG_CUDA(cudaSetDevice(ctx->device));
  k_mg_spmv<<<mg_grid(ctx->num_sms, M->total_n * 8), 256, 0, ctx->stream>>>(
      M->total_n, M->rp64, M->colval, static_cast<const float*>(M->nzval), x, y);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

int gg_multigraph_bfs(gg_ctx* ctx, gg_multigraph* M, const int64_t* sources, int32_t* dist,
                      int64_t* levels_out) {
  if (!ctx || !M || !sources || !dist) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  GG_CUDA(cudaSetDevice(ctx->device));
  std::vector<int64_t> gsrc(M->ngraphs);
  for (int64_t g = 0; g < M->ngraphs; ++g) {
    const int64_t n = M->h_row_off[g + 1] - M->h_row_off[g];
    if (sources[g] < 1 || sources[g] > n)
      return set_error(GG_ERR_BOUNDS, "source %lld of graph %lld out of 1:%lld", (long long)sources[g],
                       (long long)g, (long long)n);
    gsrc[g] = M->h_row_off[g] + sources[g] - 1;
  }
  GG_CUDA(cudaMemcpyAsync(M->d_src, gsrc.data(), M->ngraphs * sizeof(int64_t),
                          cudaMemcpyHostToDevice, ctx->stream));
  if (!M->gexec || M->dist_bound != dist) {
    if (M->gexec) {
      cudaGraphExecDestroy(M->gexec);
      M->gexec = nullptr;
    }
    int per_sm = 0;
    GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mg_bfs, 256, 0));
    if (per_sm < 1) return set_error(GG_ERR_CUDA, "k_mg_bfs cannot be resident");
    M->grid = ctx->num_sms * per_sm;  // every block resident: the cooperative barrier is safe
    cudaStream_t cs = nullptr;
    GG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    const int64_t nw = M->total_n / 32 + 2;
    const int odd_only = dtype_is_float(M->dtype) ? 0 : 1;  // floats: the Bool pattern
    int64_t G = M->ngraphs;
    if (e == cudaSuccess) e = cudaMemsetAsync(M->visited, 0, nw * sizeof(unsigned), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(M->bar, 0, 4 * sizeof(unsigned), cs);
    if (e == cudaSuccess) {
      k_mg_fill<<<mg_grid(ctx->num_sms, M->total_n), 256, 0, cs>>>(dist, M->total_n, INT32_MAX);
      k_mg_bfs_init<<<mg_grid(ctx->num_sms, G), 256, 0, cs>>>(G, M->d_src, M->visited, dist, M->q[0],
                                                              M->ctr);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
      int tv = M->dtype;
      void* args[] = {&G, &M->row_off, &M->rp64, &M->colval, &M->nzval, &tv,
                      (void*)&odd_only, &M->visited, &dist, &M->q[0], &M->q[1], &M->ctr, &M->bar};
      e = cudaLaunchCooperativeKernel((const void*)k_mg_bfs, dim3(M->grid), dim3(256), args, 0, cs);
    }
    cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&M->gexec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return cuda_error(e, "multigraph BFS graph capture");
    M->dist_bound = dist;
  }
  GG_CHECK(mg_set_polls(ctx, M));
  GG_CUDA(cudaGraphLaunch(M->gexec, ctx->stream));
  unsigned hb[4] = {0, 0, 0, 0};
  GG_CUDA(cudaMemcpyAsync(hb, M->bar, sizeof(hb), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hb[2]) return set_error(GG_ERR_TIMEOUT, "multigraph BFS barrier wait ran out");
  if (levels_out) *levels_out = hb[3];
  return GG_OK;
}

}  // extern "C"

template <typename T>
static int mg_sssp_capture(gg_ctx* ctx, gg_multigraph* M, T* dist) {
  int per_sm = 0;
  GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mg_sssp<T>, 256, 0));
  if (per_sm < 1) return set_error(GG_ERR_CUDA, "k_mg_sssp cannot be resident");
  const int grid = ctx->num_sms * per_sm;  // every block resident: the barrier is safe
  cudaStream_t cs = nullptr;
  GG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  const int64_t nw = M->total_n / 32 + 2;
  int64_t G = M->ngraphs;
  int64_t max_rounds = M->total_n + 1;
  if (e == cudaSuccess) e = cudaMemsetAsync(M->inq[0], 0, nw * sizeof(unsigned), cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(M->inq[1], 0, nw * sizeof(unsigned), cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(M->bar, 0, 4 * sizeof(unsigned), cs);
  if (e == cudaSuccess) {
    k_mg_fill_t<T><<<mg_grid(ctx->num_sms, M->total_n), 256, 0, cs>>>(dist, M->total_n, Lim<T>::max());
    k_mg_sssp_seed<T><<<mg_grid(ctx->num_sms, G), 256, 0, cs>>>(G, M->d_src, dist, M->inq[0],
                                                                M->q[0], M->ctr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    int tv = M->dtype;
    void* args[] = {&G, &M->row_off, &M->rp64, &M->colval, &M->nzval, &tv, &dist, &M->inq[0],
                    &M->inq[1], &M->q[0], &M->q[1], &M->ctr, &M->bar, &max_rounds};
    e = cudaLaunchCooperativeKernel((const void*)k_mg_sssp<T>, dim3(grid), dim3(256), args, 0, cs);
  }
  cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&M->sssp_gexec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) return cuda_error(e, "multigraph shortest-path graph capture");
  M->sssp_dist_bound = dist;
  return GG_OK;
}

extern "C" {

int gg_multigraph_sssp(gg_ctx* ctx, gg_multigraph* M, const int64_t* sources, void* dist,
                       int dist_dtype, int64_t* rounds_out) {
  if (!ctx || !M || !sources || !dist) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  const int want = M->dtype == GG_BOOL ? GG_INT32 : M->dtype;
  if (dist_dtype != want)
    return set_error(GG_ERR_TYPE, "dist element type must be Int32 for Bool graphs, else the graphs' type");
  GG_CUDA(cudaSetDevice(ctx->device));
  if (M->nonneg < 0) {
    GG_CUDA(cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream));
    k_mg_nonneg<<<mg_grid(ctx->num_sms, M->total_nnz), 256, 0, ctx->stream>>>(
        M->nzval, M->dtype, M->total_nnz, ctx->d_flags);
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    M->nonneg = ctx->h_flags[0] ? 0 : 1;
  }
  if (!M->nonneg)
    return set_error(GG_ERR_UNSUPPORTED, "multigraph shortest paths need non-negative weights");
  std::vector<int64_t> gsrc(M->ngraphs);
  for (int64_t g = 0; g < M->ngraphs; ++g) {
    const int64_t n = M->h_row_off[g + 1] - M->h_row_off[g];
    if (sources[g] < 1 || sources[g] > n)
      return set_error(GG_ERR_BOUNDS, "source %lld of graph %lld out of 1:%lld", (long long)sources[g],
                       (long long)g, (long long)n);
    gsrc[g] = M->h_row_off[g] + sources[g] - 1;
  }
  const int64_t nw = M->total_n / 32 + 2;
  if (!M->inq[0]) {
    GG_CUDA(cudaMalloc((void**)&M->inq[0], nw * sizeof(unsigned)));
    GG_CUDA(cudaMalloc((void**)&M->inq[1], nw * sizeof(unsigned)));
  }
  GG_CUDA(cudaMemcpyAsync(M->d_src, gsrc.data(), M->ngraphs * sizeof(int64_t),
                          cudaMemcpyHostToDevice, ctx->stream));
  if (!M->sssp_gexec || M->sssp_dist_bound != dist) {
    if (M->sssp_gexec) {
      cudaGraphExecDestroy(M->sssp_gexec);
      M->sssp_gexec = nullptr;
    }
    switch (dist_dtype) {
      case GG_INT32: GG_CHECK(mg_sssp_capture<int32_t>(ctx, M, static_cast<int32_t*>(dist))); break;
      case GG_INT64: GG_CHECK(mg_sssp_capture<int64_t>(ctx, M, static_cast<int64_t*>(dist))); break;
      case GG_FLOAT32: GG_CHECK(mg_sssp_capture<float>(ctx, M, static_cast<float*>(dist))); break;
      default: GG_CHECK(mg_sssp_capture<double>(ctx, M, static_cast<double*>(dist))); break;
    }
  }
  GG_CHECK(mg_set_polls(ctx, M));
  GG_CUDA(cudaGraphLaunch(M->sssp_gexec, ctx->stream));
  unsigned hb[4] = {0, 0, 0, 0};
  GG_CUDA(cudaMemcpyAsync(hb, M->bar, sizeof(hb), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hb[2] == 1) return set_error(GG_ERR_TIMEOUT, "multigraph shortest-path barrier wait ran out");
  if (hb[2] == 2) return set_error(GG_ERR_NOT_CONVERGED, "multigraph shortest paths did not converge");
  if (rounds_out) *rounds_out = hb[3];
  return GG_OK;
}

}  // extern "C"
