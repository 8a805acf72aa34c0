// gg_serve.cu -- continuous-batching query server over resident graphs.
//
// Queries: BFS levels from a source, shortest paths from a source, and k-step
// plus-times SpMV iterations (x <- A x, k times) from a dense start vector, each
// against one of the server's resident graphs.  A scheduler thread keeps, per graph
// and query kind, an executor with a fixed number of slots and advances all active
// slots together, one step per tick:
//  * BFS: 256 slots, one bit each in the packed frontier / visited words; a tick is
//    one bottom-up level for every active slot, each slot writing its own levels
//    (tick - admission tick) into its output;
//  * shortest paths: 32 slots, one distance column each (vertex-major, so one
//    in-neighbour is one 128-byte read); a tick is one relaxation round from the
//    vertices that changed in the previous round; a slot completes after a round
//    in which none of its distances dropped;
//  * SpMV iterations: 32 slots, one column of a row-major n x 32 block; a tick is one
//    SpMM of the block; a slot completes after its k steps.
// Requests that arrive while others run are admitted into free slots at the next
// tick (continuous batching).  Executors are created on first use and only when the
// device has the memory they need plus the configured reserve (admission by free
// HBM); requests wait in the queue otherwise.  Every slot's computation is
// independent of the other slots, so a result does not depend on the mix it ran in.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "gg_semiring.cuh"

namespace gg {

int graph_view(gg_ctx* ctx, gg_mat* A, const int32_t** rp, const int32_t** cv, const void** nz,
               bool* all_odd, bool* nonneg);

static const unsigned kFullS = 0xffffffffu;
static const int kBfsSlots = 256, kBfsW = 8, kColSlots = 32;

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t id;
  int kind;
  int graph;
  int64_t source;
  const float* x;
  int steps;
  void* out;
  double t_submit;
};

struct SrvGraph {
  const int32_t* rp;
  const int32_t* cv;
  const void* nz;
  int tv;
  bool odd_only;
  bool nonneg;
  int64_t n;
};

// ---------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool s_odd(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<const uint8_t*>(nz)[k] & 1;
    case GG_INT32: return static_cast<const int32_t*>(nz)[k] & 1;
    case GG_INT64: return static_cast<const int64_t*>(nz)[k] & 1;
  }
  return false;
}

// admission of BFS slots (bits in amask): clear their visited / frontier bits,
// fill their outputs with typemax, then seed their sources
__global__ void k_sb_admit_clear(int64_t n, unsigned* V, unsigned* F, const unsigned* amask,
                                 int32_t* const* outp, const int* slots, int nslots) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int w = 0; w < kBfsW; ++w) {
      V[v * kBfsW + w] &= ~amask[w];
      F[v * kBfsW + w] &= ~amask[w];
    }
    for (int i = 0; i < nslots; ++i) outp[slots[i]][v] = INT32_MAX;
  }
}

__global__ void k_sb_admit_seed(unsigned* V, unsigned* F, int32_t* const* outp, const int* slots,
                                const int64_t* srcs, int nslots) {
  for (int i = threadIdx.x; i < nslots; i += blockDim.x) {
    const int q = slots[i];
    const int64_t s = srcs[i];
    atomicOr(V + s * kBfsW + (q >> 5), 1u << (q & 31));
    atomicOr(F + s * kBfsW + (q >> 5), 1u << (q & 31));
    outp[q][s] = 0;
  }
}

// one level for every active BFS slot; act receives the OR of the new bits
__global__ void __launch_bounds__(256)
    k_sb_level(int64_t n, SrvGraph g, const unsigned* __restrict__ F, unsigned* Fn, unsigned* V,
               const unsigned* __restrict__ live, int32_t tick, const int32_t* __restrict__ start,
               int32_t* const* __restrict__ outp, unsigned* act) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned lm[kBfsW], seen[kBfsW];
#pragma unroll
  for (int w = 0; w < kBfsW; ++w) {
    lm[w] = live[w];
    seen[w] = 0;
  }
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t v = base + threadIdx.x;
    unsigned m[kBfsW], acc[kBfsW];
    bool open = false;
#pragma unroll
    for (int w = 0; w < kBfsW; ++w) {
      m[w] = 0;
      acc[w] = 0;
    }
    if (v < n) {
#pragma unroll
      for (int w = 0; w < kBfsW; ++w) {
        m[w] = ~V[v * kBfsW + w] & lm[w];
        open |= m[w] != 0;
      }
    }
    if (open) {
      const int64_t k1 = (int64_t)g.rp[v + 1] - 1;
      for (int64_t k = (int64_t)g.rp[v] - 1; k < k1; ++k) {
        if (g.odd_only && !s_odd(g.nz, g.tv, k)) continue;
        const int64_t u = (int64_t)__ldg(g.cv + k) - 1;
        bool full = true;
#pragma unroll
        for (int w = 0; w < kBfsW; ++w) {
          acc[w] |= __ldg(F + u * kBfsW + w);
          full &= (acc[w] & m[w]) == m[w];
        }
        if (full) break;
      }
    }
#pragma unroll
    for (int w = 0; w < kBfsW; ++w) {
      acc[w] &= m[w];
      seen[w] |= acc[w];
      if (v < n) {
        if (acc[w]) V[v * kBfsW + w] |= acc[w];
        Fn[v * kBfsW + w] = acc[w];
      }
    }
#pragma unroll
    for (int w = 0; w < kBfsW; ++w) {
      unsigned u = __reduce_or_sync(kFullS, acc[w]);
      while (u) {
        const int b = __ffs(u) - 1;
        u &= u - 1;
        const int q = w * 32 + b;
        if ((acc[w] >> b) & 1u) outp[q][v] = tick - start[q];
      }
    }
  }
#pragma unroll
  for (int w = 0; w < kBfsW; ++w) {
    const unsigned r = __reduce_or_sync(kFullS, seen[w]);
    if ((threadIdx.x & 31) == 0 && r) atomicOr(act + w, r);
  }
}

template <typename T> __device__ __forceinline__ T s_relax(T w, T d) {
  return (w == Lim<T>::max() || d == Lim<T>::max()) ? Lim<T>::max() : w_add(w, d);
}
template <typename T> __device__ __forceinline__ T s_weight(const void* nz, int tv, int64_t k) {
  switch (tv) {
    case GG_BOOL: return static_cast<T>(static_cast<const uint8_t*>(nz)[k]);
    case GG_INT32: return static_cast<T>(static_cast<const int32_t*>(nz)[k]);
    case GG_INT64: return static_cast<T>(static_cast<const int64_t*>(nz)[k]);
    case GG_FLOAT32: return static_cast<T>(static_cast<const float*>(nz)[k]);
  }
  return static_cast<T>(static_cast<const double*>(nz)[k]);
}

// admission of shortest-path columns: D[:, q] = typemax, D[s, q] = 0, s changed
template <typename T>
__global__ void k_ss_admit(int64_t n, T* D, unsigned qmask, uint8_t* chg, const int* slots,
                           const int64_t* srcs, int nslots) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    for (int q = 0; q < kColSlots; ++q)
      if ((qmask >> q) & 1u) D[v * kColSlots + q] = Lim<T>::max();
}
template <typename T>
__global__ void k_ss_seed(T* D, uint8_t* chg, const int* slots, const int64_t* srcs, int nslots) {
  for (int i = threadIdx.x; i < nslots; i += blockDim.x) {
    D[srcs[i] * kColSlots + slots[i]] = T(0);
    chg[srcs[i]] = 1;
  }
}

// one round for every column (inactive columns are at their fixpoint and do not
// move); drop receives the columns whose distances fell
template <typename T>
__global__ void __launch_bounds__(256)
    k_ss_round(int64_t n, SrvGraph g, T* D, const uint8_t* __restrict__ chg, uint8_t* chg_next,
               unsigned* drop) {
  const int lane = threadIdx.x & 31;
  unsigned dropped_cols = 0;
  for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n;
       v += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t k0 = (int64_t)g.rp[v] - 1, k1 = (int64_t)g.rp[v + 1] - 1;
    T best = Lim<T>::max();
    bool any = false;
    for (int64_t kb = k0; kb < k1; kb += 32) {
      const int64_t kk = kb + lane;
      int32_t u = -1;
      if (kk < k1) {
        const int32_t c = __ldg(g.cv + kk) - 1;
        if (chg[c]) u = c;
      }
      unsigned a = __ballot_sync(kFullS, u >= 0);
      while (a) {
        const int sl = __ffs(a) - 1;
        a &= a - 1;
        const int32_t uu = __shfl_sync(kFullS, u, sl);
        const T cand = s_relax(s_weight<T>(g.nz, g.tv, kb + sl), D[(int64_t)uu * kColSlots + lane]);
        if (cand < best) best = cand;
        any = true;
      }
    }
    bool dr = false;
    if (any) {
      T* dv = D + v * kColSlots + lane;
      if (best < *dv) {
        *dv = best;
        dr = true;
      }
    }
    const unsigned b = __ballot_sync(kFullS, dr);
    if (lane == 0) chg_next[v] = b ? 1 : 0;
    dropped_cols |= b;
  }
  if (lane == 0 && dropped_cols) atomicOr(drop, dropped_cols);
}

template <typename T>
__global__ void k_ss_out(const T* D, int64_t n, int q, T* out) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    out[v] = D[v * kColSlots + q];
}

// SpMV-iteration columns
__global__ void k_si_load(int64_t n, float* X, int q, const float* x) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    X[v * kColSlots + q] = x[v];
}
__global__ void k_si_out(int64_t n, const float* X, int q, float* out) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    out[v] = X[v * kColSlots + q];
}

int spmm_dispatch(gg_ctx* ctx, gg_mat* A, int tc, int mul, int add, int accum, void* C, int tcm,
                  int64_t ldc, const void* B, int tb, int64_t ldb, int64_t k, int layout,
                  const void* mask, int tmask, int64_t lo, int64_t hi);

// ---------------------------------------------------------------------------------
// executors
// ---------------------------------------------------------------------------------
struct Slot {
  bool busy = false;
  Request req;
  int32_t start = 0;
  int steps_left = 0;
};

struct Executor {
  int kind = 0;
  bool ready = false;
  std::vector<Slot> slots;
  std::vector<int> free_list;
  // BFS
  unsigned *F = nullptr, *Fn = nullptr, *V = nullptr, *live = nullptr, *act = nullptr;
  int32_t** outp = nullptr;
  int32_t* start = nullptr;
  int32_t tick = 0;
  // SSSP
  void* D = nullptr;
  uint8_t *c0 = nullptr, *c1 = nullptr;
  unsigned* drop = nullptr;
  int dtype = 0;
  // SpMV iterations
  float *X = nullptr, *Y = nullptr;
  // admission staging
  int* d_slots = nullptr;
  int64_t* d_srcs = nullptr;
  unsigned* d_amask = nullptr;
  unsigned* h_result = nullptr;  // pinned: act / drop of the last tick
  size_t bytes = 0;
  int active() const {
    int a = 0;
    for (auto& s : slots) a += s.busy;
    return a;
  }
};

}  // namespace gg

struct gg_server {
  gg_ctx* ctx = nullptr;
  gg_ctx own;  // private context state bound to the server stream
  cudaStream_t stream = nullptr;
  int64_t reserve = 0;
  std::vector<gg_mat*> graphs;
  std::vector<gg::SrvGraph> views;
  std::vector<std::vector<gg::Executor>> exec;  // [graph][kind]
  std::mutex mu;
  std::condition_variable cv;
  std::deque<gg::Request> queue;
  std::vector<int64_t> done_ids;
  std::vector<double> done_lat;
  int64_t next_id = 1;
  int64_t inflight = 0;
  bool stop = false;
  int error = GG_OK;
  std::string error_msg;
  std::thread worker;
  // statistics
  int64_t ticks = 0, admission_waits = 0;
};

namespace gg {

static int grid_s(gg_server* S, int64_t work) {
  int64_t g = (work + 255) / 256;
  const int64_t cap = (int64_t)S->own.num_sms * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

static size_t exec_bytes(int kind, int64_t n, int dtype) {
  switch (kind) {
    case GG_QUERY_BFS: return (size_t)n * kBfsW * 4 * 3 + 4096;
    case GG_QUERY_SSSP: return (size_t)n * kColSlots * dtype_size(dtype) + 2 * (size_t)n + 4096;
    default: return (size_t)n * kColSlots * 4 * 2 + 4096;
  }
}

static int exec_create(gg_server* S, int gi, int kind, Executor& E) {
  const SrvGraph& g = S->views[gi];
  const int64_t n = g.n;
  const int dt = S->graphs[gi]->dtype == GG_BOOL ? GG_INT32 : S->graphs[gi]->dtype;
  const size_t need = exec_bytes(kind, n, dt);
  size_t fr = 0, tot = 0;
  GG_CUDA(cudaMemGetInfo(&fr, &tot));
  if (fr < need + (size_t)S->reserve) return GG_ERR_OOM;  // stays queued
  E.kind = kind;
  E.dtype = dt;
  E.bytes = need;
  cudaStream_t st = S->stream;
  const int nslots = kind == GG_QUERY_BFS ? kBfsSlots : kColSlots;
  E.slots.assign(nslots, Slot());
  E.free_list.clear();
  for (int q = nslots - 1; q >= 0; --q) E.free_list.push_back(q);
  GG_CUDA(cudaMalloc((void**)&E.d_slots, nslots * sizeof(int)));
  GG_CUDA(cudaMalloc((void**)&E.d_srcs, nslots * sizeof(int64_t)));
  GG_CUDA(cudaMalloc((void**)&E.d_amask, 64));
  GG_CUDA(cudaMallocHost((void**)&E.h_result, 64));
  if (kind == GG_QUERY_BFS) {
    const size_t b = (size_t)n * kBfsW * 4;
    GG_CUDA(cudaMalloc((void**)&E.F, b));
    GG_CUDA(cudaMalloc((void**)&E.Fn, b));
    GG_CUDA(cudaMalloc((void**)&E.V, b));
    GG_CUDA(cudaMalloc((void**)&E.live, 64));
    GG_CUDA(cudaMalloc((void**)&E.act, 64));
    GG_CUDA(cudaMalloc((void**)&E.outp, kBfsSlots * sizeof(int32_t*)));
    GG_CUDA(cudaMalloc((void**)&E.start, kBfsSlots * sizeof(int32_t)));
    GG_CUDA(cudaMemsetAsync(E.F, 0, b, st));
    GG_CUDA(cudaMemsetAsync(E.Fn, 0, b, st));
    GG_CUDA(cudaMemsetAsync(E.V, 0, b, st));
    GG_CUDA(cudaMemsetAsync(E.outp, 0, kBfsSlots * sizeof(int32_t*), st));
  } else if (kind == GG_QUERY_SSSP) {
    GG_CUDA(cudaMalloc(&E.D, (size_t)n * kColSlots * dtype_size(dt)));
    GG_CUDA(cudaMalloc((void**)&E.c0, (size_t)n + 64));
    GG_CUDA(cudaMalloc((void**)&E.c1, (size_t)n + 64));
    GG_CUDA(cudaMalloc((void**)&E.drop, 64));
    GG_CUDA(cudaMemsetAsync(E.c0, 0, (size_t)n + 64, st));
    GG_CUDA(cudaMemsetAsync(E.c1, 0, (size_t)n + 64, st));
    // every column starts at the fixpoint of "no source": typemax everywhere
    GG_CUDA(cudaMemsetAsync(E.D, 0, (size_t)n * kColSlots * dtype_size(dt), st));
    const unsigned all = 0xffffffffu;
    switch (dt) {
      case GG_INT32: k_ss_admit<int32_t><<<grid_s(S, n), 256, 0, st>>>(n, (int32_t*)E.D, all, E.c0, nullptr, nullptr, 0); break;
      case GG_INT64: k_ss_admit<int64_t><<<grid_s(S, n), 256, 0, st>>>(n, (int64_t*)E.D, all, E.c0, nullptr, nullptr, 0); break;
      case GG_FLOAT32: k_ss_admit<float><<<grid_s(S, n), 256, 0, st>>>(n, (float*)E.D, all, E.c0, nullptr, nullptr, 0); break;
      default: k_ss_admit<double><<<grid_s(S, n), 256, 0, st>>>(n, (double*)E.D, all, E.c0, nullptr, nullptr, 0); break;
    }
  } else {
    GG_CUDA(cudaMalloc((void**)&E.X, (size_t)n * kColSlots * 4));
    GG_CUDA(cudaMalloc((void**)&E.Y, (size_t)n * kColSlots * 4));
    GG_CUDA(cudaMemsetAsync(E.X, 0, (size_t)n * kColSlots * 4, st));
  }
  GG_CUDA(cudaGetLastError());
  E.ready = true;
  return GG_OK;
}

static void exec_free(Executor& E) {
  cudaFree(E.F);
  cudaFree(E.Fn);
  cudaFree(E.V);
  cudaFree(E.live);
  cudaFree(E.act);
  cudaFree(E.outp);
  cudaFree(E.start);
  cudaFree(E.D);
  cudaFree(E.c0);
  cudaFree(E.c1);
  cudaFree(E.drop);
  cudaFree(E.X);
  cudaFree(E.Y);
  cudaFree(E.d_slots);
  cudaFree(E.d_srcs);
  cudaFree(E.d_amask);
  cudaFreeHost(E.h_result);
  E = Executor();
}

// admit waiting requests of (graph, kind) into free slots; returns how many
static int exec_admit(gg_server* S, int gi, Executor& E, std::vector<Request>& waiting) {
  if (waiting.empty() || E.free_list.empty()) return 0;
  const int64_t n = S->views[gi].n;
  cudaStream_t st = S->stream;
  std::vector<int> qs;
  std::vector<int64_t> srcs;
  unsigned amask[kBfsW] = {0};
  size_t taken = 0;
  while (taken < waiting.size() && !E.free_list.empty()) {
    const int q = E.free_list.back();
    E.free_list.pop_back();
    Slot& sl = E.slots[q];
    sl.busy = true;
    sl.req = waiting[taken++];
    sl.start = E.tick;
    sl.steps_left = sl.req.steps;
    qs.push_back(q);
    srcs.push_back(sl.req.source - 1);
    amask[q >> 5] |= 1u << (q & 31);
  }
  waiting.erase(waiting.begin(), waiting.begin() + taken);
  const int k = (int)qs.size();
  cudaMemcpyAsync(E.d_slots, qs.data(), k * sizeof(int), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(E.d_srcs, srcs.data(), k * sizeof(int64_t), cudaMemcpyHostToDevice, st);
  if (E.kind == GG_QUERY_BFS) {
    for (int i = 0; i < k; ++i) {
      int32_t* p = static_cast<int32_t*>(E.slots[qs[i]].req.out);
      cudaMemcpyAsync(E.outp + qs[i], &p, sizeof(p), cudaMemcpyHostToDevice, st);
      int32_t t0 = E.tick;
      cudaMemcpyAsync(E.start + qs[i], &t0, sizeof(t0), cudaMemcpyHostToDevice, st);
    }
    cudaMemcpyAsync(E.d_amask, amask, sizeof(amask), cudaMemcpyHostToDevice, st);
    k_sb_admit_clear<<<grid_s(S, n), 256, 0, st>>>(n, E.V, E.F, E.d_amask, E.outp, E.d_slots, k);
    k_sb_admit_seed<<<1, 256, 0, st>>>(E.V, E.F, E.outp, E.d_slots, E.d_srcs, k);
  } else if (E.kind == GG_QUERY_SSSP) {
    unsigned qm = 0;
    for (int q : qs) qm |= 1u << q;
    switch (E.dtype) {
      case GG_INT32:
        k_ss_admit<int32_t><<<grid_s(S, n), 256, 0, st>>>(n, (int32_t*)E.D, qm, E.c0, nullptr, nullptr, 0);
        k_ss_seed<int32_t><<<1, 64, 0, st>>>((int32_t*)E.D, E.c0, E.d_slots, E.d_srcs, k);
        break;
      case GG_INT64:
        k_ss_admit<int64_t><<<grid_s(S, n), 256, 0, st>>>(n, (int64_t*)E.D, qm, E.c0, nullptr, nullptr, 0);
        k_ss_seed<int64_t><<<1, 64, 0, st>>>((int64_t*)E.D, E.c0, E.d_slots, E.d_srcs, k);
        break;
      case GG_FLOAT32:
        k_ss_admit<float><<<grid_s(S, n), 256, 0, st>>>(n, (float*)E.D, qm, E.c0, nullptr, nullptr, 0);
        k_ss_seed<float><<<1, 64, 0, st>>>((float*)E.D, E.c0, E.d_slots, E.d_srcs, k);
        break;
      default:
        k_ss_admit<double><<<grid_s(S, n), 256, 0, st>>>(n, (double*)E.D, qm, E.c0, nullptr, nullptr, 0);
        k_ss_seed<double><<<1, 64, 0, st>>>((double*)E.D, E.c0, E.d_slots, E.d_srcs, k);
        break;
    }
  } else {
    for (int q : qs) k_si_load<<<grid_s(S, n), 256, 0, st>>>(n, E.X, q, E.slots[q].req.x);
  }
  return k;
}

// one tick of an executor (enqueued only; results read after the sync)
static int exec_tick(gg_server* S, int gi, Executor& E) {
  const SrvGraph& g = S->views[gi];
  const int64_t n = g.n;
  cudaStream_t st = S->stream;
  ++E.tick;
  if (E.kind == GG_QUERY_BFS) {
    unsigned live[kBfsW] = {0};
    for (int q = 0; q < kBfsSlots; ++q)
      if (E.slots[q].busy) live[q >> 5] |= 1u << (q & 31);
    cudaMemcpyAsync(E.live, live, sizeof(live), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(E.act, 0, 64, st);
    k_sb_level<<<grid_s(S, n), 256, 0, st>>>(n, g, E.F, E.Fn, E.V, E.live, E.tick, E.start, E.outp,
                                            E.act);
    std::swap(E.F, E.Fn);
    cudaMemcpyAsync(E.h_result, E.act, kBfsW * 4, cudaMemcpyDeviceToHost, st);
  } else if (E.kind == GG_QUERY_SSSP) {
    cudaMemsetAsync(E.drop, 0, 4, st);
    const int gw = grid_s(S, n * 32);
    switch (E.dtype) {
      case GG_INT32: k_ss_round<int32_t><<<gw, 256, 0, st>>>(n, g, (int32_t*)E.D, E.c0, E.c1, E.drop); break;
      case GG_INT64: k_ss_round<int64_t><<<gw, 256, 0, st>>>(n, g, (int64_t*)E.D, E.c0, E.c1, E.drop); break;
      case GG_FLOAT32: k_ss_round<float><<<gw, 256, 0, st>>>(n, g, (float*)E.D, E.c0, E.c1, E.drop); break;
      default: k_ss_round<double><<<gw, 256, 0, st>>>(n, g, (double*)E.D, E.c0, E.c1, E.drop); break;
    }
    std::swap(E.c0, E.c1);
    cudaMemcpyAsync(E.h_result, E.drop, 4, cudaMemcpyDeviceToHost, st);
  } else {
    int tc = GG_FLOAT32;
    GG_CHECK(spmm_dispatch(&S->own, S->graphs[gi], tc, GG_OP_MUL, GG_OP_ADD, GG_OP_SECOND, E.Y,
                           GG_FLOAT32, kColSlots, E.X, GG_FLOAT32, kColSlots, kColSlots,
                           GG_ROW_MAJOR, nullptr, 0, 0, 0));
    std::swap(E.X, E.Y);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// after the tick's sync: retire the slots that finished
static void exec_retire(gg_server* S, int gi, Executor& E, std::vector<Request>& finished) {
  const int64_t n = S->views[gi].n;
  cudaStream_t st = S->stream;
  for (int q = 0; q < (int)E.slots.size(); ++q) {
    Slot& sl = E.slots[q];
    if (!sl.busy) continue;
    bool done = false;
    if (E.kind == GG_QUERY_BFS) {
      done = !((E.h_result[q >> 5] >> (q & 31)) & 1u);  // no new vertex this level
    } else if (E.kind == GG_QUERY_SSSP) {
      done = !((E.h_result[0] >> q) & 1u);  // no distance of this column dropped
      if (done) {
        switch (E.dtype) {
          case GG_INT32: k_ss_out<int32_t><<<grid_s(S, n), 256, 0, st>>>((const int32_t*)E.D, n, q, (int32_t*)sl.req.out); break;
          case GG_INT64: k_ss_out<int64_t><<<grid_s(S, n), 256, 0, st>>>((const int64_t*)E.D, n, q, (int64_t*)sl.req.out); break;
          case GG_FLOAT32: k_ss_out<float><<<grid_s(S, n), 256, 0, st>>>((const float*)E.D, n, q, (float*)sl.req.out); break;
          default: k_ss_out<double><<<grid_s(S, n), 256, 0, st>>>((const double*)E.D, n, q, (double*)sl.req.out); break;
        }
      }
    } else {
      done = --sl.steps_left <= 0;
      if (done) k_si_out<<<grid_s(S, n), 256, 0, st>>>(n, E.X, q, static_cast<float*>(sl.req.out));
    }
    if (done) {
      sl.busy = false;
      E.free_list.push_back(q);
      finished.push_back(sl.req);
    }
  }
}

static void server_loop(gg_server* S) {
  cudaSetDevice(S->own.device);
  // waiting requests per (graph, kind)
  std::vector<std::vector<std::vector<Request>>> waiting(S->graphs.size(),
                                                        std::vector<std::vector<Request>>(3));
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      bool busy = false;
      for (auto& per_g : S->exec)
        for (auto& E : per_g) busy |= E.ready && E.active() > 0;
      for (auto& per_g : waiting)
        for (auto& w : per_g) busy |= !w.empty();
      if (!busy && S->queue.empty() && !S->stop)
        S->cv.wait_for(lk, std::chrono::milliseconds(50));
      if (S->stop) break;
      while (!S->queue.empty()) {
        Request r = S->queue.front();
        S->queue.pop_front();
        waiting[r.graph][r.kind - 1].push_back(r);
      }
    }
    int rc = GG_OK;
    bool ticked = false;
    for (size_t gi = 0; gi < S->graphs.size() && rc == GG_OK; ++gi) {
      for (int kk = 0; kk < 3 && rc == GG_OK; ++kk) {
        Executor& E = S->exec[gi][kk];
        if (!E.ready && !waiting[gi][kk].empty()) {
          const int c = exec_create(S, (int)gi, kk + 1, E);
          if (c == GG_ERR_OOM) {
            exec_free(E);
            ++S->admission_waits;  // not enough free HBM yet: keep the requests queued
            continue;
          }
          rc = c;
          if (rc) break;
        }
        if (!E.ready) continue;
        exec_admit(S, (int)gi, E, waiting[gi][kk]);
        if (E.active() > 0) {
          rc = exec_tick(S, (int)gi, E);
          ticked = true;
        }
      }
    }
    if (rc == GG_OK && ticked) {
      cudaError_t e = cudaStreamSynchronize(S->stream);
      if (e != cudaSuccess) rc = cuda_error(e, "server tick");
    }
    std::vector<Request> finished;
    if (rc == GG_OK && ticked) {
      for (size_t gi = 0; gi < S->graphs.size(); ++gi)
        for (int kk = 0; kk < 3; ++kk)
          if (S->exec[gi][kk].ready) exec_retire(S, (int)gi, S->exec[gi][kk], finished);
      if (!finished.empty()) {
        cudaError_t e = cudaStreamSynchronize(S->stream);  // result copies
        if (e != cudaSuccess) rc = cuda_error(e, "server results");
      }
      ++S->ticks;
    }
    const double t = now_s();
    std::lock_guard<std::mutex> lk(S->mu);
    for (auto& r : finished) {
      S->done_ids.push_back(r.id);
      S->done_lat.push_back(t - r.t_submit);
      --S->inflight;
    }
    if (rc != GG_OK) {
      S->error = rc;
      S->error_msg = gg_last_error();
      S->stop = true;
      break;
    }
  }
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_server_create(gg_ctx* ctx, int64_t reserve_bytes, gg_server** out) {
  if (!ctx || !out) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  *out = nullptr;
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_server* S = new gg_server();
  S->ctx = ctx;
  S->reserve = reserve_bytes < 0 ? 0 : reserve_bytes;
  cudaError_t e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete S;
    return cuda_error(e, "gg_server_create");
  }
  S->own.device = ctx->device;
  S->own.num_sms = ctx->num_sms;
  S->own.stream = S->stream;
  e = cudaMalloc((void**)&S->own.d_flags, 64 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&S->own.h_flags, 64 * sizeof(unsigned));
  if (e != cudaSuccess) {
    cudaStreamDestroy(S->stream);
    delete S;
    return cuda_error(e, "gg_server_create");
  }
  *out = S;
  return GG_OK;
}

int gg_server_add_graph(gg_server* S, const gg_mat* A_T, int* graph_id) {
  if (!S || !A_T || !graph_id) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (S->worker.joinable()) return set_error(GG_ERR_ARGUMENT, "add graphs before the first submit");
  if (A_T->m != A_T->n) return set_error(GG_ERR_DIMENSION, "A_T must be square");
  gg_mat* A = const_cast<gg_mat*>(A_T);
  SrvGraph g;
  bool all_odd = false, nonneg = false;
  GG_CHECK(graph_view(&S->own, A, &g.rp, &g.cv, &g.nz, &all_odd, &nonneg));
  g.tv = A->dtype;
  g.odd_only = !all_odd;
  g.nonneg = nonneg;
  g.n = A->m;
  S->graphs.push_back(A);
  S->views.push_back(g);
  S->exec.emplace_back(3);
  *graph_id = (int)S->graphs.size() - 1;
  return GG_OK;
}

int gg_server_submit(gg_server* S, int kind, int graph, int64_t source, const float* x, int steps,
                     void* out, int64_t* request_id) {
  if (!S || !out) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (graph < 0 || graph >= (int)S->graphs.size()) return set_error(GG_ERR_ARGUMENT, "unknown graph %d", graph);
  const SrvGraph& g = S->views[graph];
  if (kind == GG_QUERY_BFS || kind == GG_QUERY_SSSP) {
    if (source < 1 || source > g.n) return set_error(GG_ERR_BOUNDS, "source %lld out of 1:%lld", (long long)source, (long long)g.n);
    if (kind == GG_QUERY_BFS && dtype_is_float(g.tv))
      return set_error(GG_ERR_UNSUPPORTED, "GPUGraphs_band has no method for floating-point matrices");
    if (kind == GG_QUERY_SSSP && !g.nonneg)
      return set_error(GG_ERR_UNSUPPORTED, "served shortest paths need non-negative weights");
  } else if (kind == GG_QUERY_SPMV_ITER) {
    if (!x || steps < 1) return set_error(GG_ERR_ARGUMENT, "SpMV iteration needs x and steps >= 1");
    if (S->graphs[graph]->dtype != GG_FLOAT32)
      return set_error(GG_ERR_TYPE, "served SpMV iterations need a Float32 matrix");
  } else {
    return set_error(GG_ERR_ARGUMENT, "unknown query kind %d", kind);
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return S->error ? set_error(S->error, "server stopped: %s", S->error_msg.c_str())
                                 : set_error(GG_ERR_ARGUMENT, "server stopped");
    Request r;
    r.id = S->next_id++;
    r.kind = kind;
    r.graph = graph;
    r.source = source;
    r.x = x;
    r.steps = steps;
    r.out = out;
    r.t_submit = now_s();
    S->queue.push_back(r);
    ++S->inflight;
    if (request_id) *request_id = r.id;
    if (!S->worker.joinable()) S->worker = std::thread(server_loop, S);
  }
  S->cv.notify_one();
  return GG_OK;
}

int gg_server_poll(gg_server* S, int64_t* ids, double* latency_s, int64_t max, int64_t* ndone,
                   int64_t* inflight) {
  if (!S || !ndone) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  const int64_t k = std::min<int64_t>(max, (int64_t)S->done_ids.size());
  for (int64_t i = 0; i < k; ++i) {
    if (ids) ids[i] = S->done_ids[i];
    if (latency_s) latency_s[i] = S->done_lat[i];
  }
  S->done_ids.erase(S->done_ids.begin(), S->done_ids.begin() + k);
  S->done_lat.erase(S->done_lat.begin(), S->done_lat.begin() + k);
  *ndone = k;
  if (inflight) *inflight = S->inflight;
  if (S->error) return set_error(S->error, "server stopped: %s", S->error_msg.c_str());
  return GG_OK;
}

int gg_server_stats(gg_server* S, int64_t* ticks, int64_t* admission_waits, int64_t* exec_bytes) {
  if (!S) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  if (ticks) *ticks = S->ticks;
  if (admission_waits) *admission_waits = S->admission_waits;
  if (exec_bytes) {
    int64_t b = 0;
    for (auto& per_g : S->exec)
      for (auto& E : per_g) b += E.ready ? (int64_t)E.bytes : 0;
    *exec_bytes = b;
  }
  return GG_OK;
}

int gg_server_destroy(gg_server* S) {
  if (!S) return GG_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv.notify_one();
  if (S->worker.joinable()) S->worker.join();
  cudaSetDevice(S->own.device);
  cudaStreamSynchronize(S->stream);
  for (auto& per_g : S->exec)
    for (auto& E : per_g) exec_free(E);
  cudaFree(S->own.d_flags);
  cudaFreeHost(S->own.h_flags);
  cudaFree(S->own.scratch);
  cudaStreamDestroy(S->stream);
  delete S;
  return GG_OK;
}

}  // extern "C"
