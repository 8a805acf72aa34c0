// gg_serve.cu -- continuous-batching query server over resident graphs.
//
// Queries: BFS levels from a source, shortest paths from a source, and k-step
// plus-times SpMV iterations (x <- A x, k times) from a dense start vector, each
// against one of the server's resident graphs.  A scheduler thread keeps, per graph
// and query kind, an executor with a fixed number of slots and advances all active
// slots of an executor together, one step per tick:
//  * BFS: 256 slots, one bit each in the packed frontier / visited words; a tick is
//    one bottom-up level for the slots whose frontier is not empty, each slot
//    writing its own levels (tick - admission tick) into its output;
//  * shortest paths: 32 slots, one distance column each (vertex-major); a tick is
//    one relaxation round from the vertices that changed in the previous round; a
//    slot completes after a round in which none of its distances dropped;
//  * SpMV iterations: 32 slots, one column of a row-major n x 32 block; a tick is one
//    SpMM of the block; a slot completes after its k steps.
// (BFS and shortest-path kernels: gg_msearch.cuh, hub-aware.)  Every executor owns
// a CUDA stream and a private context; the scheduler never waits for the GPU: it
// polls each executor's tick event, retires finished slots, admits waiting requests
// into free slots (continuous batching) and enqueues the next tick, so small graphs'
// queries advance at their own pace beside long searches on large graphs.
// Executors are created on first use and only when the device has the memory they
// need plus the configured reserve (admission by free HBM); requests wait in the
// queue otherwise.  Every slot's computation is independent of the other slots, so a
// result does not depend on the mix it ran in.
#include <algorithm>
#include <cstring>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "gg_msearch.cuh"

namespace gg {

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
  BatchGraph g;
  bool nonneg;
  int64_t n;
};

// ---------------------------------------------------------------------------------
// admission / output kernels
// ---------------------------------------------------------------------------------
// BFS slots (bits in amask): clear their visited / frontier bits and fill their
// outputs with typemax, then seed their sources
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

// shortest-path columns in qmask: D[:, q] = typemax
template <typename T>
__global__ void k_ss_admit(int64_t n, T* D, unsigned qmask) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    for (int q = 0; q < kColSlots; ++q)
      if ((qmask >> q) & 1u) D[v * kColSlots + q] = Lim<T>::max();
}
template <typename T>
__global__ void k_ss_seed(T* D, unsigned* chg, const int* slots, const int64_t* srcs, int nslots,
                          int32_t* cq, unsigned long long* ncq) {
  for (int i = threadIdx.x; i < nslots; i += blockDim.x) {
    D[srcs[i] * kColSlots + slots[i]] = T(0);
    atomicOr(chg + srcs[i], 1u << slots[i]);
    cq[atomicAdd(ncq, 1ull)] = (int32_t)srcs[i];  // changed for the next round's marking
  }
}

template <typename T>
__global__ void k_ss_out(const T* D, int64_t n, int q, T* out) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    out[v] = D[v * kColSlots + q];
}

__global__ void k_fill_levels(int32_t* d, int64_t n) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    d[v] = INT32_MAX;
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
  gg_ctx ectx;  // private stream and scratch
  cudaEvent_t ev = nullptr, ev_out = nullptr;
  bool inflight = false;
  std::vector<Request> finishing;  // results being copied out (ev_out)
  std::vector<Slot> slots;
  std::vector<int> free_list;
  // BFS
  unsigned *F = nullptr, *Fn = nullptr, *V = nullptr, *act = nullptr, *hacc = nullptr;
  int32_t** outp = nullptr;
  int32_t* start = nullptr;
  int32_t tick = 0;
  unsigned act_host[kBfsW] = {0};  // sources whose frontier is not empty
  // SSSP
  void* D = nullptr;
  unsigned *c0 = nullptr, *c1 = nullptr;  // columns of each vertex that dropped
  // frontier-restricted rounds: changed queues, marked vertices (gg_msearch.cuh)
  int32_t* cq[2] = {nullptr, nullptr};
  int32_t* vlist = nullptr;
  unsigned* mark = nullptr;
  int32_t* mhq = nullptr;    // hubs among the changed vertices, marked in pieces
  int32_t* mhoff = nullptr;  // their piece offsets
  int cq_cur = 0;
  int64_t nchanged = 0;
  const int32_t* prow = nullptr;
  const int32_t* pcol = nullptr;
  int dtype = 0;
  // SpMV iterations
  float *X = nullptr, *Y = nullptr;
  // staging (pinned host / device)
  int* d_slots = nullptr;
  int64_t* d_srcs = nullptr;
  unsigned* d_amask = nullptr;
  unsigned long long* d_cnt = nullptr;
  unsigned* h_stage = nullptr;   // pinned: small uploads
  unsigned* h_result = nullptr;  // pinned: new bits / dropped columns of the last tick
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
  gg_ctx own;  // context used for graph analysis on the server's stream
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
  // solo workers: a request that finds its executor idle runs alone through the
  // single-query engine on a worker's own context and stream
  struct SoloJob {
    gg::Request req;
  };
  std::vector<std::thread> solo_threads;
  std::vector<gg_ctx*> solo_ctx;
  // each worker's two streams: highest priority for short queries (BFS, and every
  // query on graphs below 2^20 vertices), lowest for long searches and iterations
  std::vector<cudaStream_t> solo_hi, solo_lo;
  std::deque<SoloJob> solo_q;
  std::condition_variable solo_cv;
  int solo_idle = 0;
  std::vector<std::vector<char>> solo_active;  // [graph][kind], scheduler-owned
  std::vector<std::pair<int, int>> solo_finished;  // (graph, kind) released by workers
  // statistics
  int64_t ticks = 0, admission_waits = 0, solo_runs = 0;
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
    // distances, changed-column masks (2 x 4n), changed queues, marks and hub lists (~20n)
    case GG_QUERY_SSSP: return (size_t)n * kColSlots * dtype_size(dtype) + 28 * (size_t)n + 4096;
    default: return (size_t)n * kColSlots * 4 * 2 + 4096;
  }
}

static void exec_free(Executor& E) {
  if (E.ectx.stream) cudaStreamSynchronize(E.ectx.stream);
  cudaFree(E.F);
  cudaFree(E.Fn);
  cudaFree(E.V);
  cudaFree(E.act);
  cudaFree(E.hacc);
  cudaFree(E.outp);
  cudaFree(E.start);
  cudaFree(E.D);
  cudaFree(E.c0);
  cudaFree(E.c1);
  cudaFree(E.cq[0]);
  cudaFree(E.cq[1]);
  cudaFree(E.vlist);
  cudaFree(E.mark);
  cudaFree(E.mhq);
  cudaFree(E.mhoff);
  cudaFree(E.X);
  cudaFree(E.Y);
  cudaFree(E.d_slots);
  cudaFree(E.d_srcs);
  cudaFree(E.d_amask);
  cudaFree(E.d_cnt);
  cudaFreeHost(E.h_stage);
  cudaFreeHost(E.h_result);
  cudaFree(E.ectx.scratch);
  cudaFree(E.ectx.d_flags);
  cudaFreeHost(E.ectx.h_flags);
  if (E.ev) cudaEventDestroy(E.ev);
  if (E.ev_out) cudaEventDestroy(E.ev_out);
  if (E.ectx.stream) cudaStreamDestroy(E.ectx.stream);
  E.ectx.scratch = nullptr;
  E = Executor();
}

static int exec_create(gg_server* S, int gi, int kind, Executor& E) {
  const SrvGraph& sg = S->views[gi];
  const int64_t n = sg.n;
  const int dt = S->graphs[gi]->dtype == GG_BOOL ? GG_INT32 : S->graphs[gi]->dtype;
  const size_t need = exec_bytes(kind, n, dt);
  size_t fr = 0, tot = 0;
  GG_CUDA(cudaMemGetInfo(&fr, &tot));
  if (fr < need + (size_t)S->reserve) return GG_ERR_OOM;  // stays queued
  E.kind = kind;
  E.dtype = dt;
  E.bytes = need;
  E.ectx.device = S->own.device;
  E.ectx.num_sms = S->own.num_sms;
  // short queries first: executors of smaller graphs get higher stream priorities,
  // so their ticks are scheduled ahead of long searches on large graphs
  int least = 0, greatest = 0;
  GG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  int lg = 0;
  while ((int64_t(1) << (lg + 1)) <= n) ++lg;
  int prio = greatest + (lg > 16 ? (lg - 16) / 2 : 0);
  if (kind == GG_QUERY_SSSP) prio += 1;
  if (prio > least) prio = least;
  GG_CUDA(cudaStreamCreateWithPriority(&E.ectx.stream, cudaStreamNonBlocking, prio));
  GG_CUDA(cudaEventCreateWithFlags(&E.ev, cudaEventDisableTiming));
  GG_CUDA(cudaEventCreateWithFlags(&E.ev_out, cudaEventDisableTiming));
  GG_CUDA(cudaMalloc((void**)&E.ectx.d_flags, 64 * sizeof(unsigned)));
  GG_CUDA(cudaMallocHost((void**)&E.ectx.h_flags, 64 * sizeof(unsigned)));
  cudaStream_t st = E.ectx.stream;
  const int nslots = kind == GG_QUERY_BFS ? kBfsSlots : kColSlots;
  E.slots.assign(nslots, Slot());
  E.free_list.clear();
  for (int q = nslots - 1; q >= 0; --q) E.free_list.push_back(q);
  GG_CUDA(cudaMalloc((void**)&E.d_slots, nslots * sizeof(int)));
  GG_CUDA(cudaMalloc((void**)&E.d_srcs, nslots * sizeof(int64_t)));
  GG_CUDA(cudaMalloc((void**)&E.d_amask, 64));
  GG_CUDA(cudaMalloc((void**)&E.d_cnt, 64));
  GG_CUDA(cudaMallocHost((void**)&E.h_stage, 4096));
  GG_CUDA(cudaMallocHost((void**)&E.h_result, 64));
  if (kind != GG_QUERY_SPMV_ITER)
    GG_CHECK(build_hub_plan(&S->own, S->graphs[gi], sg.g.rowptr, n));
  if (kind == GG_QUERY_BFS) {
    const size_t b = (size_t)n * kBfsW * 4;
    const HubPlan* hp = S->graphs[gi]->hubplan;
    GG_CUDA(cudaMalloc((void**)&E.F, b));
    GG_CUDA(cudaMalloc((void**)&E.Fn, b));
    GG_CUDA(cudaMalloc((void**)&E.V, b));
    GG_CUDA(cudaMalloc((void**)&E.act, 2 * kBfsW * sizeof(unsigned)));
    GG_CUDA(cudaMalloc((void**)&E.hacc, (hp->nhub + 1) * kBfsW * sizeof(unsigned)));
    GG_CUDA(cudaMalloc((void**)&E.outp, kBfsSlots * sizeof(int32_t*)));
    GG_CUDA(cudaMalloc((void**)&E.start, kBfsSlots * sizeof(int32_t)));
    GG_CUDA(cudaMemsetAsync(E.F, 0, b, st));
    GG_CUDA(cudaMemsetAsync(E.Fn, 0, b, st));
    GG_CUDA(cudaMemsetAsync(E.V, 0, b, st));
    GG_CUDA(cudaMemsetAsync(E.hacc, 0, (hp->nhub + 1) * kBfsW * sizeof(unsigned), st));
    GG_CUDA(cudaMemsetAsync(E.outp, 0, kBfsSlots * sizeof(int32_t*), st));
  } else if (kind == GG_QUERY_SSSP) {
    GG_CUDA(cudaMalloc(&E.D, (size_t)n * kColSlots * dtype_size(dt)));
    GG_CUDA(cudaMalloc((void**)&E.c0, ((size_t)n + 64) * sizeof(unsigned)));
    GG_CUDA(cudaMalloc((void**)&E.c1, ((size_t)n + 64) * sizeof(unsigned)));
    GG_CUDA(cudaMemsetAsync(E.c0, 0, ((size_t)n + 64) * sizeof(unsigned), st));
    GG_CUDA(cudaMemsetAsync(E.c1, 0, ((size_t)n + 64) * sizeof(unsigned), st));
    const HubPlan* hp = S->graphs[gi]->hubplan;
    const int64_t qcap = n + hp->npiece + kColSlots + 64;  // a hub may be queued once per piece
    GG_CUDA(cudaMalloc((void**)&E.cq[0], qcap * sizeof(int32_t)));
    GG_CUDA(cudaMalloc((void**)&E.cq[1], qcap * sizeof(int32_t)));
    GG_CUDA(cudaMalloc((void**)&E.vlist, (n + 64) * sizeof(int32_t)));
    GG_CUDA(cudaMalloc((void**)&E.mark, ((n + 31) / 32 + 2) * sizeof(unsigned)));
    GG_CUDA(cudaMalloc((void**)&E.mhq, (n + 64) * sizeof(int32_t)));
    GG_CUDA(cudaMalloc((void**)&E.mhoff, (n + 65) * sizeof(int32_t)));
    GG_CUDA(cudaMemsetAsync(E.d_cnt, 0, 64, st));  // [0] count, [1]/[2] queue lengths, [3] marked
    GG_CHECK(push_view(&S->own, S->graphs[gi], &E.prow, &E.pcol));
    // every column starts at the fixpoint of "no source": typemax everywhere
    const unsigned all = 0xffffffffu;
    switch (dt) {
      case GG_INT32: k_ss_admit<int32_t><<<grid_s(S, n), 256, 0, st>>>(n, (int32_t*)E.D, all); break;
      case GG_INT64: k_ss_admit<int64_t><<<grid_s(S, n), 256, 0, st>>>(n, (int64_t*)E.D, all); break;
      case GG_FLOAT32: k_ss_admit<float><<<grid_s(S, n), 256, 0, st>>>(n, (float*)E.D, all); break;
      default: k_ss_admit<double><<<grid_s(S, n), 256, 0, st>>>(n, (double*)E.D, all); break;
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

// admit waiting requests of (graph, kind) into free slots; returns how many
static int exec_admit(gg_server* S, int gi, Executor& E, std::vector<Request>& waiting) {
  if (waiting.empty() || E.free_list.empty()) return 0;
  const int64_t n = S->views[gi].n;
  cudaStream_t st = E.ectx.stream;
  // staging layout in pinned memory: slots [0,256) ints | sources [256,512) int64 |
  // output pointers [512, 768) | start ticks [768, 1024) -- in 4-byte words
  int* hs = reinterpret_cast<int*>(E.h_stage);
  int64_t* hsrc = reinterpret_cast<int64_t*>(E.h_stage + 256);
  int k = 0;
  unsigned amask[kBfsW] = {0};
  size_t taken = 0;
  // lowest free slot first (descending list, taken from the back)
  std::sort(E.free_list.begin(), E.free_list.end(), [](int x, int y) { return x > y; });
  while (taken < waiting.size() && !E.free_list.empty()) {
    const int q = E.free_list.back();
    E.free_list.pop_back();
    Slot& sl = E.slots[q];
    sl.busy = true;
    sl.req = waiting[taken++];
    sl.start = E.tick;
    sl.steps_left = sl.req.steps;
    hs[k] = q;
    hsrc[k] = sl.req.source - 1;
    amask[q >> 5] |= 1u << (q & 31);
    ++k;
  }
  waiting.erase(waiting.begin(), waiting.begin() + taken);
  GG_CUDA(cudaMemcpyAsync(E.d_slots, hs, k * sizeof(int), cudaMemcpyHostToDevice, st));
  GG_CUDA(cudaMemcpyAsync(E.d_srcs, hsrc, k * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  if (E.kind == GG_QUERY_BFS) {
    for (int i = 0; i < k; ++i) {
      const int q = hs[i];
      int32_t* p = static_cast<int32_t*>(E.slots[q].req.out);
      GG_CUDA(cudaMemcpyAsync(E.outp + q, &p, sizeof(p), cudaMemcpyHostToDevice, st));
      int32_t t0 = E.tick;
      GG_CUDA(cudaMemcpyAsync(E.start + q, &t0, sizeof(t0), cudaMemcpyHostToDevice, st));
    }
    unsigned* ham = E.h_stage + 1000;
    for (int w = 0; w < kBfsW; ++w) {
      ham[w] = amask[w];
      E.act_host[w] |= amask[w];
    }
    GG_CUDA(cudaMemcpyAsync(E.d_amask, ham, kBfsW * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    k_sb_admit_clear<<<grid_s(S, n), 256, 0, st>>>(n, E.V, E.F, E.d_amask, E.outp, E.d_slots, k);
    k_sb_admit_seed<<<1, 256, 0, st>>>(E.V, E.F, E.outp, E.d_slots, E.d_srcs, k);
  } else if (E.kind == GG_QUERY_SSSP) {
    const unsigned qm = amask[0];
    E.nchanged += k;
    switch (E.dtype) {
      case GG_INT32:
        k_ss_admit<int32_t><<<grid_s(S, n), 256, 0, st>>>(n, (int32_t*)E.D, qm);
        k_ss_seed<int32_t><<<1, 64, 0, st>>>((int32_t*)E.D, E.c0, E.d_slots, E.d_srcs, k, E.cq[E.cq_cur],
                                       E.d_cnt + 1 + E.cq_cur);
        break;
      case GG_INT64:
        k_ss_admit<int64_t><<<grid_s(S, n), 256, 0, st>>>(n, (int64_t*)E.D, qm);
        k_ss_seed<int64_t><<<1, 64, 0, st>>>((int64_t*)E.D, E.c0, E.d_slots, E.d_srcs, k, E.cq[E.cq_cur],
                                       E.d_cnt + 1 + E.cq_cur);
        break;
      case GG_FLOAT32:
        k_ss_admit<float><<<grid_s(S, n), 256, 0, st>>>(n, (float*)E.D, qm);
        k_ss_seed<float><<<1, 64, 0, st>>>((float*)E.D, E.c0, E.d_slots, E.d_srcs, k, E.cq[E.cq_cur],
                                       E.d_cnt + 1 + E.cq_cur);
        break;
      default:
        k_ss_admit<double><<<grid_s(S, n), 256, 0, st>>>(n, (double*)E.D, qm);
        k_ss_seed<double><<<1, 64, 0, st>>>((double*)E.D, E.c0, E.d_slots, E.d_srcs, k, E.cq[E.cq_cur],
                                       E.d_cnt + 1 + E.cq_cur);
        break;
    }
  } else {
    for (int i = 0; i < k; ++i)
      k_si_load<<<grid_s(S, n), 256, 0, st>>>(n, E.X, hs[i], E.slots[hs[i]].req.x);
  }
  GG_CUDA(cudaGetLastError());
  return k;
}

// shared memory of the SELL-32 full rounds (more than the default 48 KB per CTA)
template <typename T>
static int sell_round_attr() {
  GG_CUDA(cudaFuncSetAttribute(k_ms_round_sell<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(kMsSellWarps * sizeof(MsSellWarpSmem<T>))));
  return GG_OK;
}

template <typename T>
static void ss_round(gg_server* S, Executor& E, const SrvGraph& sg, const HubPlan* hp,
                     int64_t nnz, const gg_mat* sell) {
  cudaStream_t st = E.ectx.stream;
  const int64_t n = sg.n;
  T* D = static_cast<T*>(E.D);
  const int cur = E.cq_cur;
  unsigned long long* ncq_cur = E.d_cnt + 1 + cur;
  unsigned long long* ncq_nxt = E.d_cnt + 1 + (cur ^ 1);
  cudaMemsetAsync(ncq_nxt, 0, sizeof(unsigned long long), st);
  const int64_t avg_deg = n > 0 ? (nnz + n - 1) / n : 1;
  // few changed vertices: visit only their out-neighbours (same fixpoint)
  const bool restricted = E.nchanged * avg_deg * (sell ? 32 : 4) < nnz;
  if (restricted) {
    cudaMemsetAsync(E.mark, 0, ((n + 31) / 32) * sizeof(unsigned), st);
    cudaMemsetAsync(E.d_cnt + 3, 0, sizeof(unsigned long long), st);
    launch_ms_mark(st, S->own.num_sms, E.nchanged, E.prow, E.pcol, E.cq[cur], ncq_cur, E.mark,
                   E.vlist, E.d_cnt + 3, E.mhq, E.d_cnt + 4, E.mhoff);
    k_ms_round<T><<<grid_s(S, n * 32), 256, 0, st>>>(n, sg.g, D, E.c0, E.c1, E.d_cnt, E.d_amask,
                                                      E.vlist, E.d_cnt + 3, E.cq[cur ^ 1], ncq_nxt);
  } else {
    if constexpr (sizeof(T) == 4) {
      if (sell) {
        // every vertex over the graph's SELL-32 copy (hubs as chunks of their rows), as
        // the batched rounds do
        k_ms_round_sell<T><<<S->own.num_sms * 4, kMsSellWarps * 32,
                             kMsSellWarps * sizeof(MsSellWarpSmem<T>), st>>>(
            sell->colval, sell->nzval, sell->dtype, sell->perm, sell->m, sell->sellplan->pitems,
            sell->sellplan->npitems, D, E.c0, E.c1, E.d_cnt, E.d_amask, E.cq[cur ^ 1], ncq_nxt);
        return;
      }
    }
    // every non-hub vertex in the plan's order (long rows first, spread over the warps)
    k_ms_round<T><<<grid_s(S, n * 32), 256, 0, st>>>(n, sg.g, D, E.c0, E.c1, E.d_cnt, E.d_amask,
                                                      hp->order, hp->d_norder, E.cq[cur ^ 1],
                                                      ncq_nxt);
  }
  if (hp->npiece > 0)
    k_ms_round_hub<T><<<grid_s(S, hp->npiece * 32), 256, 0, st>>>(
        sg.g, hp->pieces, hp->npiece, hp->hubs, D, E.c0, E.c1, E.d_cnt, E.d_amask,
        restricted ? E.mark : nullptr, E.cq[cur ^ 1], ncq_nxt);
}

// one tick of an executor, enqueued on its stream, followed by its event
static int exec_tick(gg_server* S, int gi, Executor& E) {
  const SrvGraph& sg = S->views[gi];
  const int64_t n = sg.n;
  cudaStream_t st = E.ectx.stream;
  const HubPlan* hp = S->graphs[gi]->hubplan;
  ++E.tick;
  if (E.kind == GG_QUERY_BFS) {
    unsigned* ha = E.h_stage + 1008;  // act of this tick, then zeros for act_next
    for (int w = 0; w < kBfsW; ++w) {
      ha[w] = E.act_host[w];
      ha[kBfsW + w] = 0;
    }
    GG_CUDA(cudaMemcpyAsync(E.act, ha, 2 * kBfsW * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    GG_CUDA(cudaMemsetAsync(E.d_cnt, 0, 8, st));
    const LevelOutSlots out{E.outp, E.start, E.tick};
    k_ms_level<kBfsW, LevelOutSlots><<<grid_s(S, n), 256, 0, st>>>(
        n, sg.g, E.F, E.Fn, E.V, E.act, E.act + kBfsW, out, E.d_cnt);
    if (hp->nhub > 0) {
      k_ms_hub<kBfsW><<<grid_s(S, hp->npiece * 32), 256, 0, st>>>(sg.g, hp->pieces, hp->npiece,
                                                                  hp->hubs, E.F, E.V, E.act, E.hacc);
      k_ms_hub_final<kBfsW, LevelOutSlots><<<grid_s(S, hp->nhub), 256, 0, st>>>(
          hp->hubs, hp->nhub, E.hacc, E.Fn, E.V, E.act, E.act + kBfsW, out, E.d_cnt);
    }
    std::swap(E.F, E.Fn);
    GG_CUDA(cudaMemcpyAsync(E.h_result, E.act + kBfsW, kBfsW * 4, cudaMemcpyDeviceToHost, st));
  } else if (E.kind == GG_QUERY_SSSP) {
    GG_CUDA(cudaMemsetAsync(E.d_amask, 0, 4, st));  // dropped columns of this round
    GG_CUDA(cudaMemsetAsync(E.c1, 0, (size_t)n * sizeof(unsigned), st));
    const int64_t nnz = S->graphs[gi]->nnz;
    const gg_mat* sell = nullptr;  // built when the graph was added (sssp_prepare)
    GG_CHECK(pull_sell_copy(&S->own, S->graphs[gi], &sell));
    switch (E.dtype) {
      case GG_INT32: ss_round<int32_t>(S, E, sg, hp, nnz, sell); break;
      case GG_INT64: ss_round<int64_t>(S, E, sg, hp, nnz, nullptr); break;
      case GG_FLOAT32: ss_round<float>(S, E, sg, hp, nnz, sell); break;
      default: ss_round<double>(S, E, sg, hp, nnz, nullptr); break;
    }
    std::swap(E.c0, E.c1);
    GG_CUDA(cudaMemcpyAsync(E.h_result, E.d_amask, 4, cudaMemcpyDeviceToHost, st));
    // length of the changed queue of this round (h_result[2..3]) for the next decision
    GG_CUDA(cudaMemcpyAsync(E.h_result + 2, E.d_cnt + 1 + (E.cq_cur ^ 1), 8, cudaMemcpyDeviceToHost, st));
    E.cq_cur ^= 1;
  } else {
    // only the columns up to the highest busy slot are multiplied (free slots are
    // reused lowest first, so few queries cost few columns)
    int kact = 0;
    for (int q = 0; q < kColSlots; ++q)
      if (E.slots[q].busy) kact = q + 1;
    GG_CHECK(spmm_dispatch(&E.ectx, S->graphs[gi], GG_FLOAT32, GG_OP_MUL, GG_OP_ADD, GG_OP_SECOND,
                           E.Y, GG_FLOAT32, kColSlots, E.X, GG_FLOAT32, kColSlots, kact,
                           GG_ROW_MAJOR, nullptr, 0, 0, 0));
    std::swap(E.X, E.Y);
  }
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaEventRecord(E.ev, st));
  E.inflight = true;
  return GG_OK;
}

// after the tick's event: retire the slots that finished.  BFS results are complete
// already; the others get an output copy and finish when ev_out completes.
static int exec_retire(gg_server* S, int gi, Executor& E, std::vector<Request>& finished) {
  const int64_t n = S->views[gi].n;
  cudaStream_t st = E.ectx.stream;
  bool copies = false;
  if (E.kind == GG_QUERY_BFS)
    for (int w = 0; w < kBfsW; ++w) E.act_host[w] = E.h_result[w];
  if (E.kind == GG_QUERY_SSSP) {
    unsigned long long nq = 0;
    memcpy(&nq, E.h_result + 2, sizeof(nq));
    E.nchanged = (int64_t)nq;
  }
  for (int q = 0; q < (int)E.slots.size(); ++q) {
    Slot& sl = E.slots[q];
    if (!sl.busy) continue;
    bool done = false;
    if (E.kind == GG_QUERY_BFS) {
      done = !((E.h_result[q >> 5] >> (q & 31)) & 1u);  // no new vertex this level
      if (done) finished.push_back(sl.req);
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
      if (E.kind != GG_QUERY_BFS) {
        E.finishing.push_back(sl.req);
        copies = true;
      }
    }
  }
  if (copies) GG_CUDA(cudaEventRecord(E.ev_out, st));
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

static const int kSoloWorkers = 4;

// one request through the single-query engines (the plain per-query path); SpMV
// iterations use the one-column SpMM so that they fold exactly like an executor slot
static int solo_run(gg_server* S, int w, const Request& r) {
  gg_ctx* c = S->solo_ctx[w];
  gg_mat* A = S->graphs[r.graph];
  const int64_t n = A->m;
  const bool short_query = r.kind == GG_QUERY_BFS || n < (int64_t(1) << 20);
  c->stream = short_query ? S->solo_hi[w] : S->solo_lo[w];
  if (r.kind == GG_QUERY_BFS) {
    // bfs_distances: typemax(Int32) for every vertex the search does not reach
    int32_t* out = static_cast<int32_t*>(r.out);
    k_fill_levels<<<grid_s(S, n), 256, 0, c->stream>>>(out, n);
    GG_CUDA(cudaGetLastError());
    return gg_bfs_levels(c, A, r.source, out, n, nullptr);
  }
  if (r.kind == GG_QUERY_SSSP) {
    const int dt = A->dtype == GG_BOOL ? GG_INT32 : A->dtype;
    const int64_t src = r.source;
    return gg_sssp(c, A, &src, 1, r.out, nullptr, dt, n, nullptr);
  }
  float* tmp = nullptr;
  GG_CUDA(cudaMallocAsync((void**)&tmp, (size_t)n * sizeof(float), c->stream));
  float* out = static_cast<float*>(r.out);
  const float* src = r.x;
  float* dst = (r.steps % 2 == 1) ? out : tmp;  // the last step lands in out
  int rc = GG_OK;
  for (int st = 0; st < r.steps && rc == GG_OK; ++st) {
    rc = spmm_dispatch(c, A, GG_FLOAT32, GG_OP_MUL, GG_OP_ADD, GG_OP_SECOND, dst, GG_FLOAT32, 1,
                       src, GG_FLOAT32, 1, 1, GG_ROW_MAJOR, nullptr, 0, 0, 0);
    src = dst;
    dst = (dst == out) ? tmp : out;
  }
  cudaFreeAsync(tmp, c->stream);
  if (rc == GG_OK) GG_CUDA(cudaStreamSynchronize(c->stream));
  return rc;
}

static void solo_loop(gg_server* S, int w) {
  gg_ctx* c = S->solo_ctx[w];
  cudaSetDevice(c->device);
  for (;;) {
    gg_server::SoloJob job;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->solo_cv.wait(lk, [&] { return S->stop || !S->solo_q.empty(); });
      if (S->stop) return;
      job = S->solo_q.front();
      S->solo_q.pop_front();
    }
    const int rc = solo_run(S, w, job.req);
    const double t = now_s();
    std::string msg = rc ? gg_last_error() : "";
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->solo_finished.emplace_back(job.req.graph, job.req.kind - 1);
      ++S->solo_idle;
      if (rc != GG_OK) {
        S->error = rc;
        S->error_msg = msg;
        S->stop = true;
      } else {
        S->done_ids.push_back(job.req.id);
        S->done_lat.push_back(t - job.req.t_submit);
        --S->inflight;
        ++S->solo_runs;
      }
    }
    S->cv.notify_one();
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
        for (auto& E : per_g) busy |= E.ready && (E.active() > 0 || E.inflight || !E.finishing.empty());
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
      for (auto& f : S->solo_finished) S->solo_active[f.first][f.second] = 0;
      S->solo_finished.clear();
      // a lone request whose executor is idle runs on a solo worker (no batching
      // needed: the single-query engine is the fastest path for one query), when free
      // HBM covers its working set plus the reserve (admission by free memory)
      size_t fr = 0, tot = 0;
      bool mem_known = false;
      for (size_t gi = 0; gi < S->graphs.size() && S->solo_idle > 0; ++gi)
        for (int kk = 0; kk < 3 && S->solo_idle > 0; ++kk) {
          Executor& E = S->exec[gi][kk];
          const bool idle = !E.ready || (E.active() == 0 && !E.inflight && E.finishing.empty());
          if (waiting[gi][kk].size() == 1 && idle && !S->solo_active[gi][kk]) {
            if (!mem_known) {
              if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = 0;
              mem_known = true;
            }
            const size_t need = (size_t)S->views[gi].n * 24 + ((size_t)1 << 20);
            if (fr < need + (size_t)S->reserve) {
              ++S->admission_waits;
              continue;  // stays queued; the executor path checks memory the same way
            }
            fr -= need;
            gg_server::SoloJob job;
            job.req = waiting[gi][kk].front();
            waiting[gi][kk].clear();
            S->solo_active[gi][kk] = 1;
            --S->solo_idle;
            S->solo_q.push_back(job);
            S->solo_cv.notify_one();
          }
        }
    }
    int rc = GG_OK;
    bool progress = false;
    std::vector<Request> finished;
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
        if (!E.finishing.empty()) {
          const cudaError_t q = cudaEventQuery(E.ev_out);
          if (q == cudaSuccess) {
            finished.insert(finished.end(), E.finishing.begin(), E.finishing.end());
            E.finishing.clear();
            progress = true;
          } else if (q != cudaErrorNotReady) {
            rc = cuda_error(q, "server results");
            break;
          }
        }
        if (E.inflight) {
          const cudaError_t q = cudaEventQuery(E.ev);
          if (q == cudaErrorNotReady) continue;
          if (q != cudaSuccess) {
            rc = cuda_error(q, "server tick");
            break;
          }
          E.inflight = false;
          ++S->ticks;
          progress = true;
          rc = exec_retire(S, (int)gi, E, finished);
          if (rc) break;
        }
        if (exec_admit(S, (int)gi, E, waiting[gi][kk]) > 0) progress = true;
        if (E.active() > 0) {
          rc = exec_tick(S, (int)gi, E);
          progress = true;
        }
      }
    }
    if (!finished.empty() || rc != GG_OK) {
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
    if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
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
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  for (int w = 0; w < kSoloWorkers; ++w) {
    gg_ctx* c = nullptr;
    int rc = gg_init(ctx->device, &c);
    cudaStream_t hi = nullptr, lo = nullptr;
    if (rc == GG_OK &&
        (cudaStreamCreateWithPriority(&hi, cudaStreamNonBlocking, greatest) != cudaSuccess ||
         cudaStreamCreateWithPriority(&lo, cudaStreamNonBlocking, least) != cudaSuccess))
      rc = set_error(GG_ERR_CUDA, "solo worker stream");
    if (rc == GG_OK) rc = gg_set_stream(c, hi);
    if (rc != GG_OK) {
      if (c) gg_destroy(c);
      if (hi) cudaStreamDestroy(hi);
      if (lo) cudaStreamDestroy(lo);
      break;  // fewer solo workers; batching alone still serves every request
    }
    S->solo_ctx.push_back(c);
    S->solo_hi.push_back(hi);
    S->solo_lo.push_back(lo);
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
  GG_CHECK(graph_view(&S->own, A, &g.g.rowptr, &g.g.colval, &g.g.nz, &all_odd, &nonneg));
  g.g.tv = A->dtype;
  g.g.odd_only = !all_odd;
  g.nonneg = nonneg;
  g.n = A->m;
  // Build every per-matrix analysis the executors and the solo engines use now, so
  // that later concurrent calls on this matrix only read it.
  {
    const int64_t n = A->m;
    void* tmp = nullptr;
    GG_CUDA(cudaMalloc(&tmp, (size_t)(n > 0 ? n : 1) * 16));
    int rc = build_hub_plan(&S->own, A, g.g.rowptr, n);
    if (rc == GG_OK && nonneg) {
      const int32_t* pr = nullptr;
      const int32_t* pc = nullptr;
      rc = push_view(&S->own, A, &pr, &pc);
    }
    if (rc == GG_OK && !dtype_is_float(A->dtype) && n > 0)
      rc = gg_bfs_levels(&S->own, A, 1, static_cast<int32_t*>(tmp), n, nullptr);
    if (rc == GG_OK && nonneg && n > 0) {
      const int64_t one = 1;
      rc = sssp_prepare(&S->own, A);
      // the full rounds of the shortest-path executors run over the SELL-32 copy
      if (rc == GG_OK)
        rc = sell_round_attr<int32_t>();
      if (rc == GG_OK)
        rc = sell_round_attr<float>();
      if (rc == GG_OK)
        rc = gg_sssp(&S->own, A, &one, 1, tmp, nullptr, A->dtype == GG_BOOL ? GG_INT32 : A->dtype,
                     n, nullptr);
    }
    // every solo worker's scratch arena grows to this graph's needs now, not during
    // serving (growing it frees and allocates, which waits for the whole device)
    for (size_t w = 0; rc == GG_OK && w < S->solo_ctx.size() && n > 0; ++w) {
      gg_ctx* c = S->solo_ctx[w];
      if (!dtype_is_float(A->dtype))
        rc = gg_bfs_levels(c, A, 1, static_cast<int32_t*>(tmp), n, nullptr);
      if (rc == GG_OK && nonneg) {
        const int64_t one = 1;
        rc = gg_sssp(c, A, &one, 1, tmp, nullptr, A->dtype == GG_BOOL ? GG_INT32 : A->dtype, n,
                     nullptr);
      }
      if (rc == GG_OK && A->dtype == GG_FLOAT32) {  // one step of a served SpMV iteration
        float* xb = static_cast<float*>(tmp);
        cudaMemsetAsync(xb, 0, (size_t)n * 4, c->stream);
        rc = spmm_dispatch(c, A, GG_FLOAT32, GG_OP_MUL, GG_OP_ADD, GG_OP_SECOND, xb + n,
                           GG_FLOAT32, 1, xb, GG_FLOAT32, 1, 1, GG_ROW_MAJOR, nullptr, 0, 0, 0);
      }
      if (rc == GG_OK) rc = gg_stream_sync(c);
    }
    if (rc == GG_OK && A->dtype == GG_FLOAT32 && n > 0) {
      float* xb = static_cast<float*>(tmp);
      cudaMemsetAsync(xb, 0, (size_t)n * 4, S->stream);
      rc = spmm_dispatch(&S->own, A, GG_FLOAT32, GG_OP_MUL, GG_OP_ADD, GG_OP_SECOND, xb + n,
                         GG_FLOAT32, 1, xb, GG_FLOAT32, 1, 1, GG_ROW_MAJOR, nullptr, 0, 0, 0);
    }
    cudaStreamSynchronize(S->stream);
    cudaFree(tmp);
    if (rc != GG_OK) return rc;
  }
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
    if (kind == GG_QUERY_BFS && dtype_is_float(g.g.tv))
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
    if (!S->worker.joinable()) {
      S->solo_active.assign(S->graphs.size(), std::vector<char>(3, 0));
      for (int w = 0; w < (int)S->solo_ctx.size(); ++w) S->solo_threads.emplace_back(solo_loop, S, w);
      S->solo_idle = (int)S->solo_ctx.size();
      S->worker = std::thread(server_loop, S);
    }
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
  S->solo_cv.notify_all();
  if (S->worker.joinable()) S->worker.join();
  for (auto& t : S->solo_threads)
    if (t.joinable()) t.join();
  for (size_t w = 0; w < S->solo_ctx.size(); ++w) {
    gg_destroy(S->solo_ctx[w]);
    cudaStreamDestroy(S->solo_hi[w]);
    cudaStreamDestroy(S->solo_lo[w]);
  }
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
