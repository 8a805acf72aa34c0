// gg_noalloc.cu -- BFS levels without any device allocation.
//
// Some callers cannot allocate GPU memory: code that runs inside another runtime's
// memory pool or arena (a host application that hands this library fixed buffers
// and forbids cudaMalloc, for example one whose allocator reserves the whole device
// up front), or code that must not take the allocator's implicit device-wide
// synchronisation in the middle of its work.  gg_bfs_levels_noalloc serves them: it
// takes the CSR arrays of A_T and the output vector as plain device pointers and
// keeps its working state (visited bitmap, two frontier bitmaps, one counter) in a
// fixed array compiled into the library.
//
// The fixed array holds 3 bitmaps of kNoAllocMaxN bits (1.5 MiB).  Every GPU that
// loads the library keeps it until the process exits.  Graphs with more vertices are
// rejected.  The search is bottom-up only (every level scans the unvisited
// vertices' in-edges), so it needs neither the transposed graph nor any analysis,
// and costs O(levels * (n + nnz)) work.
#include "gg_common.cuh"

namespace gg {

static const int64_t kNoAllocMaxN = 4194304;  // 2^22 vertices
static const int64_t kNoAllocWords = kNoAllocMaxN / 32;

// [visited | frontier A | frontier B] bitmaps, then the level counter
static __device__ __align__(256) unsigned g_noalloc_scratch[3 * kNoAllocWords + 64];

// Device address of g_noalloc_scratch on the current device.  The symbol's name in
// host code is only a stand-in, never a device address, so it is looked up through
// the runtime -- on every call, with the caller's device current: the lookup
// allocates nothing, and a cached address would go stale once cudaDeviceReset has
// unloaded the module (it may load elsewhere afterwards).
static int noalloc_scratch(unsigned** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  *out = static_cast<unsigned*>(p);
  return GG_OK;
}

__device__ __forceinline__ bool na_odd(const void* nz, int tv, int64_t k) {
  if (!nz) return true;
  switch (tv) {
    case GG_BOOL: return static_cast<const uint8_t*>(nz)[k] & 1;
    case GG_INT32: return static_cast<const int32_t*>(nz)[k] & 1;
    case GG_INT64: return static_cast<const int64_t*>(nz)[k] & 1;
  }
  return false;
}

__global__ void k_na_seed(int32_t s, unsigned* visited, unsigned* frontier, int32_t* dist) {
  visited[s >> 5] = 1u << (s & 31);
  frontier[s >> 5] = 1u << (s & 31);
  dist[s] = 0;
}

// one bottom-up level: an unvisited vertex joins when an in-neighbour (row of A_T)
// is in the frontier over an edge with an odd stored value (band semiring)
__global__ void __launch_bounds__(256)
    k_na_pull(int64_t n, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
              const void* nz, int tv, const unsigned* __restrict__ fb, unsigned* visited,
              unsigned* fbn, int32_t* dist, int32_t level, unsigned* count) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t v = base + threadIdx.x;
    bool found = false;
    const unsigned vw = v < n ? visited[v >> 5] : ~0u;
    if (v < n && !((vw >> (v & 31)) & 1u)) {
      for (int64_t k = (int64_t)rowptr[v] - 1; k < (int64_t)rowptr[v + 1] - 1; ++k) {
        const int32_t u = colval[k] - 1;
        if ((uint64_t)(uint32_t)u >= (uint64_t)n) continue;  // never read past the bitmaps
        if (((fb[u >> 5] >> (u & 31)) & 1u) && na_odd(nz, tv, k)) {
          found = true;
          break;
        }
      }
    }
    if (found) dist[v] = level;
    const unsigned bal = __ballot_sync(0xffffffffu, found);
    if (lane == 0 && bal) {
      visited[v >> 5] = vw | bal;  // the warp's 32 vertices share this word
      fbn[v >> 5] = bal;
      atomicAdd(count, (unsigned)__popc(bal));
    }
  }
}

}  // namespace gg

using namespace gg;

extern "C" int gg_bfs_levels_noalloc(const int32_t* rowptr, const int32_t* colval,
                                     const void* nzval, int dtype, int64_t n, int64_t nnz,
                                     int64_t source, int32_t* dist, void* stream,
                                     int64_t* levels_out) {
  if (n < 0 || nnz < 0) return set_error(GG_ERR_ARGUMENT, "negative size");
  if (n > kNoAllocMaxN)
    return set_error(GG_ERR_ARGUMENT,
                     "gg_bfs_levels_noalloc: %lld vertices exceed the fixed scratch capacity of "
                     "%lld vertices", (long long)n, (long long)kNoAllocMaxN);
  if (!rowptr || !dist || (nnz > 0 && !colval)) return set_error(GG_ERR_ARGUMENT, "NULL array");
  if (nzval && (dtype < GG_BOOL || dtype > GG_INT64))
    return set_error(GG_ERR_UNSUPPORTED, "GPUGraphs_band needs Bool or integer values");
  if (source < 1 || source > n)
    return set_error(GG_ERR_BOUNDS, "source %lld out of 1:%lld", (long long)source, (long long)n);
  int dev = 0;
  GG_CUDA(cudaGetDevice(&dev));
  unsigned* base = nullptr;
  GG_CHECK(noalloc_scratch(&base));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int num_sms = 0;
  GG_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t nw = (n + 31) / 32;
  unsigned* visited = base;
  unsigned* fb = base + kNoAllocWords;
  unsigned* fbn = base + 2 * kNoAllocWords;
  unsigned* count = base + 3 * kNoAllocWords;
  // the array keeps the previous call's contents: clear what must start at zero
  GG_CUDA(cudaMemsetAsync(visited, 0, nw * sizeof(unsigned), st));
  GG_CUDA(cudaMemsetAsync(fb, 0, nw * sizeof(unsigned), st));
  k_na_seed<<<1, 1, 0, st>>>((int32_t)(source - 1), visited, fb, dist);
  GG_CUDA(cudaGetLastError());
  int64_t g = (n + 255) / 256;
  if (g > (int64_t)num_sms * 8) g = (int64_t)num_sms * 8;
  if (g < 1) g = 1;
  unsigned found = 0;
  int32_t level = 0;
  for (;;) {
    ++level;
    GG_CUDA(cudaMemsetAsync(fbn, 0, nw * sizeof(unsigned), st));
    GG_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned), st));
    k_na_pull<<<(int)g, 256, 0, st>>>(n, rowptr, colval, nzval, dtype, fb, visited, fbn, dist,
                                      level, count);
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(&found, count, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    if (found == 0) break;
    unsigned* t = fb;
    fb = fbn;
    fbn = t;
  }
  if (levels_out) *levels_out = level;
  return GG_OK;
}
