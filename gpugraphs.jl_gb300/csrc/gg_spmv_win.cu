// gg_spmv_win.cu -- plus-times Float32 SpMV of a large CSR over column-window tiles.
//
// Why: on a power-law graph most entries of x are gathered by a minority of rows,
// and a warp's 32 scattered 4-byte gathers are 32 separate 32-byte requests to L2;
// the SELL kernel (k_sell_hot32) is bound by that request rate, not by HBM.  Here
// the rows, sorted by length, are cut into tiles, and every tile's entries are
// grouped by rank window (columns relabelled by decreasing frequency): for a window
// with enough of the tile's entries, the CTA copies the window's kWinCols x values
// (64 KB) into shared memory with one bulk copy and serves the window's gathers from
// there; the rarely gathered rest (tail segments) is read from global memory.  How
// many windows a tile stages is chosen per tile when the layout is built, from the
// tile's histogram of entries per window.
//
// Kernel (k_spmv_win): one 1024-thread CTA per SM walks its list of work units
// (segment ranges of one tile).  Every warp owns a fixed set of the tile's row pieces
// and streams its own entries of each segment: 128 entries per step (each lane loads
// 4 consecutive words and values with 16-byte loads; every warp's share of a segment
// is padded to a multiple of 4 with entries of a dump slot), products, a fold of the
// lane's own runs of equal piece, and a segmented warp scan over the lanes' last runs
// (one lane-private running sum while a whole step belongs to one piece) into a
// shared-memory accumulator per piece.  Warps never wait for one another inside a
// unit: the two 64 KB window buffers are handed over by mbarriers (the copy of window
// j completes on full[j % 2]) and an arrival counter (the last warp to leave window j
// issues the copy of window j + 2 into the same buffer).  At the end of a unit the
// pieces of every row are added in piece order, so every sum is formed in one fixed
// order and repeated calls give identical results.  Every wait on a copy is bounded
// (the context's poll limit, by default kWinPolls; then the error flag, a drain of the
// copies in flight bounded by kWinPolls whatever the limit, and an orderly return).  Sums differ from the storage-order fold by rounding only.
#include <algorithm>
#include <numeric>
#include <queue>
#include <vector>

#include "gg_semiring.cuh"
#include "gg_tma.cuh"

namespace gg {

static const int kWinThreads = 1024;
static const int kWinWarps = kWinThreads / 32;
static const uint32_t kWinColMask = (1u << kWinShift) - 1;
static const unsigned kWinPolls = 1u << 22;
static const int kMaxWinPerTile = 2048;
static const int kWinDump = kWinRows - 1;  // accumulator slot of the padding entries
// smem: two windows | accumulators | counters, flag, copies issued | 2 mbarriers
static const size_t kWinSmem = (size_t)2 * kWinCols * 4 + (size_t)kWinRows * 4 + 32 + 16;

__device__ __forceinline__ bool win_wait(uint32_t bar, uint32_t parity, unsigned limit = kWinPolls) {
  for (unsigned p = 0; p < limit; ++p)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

struct WinRun {
  int row = -1;      // piece of the lane-private run (same in every lane), -1 = none
  float sum = 0.0f;  // this lane's part of the run
};

__device__ __forceinline__ void win_flush(float* acc, WinRun& st, int lane) {
  if (st.row < 0) return;
  float t = st.sum;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, o));
  if (lane == 0) acc[st.row] = __fadd_rn(acc[st.row], t);
  __syncwarp();
  st.row = -1;
  st.sum = 0.0f;
}

// One step of 128 entries: lane l holds entries 4l..4l+3 (pieces r[], products p[];
// r = -1 past the segment), sorted by piece.  Each lane folds its own runs: a run
// strictly inside the lane is a whole piece of this step (added at once); the lane's
// first run joins the previous lane's last run when the piece continues; the lanes'
// last runs are combined by a segmented scan over the lanes and added by the lane
// that ends each piece.
__device__ __forceinline__ void win_step4(float* acc, WinRun& st, int lane, const int (&r)[4],
                                          const float (&p)[4]) {
  const bool b1 = r[1] != r[0], b2 = r[2] != r[1], b3 = r[3] != r[2];
  const bool multi = b1 || b2 || b3;
  const int R = __shfl_sync(0xffffffffu, r[0], 0);
  if (__all_sync(0xffffffffu, !multi && r[0] == R && R >= 0)) {
    // the whole step is one piece: extend the lane-private run
    if (R != st.row) {
      win_flush(acc, st, lane);
      st.row = R;
    }
    st.sum = __fadd_rn(st.sum, __fadd_rn(__fadd_rn(__fadd_rn(p[0], p[1]), p[2]), p[3]));
    return;
  }
  win_flush(acc, st, lane);
  float A, B;  // first run (piece r[0]) and last run (piece r[3]) of the lane
  if (!multi) {
    A = __fadd_rn(__fadd_rn(__fadd_rn(p[0], p[1]), p[2]), p[3]);
    B = A;
  } else {
    A = p[0];
    if (!b1) {
      A = __fadd_rn(A, p[1]);
      if (!b2) A = __fadd_rn(A, p[2]);
    }
    if (b3) B = p[3];
    else if (b2) B = __fadd_rn(p[2], p[3]);
    else B = __fadd_rn(__fadd_rn(p[1], p[2]), p[3]);
    // whole pieces strictly inside the lane
    if (b1 && b2 && r[1] >= 0) acc[r[1]] = __fadd_rn(acc[r[1]], p[1]);
    if (b1 && !b2 && b3 && r[1] >= 0) acc[r[1]] = __fadd_rn(acc[r[1]], __fadd_rn(p[1], p[2]));
    if (b2 && b3 && r[2] >= 0) acc[r[2]] = __fadd_rn(acc[r[2]], p[2]);
  }
  const int kprev = __shfl_up_sync(0xffffffffu, r[3], 1);
  // first run of a multi-run lane: handed to the previous lane when its piece goes on
  // there, else added here
  const bool give = multi && lane > 0 && kprev == r[0];
  if (multi && !give && r[0] >= 0) acc[r[0]] = __fadd_rn(acc[r[0]], A);
  const float gA = __shfl_down_sync(0xffffffffu, A, 1);
  const unsigned gives = __ballot_sync(0xffffffffu, give);
  float v = B;
  if (lane < 31 && ((gives >> (lane + 1)) & 1u)) v = __fadd_rn(v, gA);
  // segmented scan of the last runs over the lanes (key r[3])
  const bool head = lane == 0 || kprev != r[3];
  const unsigned heads = __ballot_sync(0xffffffffu, head);
  const int s0 = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
  for (int k = 1; k < 32; k <<= 1) {
    const float t = __shfl_up_sync(0xffffffffu, v, k);
    if (lane - k >= s0) v = __fadd_rn(v, t);
  }
  const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
  if (tail && r[3] >= 0) acc[r[3]] = __fadd_rn(acc[r[3]], v);
  __syncwarp();
}

// one warp's entries [p0, p1) of a window (both multiples of 4); xw = the window's x
// values in shared memory
__device__ __forceinline__ void win_part(const uint32_t* __restrict__ idx,
                                         const float* __restrict__ val, const float* xw,
                                         float* acc, int lane, int32_t p0, int32_t p1,
                                         uint64_t pol_s) {
  WinRun st;
  const int32_t q1 = p1 >> 2;
  const int32_t* id = reinterpret_cast<const int32_t*>(idx);
  int4 e = make_int4(0, 0, 0, 0), en;
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f), an;
  {
    const int32_t q = (p0 >> 2) + lane;
    if (q < q1) {
      e = ld_stream4_p(id + 4 * q, pol_s);
      a = ld_stream4_p(val + 4 * q, pol_s);
    }
  }
  for (int32_t qb = p0 >> 2; qb < q1; qb += 32) {
    const int32_t qn = qb + 32 + lane;
    en = make_int4(0, 0, 0, 0);
    an = make_float4(0.f, 0.f, 0.f, 0.f);
    if (qn < q1) {
      en = ld_stream4_p(id + 4 * qn, pol_s);
      an = ld_stream4_p(val + 4 * qn, pol_s);
    }
    const bool live = qb + lane < q1;
    const uint32_t w[4] = {(uint32_t)e.x, (uint32_t)e.y, (uint32_t)e.z, (uint32_t)e.w};
    const float av[4] = {a.x, a.y, a.z, a.w};
    int r[4];
    float p[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      p[u] = __fmul_rn(av[u], live ? xw[w[u] & kWinColMask] : 0.0f);
      r[u] = live ? (int)(w[u] >> kWinShift) : -1;
    }
    win_step4(acc, st, lane, r, p);
    e = en;
    a = an;
  }
  win_flush(acc, st, lane);
}

__global__ void __launch_bounds__(kWinThreads, 1)
    k_spmv_win(const uint32_t* __restrict__ idx, const float* __restrict__ val,
               const float* __restrict__ xr, float* __restrict__ y,
               const int32_t* __restrict__ rowperm, const WinTile* __restrict__ tiles,
               const int32_t* __restrict__ segbase, const int32_t* __restrict__ wseg,
               const int32_t* __restrict__ vptr, const int4* __restrict__ units,
               const int32_t* __restrict__ cta_ptr, const int32_t* __restrict__ cta_wptr,
               const int32_t* __restrict__ cta_win, const float* __restrict__ yt,
               float* __restrict__ partials, unsigned* err, unsigned polls) {
  extern __shared__ __align__(128) unsigned char smem[];
  float* sw = reinterpret_cast<float*>(smem);
  float* acc = sw + 2 * kWinCols;
  // scnt[0..1] arrivals per buffer, [2] abort, [3..4] copies issued per buffer
  volatile int* scnt = reinterpret_cast<volatile int*>(acc + kWinRows);
  uint64_t* sbar = reinterpret_cast<uint64_t*>(acc + kWinRows + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bar0 = smem_u32(sbar);
  const int32_t* wins = cta_win + cta_wptr[blockIdx.x];
  const int nwin = cta_wptr[blockIdx.x + 1] - cta_wptr[blockIdx.x];
  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    for (int i = 0; i < 8; ++i) scnt[i] = 0;
  }
  fence_mbar_init();
  fence_proxy_async();
  __syncthreads();
  if (tid == 0) {
    for (int j = 0; j < 2 && j < nwin; ++j) {
      mbar_expect_tx(bar0 + 8 * j, kWinCols * 4);
      bulk_g2s(smem_u32(sw + j * kWinCols), xr + wins[j], kWinCols * 4, bar0 + 8 * j);
      scnt[3 + j] = 1;
    }
  }
  const uint64_t pol_s = l2_evict_first();
  int j = 0;  // windows passed by this warp (the same sequence in every warp)
  const int uend = cta_ptr[blockIdx.x + 1];
  for (int ui = cta_ptr[blockIdx.x]; ui < uend; ++ui) {
    const int4 U = units[ui];  // (tile, first segment, end segment, slot)
    const WinTile T = tiles[U.x];
    for (int i = tid; i < T.nv; i += kWinThreads) acc[i] = 0.0f;
    __syncthreads();
    const int32_t* ws = wseg + T.wbase + warp * (T.nseg + 1);
    for (int s = U.y; s < U.z; ++s) {  // every segment is a staged window
      const int32_t p0 = ws[s], p1 = ws[s + 1];
      {
        const int b = j & 1;
        const bool ok = scnt[2] == 0 && win_wait(bar0 + 8 * b, (uint32_t)((j >> 1) & 1), polls);
        if (!ok) {
          if (lane == 0) {
            scnt[2] = 1;
            if (err) atomicExch(err, 1u);
          }
        } else if (p0 < p1) {
          win_part(idx, val, sw + b * kWinCols, acc, lane, p0, p1, pol_s);
        }
        // leave window j; the last warp out refills the buffer with window j + 2
        __syncwarp();
        if (lane == 0) {
          __threadfence_block();
          if (atomicAdd((int*)scnt + b, 1) == kWinWarps - 1) {
            __threadfence_block();
            scnt[b] = 0;
            if (j + 2 < nwin && ok) {
              fence_proxy_async();
              mbar_expect_tx(bar0 + 8 * b, kWinCols * 4);
              bulk_g2s(smem_u32(sw + b * kWinCols), xr + wins[j + 2], kWinCols * 4, bar0 + 8 * b);
              scnt[3 + b] += 1;
            }
          }
        }
        __syncwarp();
        ++j;
      }
    }
    __syncthreads();
    if (scnt[2]) break;
    const int32_t* vp = vptr + T.vbase;
    float* out = U.w >= 0 ? partials + (int64_t)U.w * kWinRows : nullptr;
    for (int i = tid; i < T.rows; i += kWinThreads) {
      const int32_t v0 = vp[i], v1 = vp[i + 1];
      float s = acc[v0];
      for (int v = v0 + 1; v < v1; ++v) s = __fadd_rn(s, acc[v]);
      if (out) out[i] = s;
      else __stcs(y + __ldg(rowperm + T.row0 + i), __fadd_rn(s, yt[T.row0 + i]));
    }
    __syncthreads();
  }
  if (tid == 0 && scnt[2]) {
    // let the copies still in flight land before the CTA's shared memory goes away
    for (int b = 0; b < 2; ++b)
      if (scnt[3 + b] > 0) win_wait(bar0 + 8 * b, (uint32_t)((scnt[3 + b] - 1) & 1));
  }
}

// rows of split tiles: y = the unit partials added in unit order, then the tail sum
__global__ void k_win_combine(const int4* __restrict__ split, int64_t nsplit,
                              const int32_t* __restrict__ rowperm, const WinTile* __restrict__ tiles,
                              const float* __restrict__ partials, const float* __restrict__ yt,
                              float* __restrict__ y) {
  const int64_t total = nsplit * kWinRows;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int4 sp = split[k / kWinRows];
    const int i = (int)(k % kWinRows);
    if (i >= sp.w) continue;
    const float* p = partials + (int64_t)sp.y * kWinRows + i;
    float s = p[0];
    for (int u = 1; u < sp.z; ++u) s = __fadd_rn(s, p[(int64_t)u * kWinRows]);
    const int32_t r = tiles[sp.x].row0 + i;
    y[rowperm[r]] = __fadd_rn(s, yt[r]);
  }
}

__global__ void k_win_gather_x(const float* __restrict__ x, const int32_t* __restrict__ inv,
                               int64_t n, float* __restrict__ xr) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    xr[i] = __ldg(x + inv[i]);
}

// ---------------------------------------------------------------------------------
// layout build
// ---------------------------------------------------------------------------------
__global__ void k_win_colcount(const int32_t* __restrict__ colval, int64_t nnz, int32_t* cnt) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + (colval[k] - 1), 1);
}

// entries of every sorted row inside the first window (warp per row)
__global__ void k_win_w0(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
                         const int32_t* __restrict__ rowperm, const int32_t* __restrict__ rank,
                         int64_t m, int32_t* w0) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t row = rowperm[r];
    const int32_t k0 = rowptr[row] - 1, k1 = rowptr[row + 1] - 1;
    int c = 0;
    for (int32_t k = k0 + lane; k < k1; k += 32) c += rank[colval[k] - 1] < kWinCols;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) w0[r] = c;
  }
}

// per tile: entries per rank window (CTA per tile; warp per row, round robin)
__global__ void k_win_hist(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
                           const int32_t* __restrict__ rowperm, const int32_t* __restrict__ rank,
                           const int32_t* __restrict__ trow, int nbins, int32_t* hist) {
  extern __shared__ int32_t sh[];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int64_t t = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int64_t r = trow[t] + warp; r < trow[t + 1]; r += nw) {
    const int32_t row = rowperm[r];
    const int32_t k0 = rowptr[row] - 1, k1 = rowptr[row + 1] - 1;
    for (int32_t k = k0 + lane; k < k1; k += 32) atomicAdd(sh + rank[colval[k] - 1] / kWinCols, 1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) hist[t * nbins + i] = sh[i];
}

// tail entries (rank >= thr[r]) of every sorted row: count, then copy in column
// order as a CSR with 1-based rank labels (warp per row)
__global__ void k_win_tail(int pass, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ colval, const float* __restrict__ nzval,
                           const int32_t* __restrict__ rowperm, const int32_t* __restrict__ rank,
                           const int32_t* __restrict__ thr, int64_t m, int32_t* tptr,
                           int32_t* tcol, float* tval) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t row = rowperm[r];
    const int32_t k0 = rowptr[row] - 1, k1 = rowptr[row + 1] - 1;
    const int32_t t = thr[r];
    int32_t pos = pass == 0 ? 0 : tptr[r] - 1;
    for (int32_t kb = k0; kb < k1; kb += 32) {
      const int32_t k = kb + lane;
      int32_t c = 0;
      bool take = false;
      if (k < k1) {
        c = rank[colval[k] - 1];
        take = c >= t;
      }
      const unsigned b = __ballot_sync(0xffffffffu, take);
      if (pass == 1 && take) {
        const int32_t q = pos + __popc(b & ((1u << lane) - 1));
        tcol[q] = c + 1;
        tval[q] = nzval[k];
      }
      pos += __popc(b);
    }
    if (pass == 0 && lane == 0) tptr[r] = pos;
  }
}

// Pieces: piece p is entries [pf0[p], pf1[p]) (0-based positions in colval) of one
// row, with accumulator slot pv[p] inside its tile.  The pieces of warp q of tile t are
// pl[plp[t * 32 + q] .. plp[t * 32 + q + 1]), in increasing slot order.
// k_win_place (one warp per (tile, warp q)): pass 0 counts q's window entries per
// window into wseg; pass 1 scatters them from the offsets then in wseg, stable in
// (piece, column) order (ties inside a step ranked by lane).
__global__ void k_win_place(int pass, const int32_t* __restrict__ colval,
                            const float* __restrict__ nzval, const int32_t* __restrict__ rank,
                            const int32_t* __restrict__ pf0, const int32_t* __restrict__ pf1,
                            const int32_t* __restrict__ pv, const int32_t* __restrict__ pl,
                            const int32_t* __restrict__ plp, const WinTile* __restrict__ tiles,
                            const int32_t* __restrict__ tile_w, const int32_t* __restrict__ segbase,
                            int32_t* wseg, uint32_t* idx, float* val) {
  extern __shared__ int32_t cur[];  // [nseg]
  const int64_t t = blockIdx.x >> 5;
  const int q = blockIdx.x & 31, lane = threadIdx.x;
  const WinTile T = tiles[t];
  const int nw = tile_w[t];
  int32_t* wq = wseg + T.wbase + q * (T.nseg + 1);
  for (int s = lane; s < T.nseg; s += 32) cur[s] = pass == 0 ? 0 : wq[s];
  __syncwarp();
  for (int32_t li = plp[t * 32 + q]; li < plp[t * 32 + q + 1]; ++li) {
    const int32_t p = pl[li];
    const uint32_t slot = (uint32_t)pv[p] << kWinShift;
    const int32_t k1 = pf1[p];
    for (int32_t kb = pf0[p]; kb < k1; kb += 32) {
      const int32_t k = kb + lane;
      const bool in = k < k1;
      int ls = -1;
      int32_t c = 0;
      if (in) {
        c = rank[colval[k] - 1];
        ls = c / kWinCols < nw ? c / kWinCols : -1;  // -1: a tail entry
      }
      if (pass == 0) {
        if (ls >= 0) atomicAdd(cur + ls, 1);
        continue;
      }
      const unsigned peers = __match_any_sync(0xffffffffu, ls);
      const int before = __popc(peers & ((1u << lane) - 1));
      if (ls >= 0) {
        const int32_t pos = cur[ls] + before;
        idx[pos] = slot | (uint32_t)(c - (segbase[T.seg0 + ls] & ~kSegWindow));
        val[pos] = nzval[k];
      }
      __syncwarp();
      if (ls >= 0 && before == 0) cur[ls] += __popc(peers);
      __syncwarp();
    }
  }
  __syncwarp();
  if (pass == 0) {
    for (int s = lane; s < T.nseg; s += 32) wq[s] = cur[s];
    return;
  }
  // pad every segment's share to a multiple of 4 entries: a dump slot, value 0
  for (int s = 0; s < T.nseg; ++s)
    for (int32_t pos = cur[s] + lane; pos < wq[s + 1]; pos += 32) {
      idx[pos] = (uint32_t)kWinDump << kWinShift;
      val[pos] = 0.0f;
    }
}

void free_win_plan(gg_mat* A) {
  WinPlan* P = A->winplan;
  if (!P) return;
  void* bufs[] = {P->rowperm, P->inv,  P->xr,   P->idx,   P->val,     P->tiles,
                  P->segbase, P->wseg, P->vptr, P->units, P->cta_ptr, P->cta_wptr,
                  P->cta_win, P->split, P->partials, P->yt};
  for (void* b : bufs) cudaFree(b);
  if (P->tail) gg_mat_destroy(P->tail);
  delete P;
  A->winplan = nullptr;
}

namespace {
struct DevBufs {
  std::vector<void*> p;
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
};
template <class T>
cudaError_t upload(gg_ctx* ctx, T** dst, const std::vector<T>& src) {
  cudaError_t e = cudaMalloc((void**)dst, (src.empty() ? 1 : src.size()) * sizeof(T));
  if (e == cudaSuccess && !src.empty())
    e = cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice,
                        ctx->stream);
  return e;
}
template <class T>
cudaError_t upload_tmp(gg_ctx* ctx, DevBufs& tmp, T** dst, const std::vector<T>& src) {
  cudaError_t e = upload(ctx, dst, src);
  if (*dst) tmp.p.push_back(*dst);
  return e;
}
std::vector<int32_t> by_count_desc(const std::vector<int32_t>& v, int32_t maxv) {
  std::vector<int64_t> start((size_t)maxv + 2, 0);
  for (size_t i = 0; i < v.size(); ++i) start[(size_t)(maxv - v[i]) + 1]++;
  for (size_t k = 1; k < start.size(); ++k) start[k] += start[k - 1];
  std::vector<int32_t> order(v.size());
  for (size_t i = 0; i < v.size(); ++i) order[start[(size_t)(maxv - v[i])]++] = (int32_t)i;
  return order;
}
}  // namespace

// cost model, in units of one entry: staging a window (a 64 KB bulk copy from L2, and
// one pass of every warp over its share) costs about as much as this many gathers
static const int64_t kWinCost = 4096;

int build_win_plan(gg_ctx* ctx, gg_mat* A) {
  if (A->winplan) return GG_OK;
  WinPlan* P = new WinPlan();
  A->winplan = P;
  const int64_t m = A->m, n = A->n, nnz = A->nnz;
  if (A->format != GG_FMT_CSR || A->dtype != GG_FLOAT32) return GG_OK;
  if (m < (1 << 16) || n < (1 << 16) || nnz == 0) return GG_OK;
  if (nnz > (int64_t)INT32_MAX - 4096 || n > ((int64_t)1 << 27)) return GG_OK;
  const int64_t nbins = (n + kWinCols - 1) / kWinCols;
  const int grid = ctx->num_sms;
  DevBufs tmp;

  // rows by decreasing length, columns by decreasing frequency (stable counting sorts)
  std::vector<int32_t> rp(m + 1);
  GG_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr, (m + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  int32_t* dcnt = nullptr;
  GG_CUDA(cudaMalloc((void**)&dcnt, n * sizeof(int32_t)));
  tmp.p.push_back(dcnt);
  GG_CUDA(cudaMemsetAsync(dcnt, 0, n * sizeof(int32_t), ctx->stream));
  k_win_colcount<<<(int)std::max<int64_t>(1, std::min<int64_t>((nnz + 255) / 256, grid * 16)), 256, 0,
                   ctx->stream>>>(A->colval, nnz, dcnt);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> ccnt(n);
  GG_CUDA(cudaMemcpyAsync(ccnt.data(), dcnt, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> deg(m);
  int32_t maxdeg = 0, maxcnt = 0;
  for (int64_t i = 0; i < m; ++i) {
    deg[i] = rp[i + 1] - rp[i];
    maxdeg = std::max(maxdeg, deg[i]);
  }
  for (int64_t c = 0; c < n; ++c) maxcnt = std::max(maxcnt, ccnt[c]);
  std::vector<int32_t> inv = by_count_desc(ccnt, maxcnt);  // rank -> column
  {  // skew test: the 1% most frequent columns hold over a quarter of the entries
    int64_t top = 0;
    for (int64_t i = 0; i < n / 100; ++i) top += ccnt[inv[i]];
    if (top * 4 <= nnz) return GG_OK;
  }
  std::vector<int32_t> rowperm = by_count_desc(deg, maxdeg);  // position -> row
  std::vector<int32_t> rank(n);
  for (int64_t i = 0; i < n; ++i) rank[inv[i]] = (int32_t)i;

  int32_t *d_rowperm = nullptr, *d_inv = nullptr, *d_rank = nullptr, *d_w0 = nullptr;
  cudaError_t e = upload(ctx, &d_rowperm, rowperm);
  P->rowperm = d_rowperm;
  if (e == cudaSuccess) e = upload(ctx, &d_inv, inv);
  P->inv = d_inv;
  if (e == cudaSuccess) e = upload_tmp(ctx, tmp, &d_rank, rank);
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_w0, m * sizeof(int32_t));
  if (d_w0) tmp.p.push_back(d_w0);
  if (e != cudaSuccess) return cuda_error(e, "window tiles");
  k_win_w0<<<(int)std::max<int64_t>(1, std::min<int64_t>((m * 32 + 255) / 256, grid * 16)), 256, 0,
             ctx->stream>>>(A->rowptr, A->colval, d_rowperm, d_rank, m, d_w0);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> w0(m);
  GG_CUDA(cudaMemcpyAsync(w0.data(), d_w0, m * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));

  // tiles: up to kTileRows rows, fewer where the first window would exceed two units
  const int64_t ubudget = std::max<int64_t>(nnz / ((int64_t)grid * 8), 4096);
  std::vector<int32_t> trow(1, 0);
  {
    int64_t r = 0;
    while (r < m) {
      int64_t rows = 0, s0 = 0;
      while (r < m && rows < kTileRows && (rows == 0 || s0 + w0[r] <= 2 * ubudget)) {
        s0 += w0[r];
        ++r;
        ++rows;
      }
      trow.push_back((int32_t)r);
    }
  }
  const int64_t ntiles = (int64_t)trow.size() - 1;
  if (ntiles * nbins > ((int64_t)1 << 27)) return GG_OK;
  int32_t *d_trow = nullptr, *d_hist = nullptr;
  e = upload_tmp(ctx, tmp, &d_trow, trow);
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_hist, ntiles * nbins * sizeof(int32_t));
  if (d_hist) tmp.p.push_back(d_hist);
  if (e != cudaSuccess) return cuda_error(e, "window tiles");
  const size_t hsm = (size_t)nbins * sizeof(int32_t);
  if (hsm > 48 * 1024)
    GG_CUDA(cudaFuncSetAttribute(k_win_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm));
  k_win_hist<<<(int)ntiles, 512, hsm, ctx->stream>>>(A->rowptr, A->colval, d_rowperm, d_rank, d_trow,
                                                     (int)nbins, d_hist);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> hist(ntiles * nbins);
  GG_CUDA(cudaMemcpyAsync(hist.data(), d_hist, hist.size() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));

  // per tile: windows (cost model), segments, pieces, warp shares
  std::vector<WinTile> tiles(ntiles);
  std::vector<int32_t> tw(ntiles), segbase, vptr, pf0, pf1, pv, pl, plp(ntiles * 32 + 1, 0);
  int64_t nwin = 0, wwords = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    const int32_t* h = hist.data() + t * nbins;
    int64_t tot = 0;
    for (int64_t b = 0; b < nbins; ++b) tot += h[b];
    int64_t best = tot, bestw = 0, cum = 0;
    const int64_t wmax = std::min<int64_t>(nbins, kMaxWinPerTile);
    for (int64_t w = 1; w <= wmax; ++w) {
      cum += h[w - 1];
      const int64_t c = w * kWinCost + (tot - cum);
      if (c < best) {
        best = c;
        bestw = w;
      }
    }
    WinTile& T = tiles[t];
    T.row0 = trow[t];
    T.rows = trow[t + 1] - trow[t];
    T.seg0 = (int32_t)segbase.size();
    tw[t] = (int32_t)bestw;
    nwin += bestw;
    for (int64_t w = 0; w < bestw; ++w) segbase.push_back((int32_t)(w * kWinCols) | kSegWindow);
    T.nseg = (int32_t)segbase.size() - T.seg0;
    T.wbase = (int32_t)wwords;
    wwords += (int64_t)32 * (T.nseg + 1);
    // pieces: rows longer than about 1/1536 of the tile are cut
    const int64_t lmax = std::max<int64_t>(64, (tot + 1535) / 1536);
    T.vbase = (int32_t)vptr.size();
    const int32_t pbase = (int32_t)pf0.size();
    int32_t nv = 0;
    for (int64_t r = T.row0; r < T.row0 + T.rows; ++r) {
      vptr.push_back(nv);
      const int64_t d = deg[rowperm[r]];
      const int64_t np = std::max<int64_t>(1, (d + lmax - 1) / lmax);
      const int64_t len = (d + np - 1) / np;
      const int32_t k0 = rp[rowperm[r]] - 1;
      for (int64_t k = 0; k < np; ++k) {
        pf0.push_back(k0 + (int32_t)std::min<int64_t>(d, k * len));
        pf1.push_back(k0 + (int32_t)std::min<int64_t>(d, (k + 1) * len));
        pv.push_back(nv++);
      }
    }
    vptr.push_back(nv);
    T.nv = nv;
    if (nv > kWinRows) return set_error(GG_ERR_ASSERTION, "window tiles: %d pieces in a tile", nv);
    // longest-first assignment of the pieces to the 32 warps, each warp's list by slot
    std::vector<int32_t> ord(nv);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t x, int32_t y) {
      return pf1[pbase + x] - pf0[pbase + x] > pf1[pbase + y] - pf0[pbase + y];
    });
    int64_t load[32] = {0};
    std::vector<int32_t> owner(nv);
    for (int32_t v : ord) {
      int q = 0;
      for (int k = 1; k < 32; ++k)
        if (load[k] < load[q]) q = k;
      owner[v] = q;
      load[q] += pf1[pbase + v] - pf0[pbase + v];
    }
    std::vector<int32_t> wcount(32, 0);
    for (int32_t v = 0; v < nv; ++v) wcount[owner[v]]++;
    const size_t lbase = pl.size();
    pl.resize(lbase + nv);
    std::vector<size_t> wpos(32);
    size_t acc0 = lbase;
    for (int q = 0; q < 32; ++q) {
      plp[t * 32 + q] = (int32_t)acc0;
      wpos[q] = acc0;
      acc0 += wcount[q];
    }
    plp[t * 32 + 32] = (int32_t)acc0;
    for (int32_t v = 0; v < nv; ++v) pl[wpos[owner[v]]++] = pbase + v;
  }
  if (wwords > (int64_t)INT32_MAX) return GG_OK;

  // tail CSR: the entries of every row beyond its tile's staged windows
  {
    std::vector<int32_t> thr(m);
    for (int64_t t = 0; t < ntiles; ++t)
      for (int64_t r = trow[t]; r < trow[t + 1]; ++r) thr[r] = (int32_t)((int64_t)tw[t] * kWinCols);
    int32_t *d_thr = nullptr, *d_tptr = nullptr;
    e = upload_tmp(ctx, tmp, &d_thr, thr);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_tptr, (m + 1) * sizeof(int32_t));
    if (d_tptr) tmp.p.push_back(d_tptr);
    if (e != cudaSuccess) return cuda_error(e, "window tiles");
    const int tg = (int)std::max<int64_t>(1, std::min<int64_t>((m * 32 + 255) / 256, grid * 16));
    k_win_tail<<<tg, 256, 0, ctx->stream>>>(0, A->rowptr, A->colval, nullptr, d_rowperm, d_rank, d_thr,
                                            m, d_tptr, nullptr, nullptr);
    GG_CUDA(cudaGetLastError());
    std::vector<int32_t> tcnt(m), tptr(m + 1);
    GG_CUDA(cudaMemcpyAsync(tcnt.data(), d_tptr, m * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    tptr[0] = 1;
    for (int64_t r = 0; r < m; ++r) tptr[r + 1] = tptr[r] + tcnt[r];
    const int64_t tnnz = (int64_t)tptr[m] - 1;
    gg_mat* Tm = new gg_mat();
    Tm->format = GG_FMT_CSR;
    Tm->m = m;
    Tm->n = n;
    Tm->nnz = tnnz;
    Tm->dtype = GG_FLOAT32;
    Tm->device = ctx->device;
    Tm->tuned_spmv = 1;  // row blocks
    P->tail = Tm;
    e = upload(ctx, &Tm->rowptr, tptr);
    if (e == cudaSuccess) e = cudaMalloc((void**)&Tm->colval, (tnnz > 0 ? tnnz : 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&Tm->nzval, (tnnz > 0 ? tnnz : 1) * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&P->yt, m * sizeof(float));
    if (e != cudaSuccess) return cuda_error(e, "window tiles");
    k_win_tail<<<tg, 256, 0, ctx->stream>>>(1, A->rowptr, A->colval, static_cast<const float*>(A->nzval),
                                            d_rowperm, d_rank, d_thr, m, Tm->rowptr, Tm->colval,
                                            static_cast<float*>(Tm->nzval));
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  const int64_t nseg = (int64_t)segbase.size();

  // entry offsets: count per (tile, warp, segment), then place
  WinTile* d_tiles = nullptr;
  int32_t *d_tw = nullptr, *d_segbase = nullptr, *d_wseg = nullptr, *d_pf0 = nullptr, *d_pf1 = nullptr,
          *d_pv = nullptr, *d_pl = nullptr, *d_plp = nullptr;
  e = upload(ctx, &d_tiles, tiles);
  P->tiles = d_tiles;
  if (e == cudaSuccess) e = upload(ctx, &d_segbase, segbase);
  P->segbase = d_segbase;
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_wseg, wwords * sizeof(int32_t));
  P->wseg = d_wseg;
  if (e == cudaSuccess) e = upload(ctx, &P->vptr, vptr);
  if (e == cudaSuccess) e = upload_tmp(ctx, tmp, &d_tw, tw);
  if (e == cudaSuccess) e = upload_tmp(ctx, tmp, &d_pf0, pf0);
  if (e == cudaSuccess) e = upload_tmp(ctx, tmp, &d_pf1, pf1);
  if (e == cudaSuccess) e = upload_tmp(ctx, tmp, &d_pv, pv);
  if (e == cudaSuccess) e = upload_tmp(ctx, tmp, &d_pl, pl);
  if (e == cudaSuccess) e = upload_tmp(ctx, tmp, &d_plp, plp);
  if (e != cudaSuccess) return cuda_error(e, "window tiles");
  int maxnseg = 0;
  for (const WinTile& T : tiles) maxnseg = std::max(maxnseg, T.nseg);
  const size_t psm = (size_t)maxnseg * sizeof(int32_t);
  if (psm > 48 * 1024)
    GG_CUDA(cudaFuncSetAttribute(k_win_place, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm));
  k_win_place<<<(int)(ntiles * 32), 32, psm, ctx->stream>>>(
      0, A->colval, static_cast<const float*>(A->nzval), d_rank, d_pf0, d_pf1, d_pv, d_pl, d_plp,
      d_tiles, d_tw, d_segbase, d_wseg, P->idx, P->val);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> wseg(wwords);
  GG_CUDA(cudaMemcpyAsync(wseg.data(), d_wseg, wwords * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> segcost(nseg, 0);  // entries of each segment over all warps
  int64_t nstored = 0;                     // entries with every share padded to 4
  {
    int64_t real = 0;
    for (int64_t t = 0; t < ntiles; ++t) {
      const WinTile& T = tiles[t];
      for (int q = 0; q < 32; ++q) {
        int32_t* w = wseg.data() + T.wbase + q * (T.nseg + 1);
        for (int s = 0; s < T.nseg; ++s) {
          const int32_t c = w[s];
          segcost[T.seg0 + s] += c;
          real += c;
          w[s] = (int32_t)nstored;
          nstored += (c + 3) & ~3;
        }
        w[T.nseg] = (int32_t)nstored;
      }
    }
    if (real + P->tail->nnz != nnz)
      return set_error(GG_ERR_ASSERTION, "window tiles: %lld + %lld entries placed of %lld",
                       (long long)real, (long long)P->tail->nnz, (long long)nnz);
    if (nstored > (int64_t)INT32_MAX - 4096) return GG_OK;
  }
  e = cudaMalloc((void**)&P->idx, nstored * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->val, nstored * sizeof(float));
  if (e != cudaSuccess) return cuda_error(e, "window tiles");
  GG_CUDA(cudaMemcpyAsync(d_wseg, wseg.data(), wwords * sizeof(int32_t), cudaMemcpyHostToDevice,
                          ctx->stream));
  k_win_place<<<(int)(ntiles * 32), 32, psm, ctx->stream>>>(
      1, A->colval, static_cast<const float*>(A->nzval), d_rank, d_pf0, d_pf1, d_pv, d_pl, d_plp,
      d_tiles, d_tw, d_segbase, d_wseg, P->idx, P->val);
  GG_CUDA(cudaGetLastError());

  // work units: segment ranges of one tile, about total / (8 * grid) cost each
  for (int64_t s = 0; s < nseg; ++s)
    if (segbase[s] & kSegWindow) segcost[s] += kWinCost;
  const int64_t budget = std::max<int64_t>((nnz + nwin * kWinCost) / ((int64_t)grid * 8), 4096);
  std::vector<int4> units, split;
  std::vector<int64_t> ucost;
  int64_t nslots = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    const WinTile& T = tiles[t];
    const size_t first = units.size();
    int s0 = 0;
    int64_t cost = 0;
    for (int s = 0; s < T.nseg; ++s) {
      cost += segcost[T.seg0 + s];
      if (cost >= budget && s + 1 < T.nseg) {
        units.push_back(make_int4((int)t, s0, s + 1, -1));
        ucost.push_back(cost);
        s0 = s + 1;
        cost = 0;
      }
    }
    units.push_back(make_int4((int)t, s0, T.nseg, -1));
    ucost.push_back(cost + T.rows / 8);
    const size_t nu = units.size() - first;
    if (nu > 1) {
      split.push_back(make_int4((int)t, (int)nslots, (int)nu, T.rows));
      for (size_t k = first; k < units.size(); ++k) units[k].w = (int)nslots++;
    }
  }
  // longest-processing-time-first assignment to the CTAs
  std::vector<int64_t> order(units.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return ucost[x] > ucost[y]; });
  typedef std::pair<int64_t, int> Load;
  std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
  for (int b = 0; b < grid; ++b) heap.push(Load(0, b));
  std::vector<std::vector<int64_t>> per(grid);
  for (int64_t k : order) {
    Load l = heap.top();
    heap.pop();
    per[l.second].push_back(k);
    l.first += ucost[k];
    heap.push(l);
  }
  std::vector<int4> uord;
  std::vector<int32_t> cta_ptr(grid + 1, 0), cta_wptr(grid + 1, 0), cta_win;
  for (int b = 0; b < grid; ++b) {
    for (int64_t k : per[b]) {
      const int4 u = units[k];
      uord.push_back(u);
      const WinTile& T = tiles[u.x];
      for (int s = u.y; s < u.z; ++s)
        if (segbase[T.seg0 + s] & kSegWindow) cta_win.push_back(segbase[T.seg0 + s] & ~kSegWindow);
    }
    cta_ptr[b + 1] = (int32_t)uord.size();
    cta_wptr[b + 1] = (int32_t)cta_win.size();
  }
  e = upload(ctx, &P->units, uord);
  if (e == cudaSuccess) e = upload(ctx, &P->cta_ptr, cta_ptr);
  if (e == cudaSuccess) e = upload(ctx, &P->cta_wptr, cta_wptr);
  if (e == cudaSuccess) e = upload(ctx, &P->cta_win, cta_win);
  if (e == cudaSuccess) e = upload(ctx, &P->split, split);
  if (e == cudaSuccess)
    e = cudaMalloc((void**)&P->partials, (nslots > 0 ? nslots : 1) * kWinRows * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->xr, nbins * kWinCols * sizeof(float));
  if (e == cudaSuccess) e = cudaMemsetAsync(P->xr, 0, nbins * kWinCols * sizeof(float), ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_error(e, "window tiles");
  P->ntiles = ntiles;
  P->nseg = nseg;
  P->nunits = (int64_t)uord.size();
  P->nslots = nslots;
  P->nsplit = (int64_t)split.size();
  P->nwin = nwin;
  P->npieces = (int64_t)pf0.size();
  P->grid = grid;
  P->enabled = true;
  return GG_OK;
}

int launch_spmv_win(gg_ctx* ctx, gg_mat* A, const float* x, float* y) {
  WinPlan* P = A->winplan;
  static bool attr_set[64] = {false};
  if (ctx->device < 64 && !attr_set[ctx->device]) {
    GG_CUDA(cudaFuncSetAttribute(k_spmv_win, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWinSmem));
    attr_set[ctx->device] = true;
  }
  {
    const int64_t g = std::min<int64_t>((A->n + 255) / 256, (int64_t)ctx->num_sms * 16);
    k_win_gather_x<<<(int)std::max<int64_t>(g, 1), 256, 0, ctx->stream>>>(x, P->inv, A->n, P->xr);
    trace_count(ctx, 1);
  }
  // main kernels: the tail rows (row blocks, into yt), then the windows
  const int tr = trace_main_begin(ctx);
  GG_CHECK(launch_pipe_f32(ctx, P->tail, static_cast<const float*>(P->tail->nzval), P->xr, P->yt,
                           P->tail->colval, false));
  k_spmv_win<<<P->grid, kWinThreads, kWinSmem, ctx->stream>>>(
      P->idx, P->val, P->xr, y, P->rowperm, P->tiles, P->segbase, P->wseg, P->vptr, P->units,
      P->cta_ptr, P->cta_wptr, P->cta_win, P->yt, P->partials, ctx->d_err, copy_polls(ctx));
  trace_main_end(ctx, tr);
  trace_count(ctx, 1);
  if (P->nsplit > 0) {
    const int64_t g = std::min<int64_t>((P->nsplit * kWinRows + 255) / 256, (int64_t)ctx->num_sms * 16);
    k_win_combine<<<(int)std::max<int64_t>(g, 1), 256, 0, ctx->stream>>>(P->split, P->nsplit, P->rowperm,
                                                                         P->tiles, P->partials, P->yt, y);
    trace_count(ctx, 1);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg
