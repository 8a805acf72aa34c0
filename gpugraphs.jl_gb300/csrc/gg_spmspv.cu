// gg_spmspv.cu -- semiring SpMV over a sparse input vector (SpMSpV) and SpMV over a
// list of rows.
//
// SpMSpV, the operation gpu_spmspv! (src/spmspv.jl:1-54) was written for, over the CSR
// storage of A_T that every other entry point takes: for each row i of A that holds at
// least one entry whose column j carries an entry of x,
//     y[i] = accum(y[i], add over those entries k, in storage order, of
//                        mul(A[k], x[j], i, j, j, 1))
// with the reference's absorb early exit (src/spmv/CSR.jl:31-54); rows without such an
// entry are not written.  Two phases:
//   push: x's entries are scattered into a dense staging vector and a membership
//         bitmap; a warp per entry j of x walks column j of a column index of A and
//         marks the rows it reaches in a second bitmap, listing each row once;
//   pull: every reached row is folded in storage order over the entries whose column
//         is marked, a thread per row of at most kSpvShort entries, a warp per longer
//         row (lanes test and multiply 32 entries at once, then every lane folds the
//         present products in lane order, so the warp stops at the same absorb point).
// The fold order is the row's storage order, whatever order the rows were reached in,
// so results equal the sequential restatement bit for bit.  Work is the out-degree of
// x's entries plus the lengths of the reached rows, not n.
//
// Row-list SpMV (sparse_masked_csr_spmv_kernel!, src/spmv/CSR.jl:90-115): the plain
// storage-order fold over a dense x of the listed rows only.
//
// Both bitmaps are all zero between calls: each call clears the bits it set (the
// reached rows while writing the ordered result pattern, or from the reached list).
#include <vector>

#include "gg_semiring.cuh"

namespace gg {

static const int kSpvShort = 32;  // longer rows are folded by a warp
static const int kEmitWords = 1024;  // bitmap words per block of the ordered pattern
static const int kSpvPiece = 2048;   // entries of a long-row piece
static const int kPushLong = 4096;   // longer columns are pushed in pieces by all warps

// column index of a CSR matrix plus the SpMSpV workspace (built on first use)
struct SpvPlan {
  bool indexed = false;
  int32_t* colptr = nullptr;  // [n + 1] 0-based offsets into rows
  int32_t* rows = nullptr;    // [nnz] 0-based row of every entry of a column
  unsigned* xbits = nullptr;  // [ceil(n / 32)] columns carrying an entry of x
  unsigned* tbits = nullptr;  // [ceil(m / 32)] rows reached
  char* xs = nullptr;         // [n * 8] x's values scattered by column
  int32_t* tlist = nullptr;   // [m] rows reached, in arrival order
  int32_t* llist = nullptr;   // [m] listed rows longer than kSpvShort
  int32_t* bsum = nullptr;    // [blocks + 1] offsets of the ordered pattern
  unsigned* ctr = nullptr;    // [4] reached rows, long rows, bad input, long columns
  unsigned* h_ctr = nullptr;  // pinned copy of ctr
  // rows longer than kSpvShort cut into pieces of kSpvPiece entries (index build)
  int4* pieces = nullptr;       // [npieces] (row, first entry, end entry, 0), 0-based
  int64_t npieces = 0;
  int32_t* first_piece = nullptr;  // [m] first piece of each long row
  int32_t* pcnt = nullptr;         // [npieces] present entries of a piece (this call)
  void* prod = nullptr;            // [nnz] products of present entries, compacted per piece
  int32_t* lcol = nullptr;         // [n] columns of x too long for one warp's push (this call)
};

void free_spv_plan(gg_mat* A) {
  SpvPlan* p = A->spv;
  if (!p) return;
  cudaFree(p->colptr);
  cudaFree(p->rows);
  cudaFree(p->xbits);
  cudaFree(p->tbits);
  cudaFree(p->xs);
  cudaFree(p->tlist);
  cudaFree(p->llist);
  cudaFree(p->bsum);
  cudaFree(p->ctr);
  cudaFreeHost(p->h_ctr);
  cudaFree(p->pieces);
  cudaFree(p->first_piece);
  cudaFree(p->pcnt);
  cudaFree(p->prod);
  cudaFree(p->lcol);
  delete p;
  A->spv = nullptr;
}

template <typename T> __device__ __forceinline__ T shfl_from(T v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}
template <> __device__ __forceinline__ uint8_t shfl_from<uint8_t>(uint8_t v, int src) {
  return static_cast<uint8_t>(__shfl_sync(0xffffffffu, static_cast<int>(v), src));
}

__device__ __forceinline__ bool bit_set(const unsigned* __restrict__ bits, int64_t i) {
  return (__ldg(bits + (i >> 5)) >> (i & 31)) & 1u;
}

// ---- column index ----
__global__ void k_spv_colcount(int64_t nnz, const int32_t* __restrict__ colval, int32_t* cnt) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + (colval[k] - 1), 1);
}

// warp per row: append the row to the list of each of its columns
__global__ void k_spv_colfill(int64_t m, const int32_t* __restrict__ rowptr,
                              const int32_t* __restrict__ colval, int32_t* cursor,
                              int32_t* rows) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m; r += nw) {
    const int32_t k1 = rowptr[r + 1] - 1;
    for (int32_t k = rowptr[r] - 1 + lane; k < k1; k += 32)
      rows[atomicAdd(cursor + (colval[k] - 1), 1)] = (int32_t)r;
  }
}

// ---- SpMSpV phases ----
// x's entries into the staging vector and the membership bitmap; indices must be
// strictly increasing and inside 1:n (ctr[2] flags a violation)
__global__ void k_spv_scatter(const int32_t* __restrict__ ind, const char* __restrict__ val,
                              int esz, int64_t nx, int64_t n, char* xs, unsigned* xbits,
                              unsigned* ctr) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nx;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t j1 = ind[t];
    if (j1 < 1 || (int64_t)j1 > n || (t > 0 && ind[t - 1] >= j1)) {
      atomicOr(ctr + 2, 1u);
      continue;
    }
    const int64_t j = j1 - 1;
    for (int b = 0; b < esz; ++b) xs[j * esz + b] = val[t * esz + b];
    atomicOr(xbits + (j >> 5), 1u << (j & 31));
  }
}

// clears the bitmap words of x's entries (every set bit belongs to one of them)
__global__ void k_spv_unscatter(const int32_t* __restrict__ ind, int64_t nx, int64_t n,
                                unsigned* xbits) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nx;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t j1 = ind[t];
    if (j1 >= 1 && (int64_t)j1 <= n) xbits[(j1 - 1) >> 5] = 0u;
  }
}

// warp per entry j of x: mark the rows of column j, listing each newly reached row
__global__ void k_spv_push(const int32_t* __restrict__ ind, int64_t nx,
                           const int32_t* __restrict__ colptr, const int32_t* __restrict__ rows,
                           unsigned* tbits, int32_t* tlist, unsigned* ctr, int32_t* lcol) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nx; t += nw) {
    const int32_t j = ind[t] - 1;
    const int32_t e0 = colptr[j], e1 = colptr[j + 1];
    if (e1 - e0 > kPushLong) {  // a hub column: k_spv_push_long spreads it over the grid
      if (lane == 0) lcol[atomicAdd(ctr + 3, 1u)] = j;
      continue;
    }
    for (int32_t b = e0; b < e1; b += 32) {
      const int32_t e = b + lane;
      bool fresh = false;
      int32_t i = 0;
      if (e < e1) {
        i = rows[e];
        const unsigned bit = 1u << (i & 31);
        fresh = (atomicOr(tbits + (i >> 5), bit) & bit) == 0u;
      }
      const unsigned fm = __ballot_sync(0xffffffffu, fresh);
      if (fm) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(ctr, (unsigned)__popc(fm));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (fresh) tlist[base + __popc(fm & ((1u << lane) - 1u))] = i;
      }
    }
  }
}

// the columns k_spv_push deferred, cut into pieces of kPushLong entries numbered across
// all of them; warp w takes pieces w, w + nw, ... (every warp walks the short list of
// deferred columns to find its pieces, so no warp waits for another)
__global__ void k_spv_push_long(const int32_t* __restrict__ lcol, const int32_t* __restrict__ colptr,
                                const int32_t* __restrict__ rows, unsigned* tbits,
                                int32_t* tlist, unsigned* ctr) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned ncols = ctr[3];
  int64_t qbase = 0;  // global number of this column's first piece
  for (unsigned c = 0; c < ncols; ++c) {
    const int32_t j = lcol[c];
    const int32_t e0 = colptr[j], e1 = colptr[j + 1];
    const int64_t np = (e1 - e0 + kPushLong - 1) / kPushLong;
    for (int64_t pi = ((w - qbase) % nw + nw) % nw; pi < np; pi += nw) {
      const int32_t pe0 = e0 + (int32_t)pi * kPushLong;
      const int32_t pe1 = e1 - pe0 < kPushLong ? e1 : pe0 + kPushLong;
      for (int32_t b = pe0; b < pe1; b += 32) {
        const int32_t e = b + lane;
        bool fresh = false;
        int32_t i = 0;
        if (e < pe1) {
          i = rows[e];
          const unsigned bit = 1u << (i & 31);
          fresh = (atomicOr(tbits + (i >> 5), bit) & bit) == 0u;
        }
        const unsigned fm = __ballot_sync(0xffffffffu, fresh);
        if (fm) {
          unsigned base = 0;
          if (lane == 0) base = atomicAdd(ctr, (unsigned)__popc(fm));
          base = __shfl_sync(0xffffffffu, base, 0);
          if (fresh) tlist[base + __popc(fm & ((1u << lane) - 1u))] = i;
        }
      }
    }
    qbase += np;
  }
}

// thread per listed row (list[t] - base = 0-based row; count from the device counter
// when dcount is set): rows of at most kSpvShort entries are folded here, longer ones
// are handed to k_spv_pull_long.  kSparse: only entries whose column is in xbits.
template <int TC, bool kSparse>
__global__ void k_spv_pull(SRGen<TC> sr, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ colval, const int32_t* __restrict__ list,
                           const unsigned* dcount, int64_t hcount, int base, int64_t m,
                           const unsigned* __restrict__ xbits, int32_t* llist, unsigned* ctr) {
  typedef typename SRGen<TC>::T T;
  const int64_t cnt = dcount ? (int64_t)*dcount : hcount;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < cnt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = (int64_t)list[t] - base;
    if (r < 0 || r >= m) {
      atomicOr(ctr + 2, 1u);
      continue;
    }
    const int32_t k0 = rowptr[r] - 1, k1 = rowptr[r + 1] - 1;
    const bool is_long = k1 - k0 > kSpvShort;
    {
      // one atomic per warp for the long rows of this pass
      const unsigned am = __activemask();
      const unsigned lm = __ballot_sync(am, is_long);
      if (lm) {
        const int lane = threadIdx.x & 31, leader = __ffs(am) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(ctr + 1, (unsigned)__popc(lm));
        base = __shfl_sync(am, base, leader);
        if (is_long) llist[base + __popc(lm & ((1u << lane) - 1u))] = (int32_t)r;
      }
    }
    if (is_long) continue;
    T acc = sr.neutral();
    for (int32_t k = k0; k < k1; ++k) {
      const int32_t c1 = colval[k];
      if (kSparse && !bit_set(xbits, c1 - 1)) continue;
      acc = sr.addv(acc, sr.mulk(k, c1, r + 1));
      if (sr.is_absorb(acc)) break;
    }
    sr.write(r, acc);
  }
}

// warp per long row: 32 entries at a time are tested and multiplied by their lanes,
// then every lane adds the present products in lane (storage) order, so all lanes
// hold the same sum and leave at the same absorb point
template <int TC, bool kSparse>
__global__ void k_spv_pull_long(SRGen<TC> sr, const int32_t* __restrict__ rowptr,
                                const int32_t* __restrict__ colval,
                                const int32_t* __restrict__ llist, const unsigned* __restrict__ ctr,
                                const unsigned* __restrict__ xbits) {
  typedef typename SRGen<TC>::T T;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t cnt = ctr[1];
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < cnt; t += nw) {
    const int32_t r = llist[t];
    const int32_t k0 = rowptr[r] - 1, k1 = rowptr[r + 1] - 1;
    T acc = sr.neutral();
    bool done = false;
    for (int32_t b = k0; b < k1 && !done; b += 32) {
      const int32_t k = b + lane;
      bool on = false;
      T p = sr.neutral();
      if (k < k1) {
        const int32_t c1 = colval[k];
        on = !kSparse || bit_set(xbits, c1 - 1);
        if (on) p = sr.mulk(k, c1, (int64_t)r + 1);
      }
      unsigned om = __ballot_sync(0xffffffffu, on);
      while (om) {
        const int src = __ffs(om) - 1;
        om &= om - 1u;
        acc = sr.addv(acc, shfl_from<T>(p, src));
        if (sr.is_absorb(acc)) {
          done = true;
          break;
        }
      }
    }
    if (lane == 0) sr.write(r, acc);
  }
}

// Long rows of SpMSpV, pass 1: a warp per piece of a reached long row tests 128 entries
// per step (4 per lane, loads issued together), multiplies the present ones and writes
// their products compacted in storage order at the start of the piece's own range of
// prod; pcnt[p] = how many.  Pieces of rows not reached cost one bitmap test.
template <int TC>
__global__ void k_spv_compact(SRGen<TC> sr, const int4* __restrict__ pieces, int64_t npieces,
                              const int32_t* __restrict__ colval, const unsigned* __restrict__ tbits,
                              const unsigned* __restrict__ xbits, int32_t* pcnt,
                              typename SRGen<TC>::T* prod) {
  typedef typename SRGen<TC>::T T;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < npieces; p += nw) {
    const int4 d = pieces[p];
    if (!bit_set(tbits, d.x)) continue;
    int32_t cnt = 0;
    for (int32_t base = d.y; base < d.z; base += 128) {
      int32_t c[4];
      bool on[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int32_t k = base + 32 * u + lane;
        c[u] = k < d.z ? __ldg(colval + k) : 0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) on[u] = c[u] > 0 && bit_set(xbits, c[u] - 1);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int32_t k = base + 32 * u + lane;
        const unsigned m = __ballot_sync(0xffffffffu, on[u]);
        if (on[u])
          prod[d.y + cnt + __popc(m & ((1u << lane) - 1u))] = sr.mulk(k, c[u], (int64_t)d.x + 1);
        cnt += __popc(m);
      }
    }
    if (lane == 0) pcnt[p] = cnt;
  }
}

// Long rows of SpMSpV, pass 2: a warp per reached long row walks its pieces 32 counts at
// a time and adds the compacted products in order (every lane holds the same sum; the
// warp leaves at the first absorbing value), then writes the row.
template <int TC>
__global__ void k_spv_fold_long(SRGen<TC> sr, const int32_t* __restrict__ rowptr,
                                const int32_t* __restrict__ llist, const unsigned* __restrict__ ctr,
                                const int32_t* __restrict__ first_piece,
                                const int32_t* __restrict__ pcnt,
                                const typename SRGen<TC>::T* __restrict__ prod) {
  typedef typename SRGen<TC>::T T;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t cnt_rows = ctr[1];
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < cnt_rows; t += nw) {
    const int32_t r = llist[t];
    const int32_t k0 = rowptr[r] - 1, k1 = rowptr[r + 1] - 1;
    const int32_t p0 = first_piece[r];
    const int32_t np = (k1 - k0 + kSpvPiece - 1) / kSpvPiece;
    T acc = sr.neutral();
    bool done = false;
    for (int32_t pb = 0; pb < np && !done; pb += 32) {
      const int32_t cl = pb + lane < np ? pcnt[p0 + pb + lane] : 0;
      unsigned nzm = __ballot_sync(0xffffffffu, cl > 0);
      while (nzm && !done) {
        const int src = __ffs(nzm) - 1;
        nzm &= nzm - 1u;
        const int32_t cnt = __shfl_sync(0xffffffffu, cl, src);
        const int64_t start = (int64_t)k0 + (int64_t)(pb + src) * kSpvPiece;
        for (int32_t q = 0; q < cnt && !done; q += 32) {
          const T v = q + lane < cnt ? prod[start + q + lane] : sr.neutral();
          const int n = cnt - q < 32 ? cnt - q : 32;
          for (int i = 0; i < n; ++i) {
            acc = sr.addv(acc, shfl_from<T>(v, i));
            if (sr.is_absorb(acc)) {
              done = true;
              break;
            }
          }
        }
      }
    }
    if (lane == 0) sr.write(r, acc);
  }
}

// ---- the result pattern in ascending order ----
__global__ void __launch_bounds__(kEmitWords) k_spv_bcount(const unsigned* __restrict__ tbits,
                                                           int64_t nwords, int32_t* bsum) {
  __shared__ int32_t ws[kEmitWords / 32];
  const int64_t w = (int64_t)blockIdx.x * kEmitWords + threadIdx.x;
  int32_t c = w < nwords ? __popc(tbits[w]) : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    int32_t s = ws[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) bsum[blockIdx.x] = s;
  }
}

// one warp: exclusive prefix sums of the nb block counts (bsum[nb] = total)
__global__ void k_spv_bscan(int32_t* bsum, int64_t nb) {
  const int lane = threadIdx.x & 31;
  int32_t carry = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += 32) {
    const int64_t i = b0 + lane;
    const int32_t v = i < nb ? bsum[i] : 0;
    int32_t s = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    if (i < nb) bsum[i] = carry + s - v;
    carry += __shfl_sync(0xffffffffu, s, 31);
  }
  if (lane == 0) bsum[nb] = carry;
}

// writes the reached rows (1-based, ascending) and clears their bitmap words
__global__ void __launch_bounds__(kEmitWords) k_spv_emit(unsigned* tbits, int64_t nwords,
                                                         const int32_t* __restrict__ bsum,
                                                         int32_t* out) {
  __shared__ int32_t ws[kEmitWords / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t w = (int64_t)blockIdx.x * kEmitWords + threadIdx.x;
  unsigned word = w < nwords ? tbits[w] : 0u;
  const int32_t c = __popc(word);
  int32_t s = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t u = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += u;
  }
  if (lane == 31) ws[wid] = s;
  __syncthreads();
  if (wid == 0) {
    int32_t t = ws[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    ws[lane] = t;
  }
  __syncthreads();
  int32_t pos = bsum[blockIdx.x] + (wid > 0 ? ws[wid - 1] : 0) + s - c;
  if (word) {
    while (word) {
      const int b = __ffs(word) - 1;
      word &= word - 1u;
      out[pos++] = (int32_t)(w * 32 + b + 1);
    }
    tbits[w] = 0u;
  }
}

// clears the bitmap words of the reached rows (when no ordered pattern is asked for)
__global__ void k_spv_unmark(const int32_t* __restrict__ tlist, const unsigned* __restrict__ ctr,
                             unsigned* tbits) {
  const int64_t cnt = ctr[0];
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < cnt;
       t += (int64_t)gridDim.x * blockDim.x)
    tbits[tlist[t] >> 5] = 0u;
}

static int spv_grid(gg_ctx* ctx, int64_t work, int block = 256) {
  int64_t g = (work + block - 1) / block;
  const int64_t cap = (int64_t)ctx->num_sms * (2048 / block);
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// workspace (bitmaps, lists, counters); the column index only when `index` is set
static int ensure_spv(gg_ctx* ctx, gg_mat* A, bool index) {
  if (!A->spv) {
    SpvPlan* p = new SpvPlan();
    A->spv = p;
    const int64_t m = A->m, n = A->n;
    const int64_t mw = (m + 31) / 32 + 1, nwd = (n + 31) / 32 + 1;
    cudaError_t e = cudaMalloc((void**)&p->xbits, nwd * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->tbits, mw * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->xs, (n > 0 ? n : 1) * 8);
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->tlist, (m > 0 ? m : 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->llist, (m > 0 ? m : 1) * sizeof(int32_t));
    if (e == cudaSuccess)
      e = cudaMalloc((void**)&p->bsum, (mw / kEmitWords + 2) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->lcol, (n > 0 ? n : 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->ctr, 4 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->h_ctr, 4 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemsetAsync(p->xbits, 0, nwd * sizeof(unsigned), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->tbits, 0, mw * sizeof(unsigned), ctx->stream);
    if (e != cudaSuccess) {
      free_spv_plan(A);
      return cuda_error(e, "SpMSpV workspace");
    }
  }
  SpvPlan* p = A->spv;
  if (!index || p->indexed) return GG_OK;
  const int64_t m = A->m, n = A->n, nnz = A->nnz;
  int32_t* cnt = nullptr;
  GG_CUDA(cudaMalloc((void**)&p->colptr, (n + 1) * sizeof(int32_t)));
  GG_CUDA(cudaMalloc((void**)&p->rows, (nnz > 0 ? nnz : 1) * sizeof(int32_t)));
  GG_CUDA(cudaMalloc((void**)&cnt, (n > 0 ? n : 1) * sizeof(int32_t)));
  GG_CUDA(cudaMemsetAsync(cnt, 0, (n > 0 ? n : 1) * sizeof(int32_t), ctx->stream));
  if (nnz > 0) k_spv_colcount<<<spv_grid(ctx, nnz), 256, 0, ctx->stream>>>(nnz, A->colval, cnt);
  cudaError_t e = cudaGetLastError();
  int rc = e == cudaSuccess ? scan_counts(ctx, cnt, n, p->colptr, 0) : cuda_error(e, "column count");
  if (rc == GG_OK) {
    e = cudaMemcpyAsync(cnt, p->colptr, (n > 0 ? n : 1) * sizeof(int32_t),
                        cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess && m > 0 && nnz > 0) {
      k_spv_colfill<<<spv_grid(ctx, m * 32), 256, 0, ctx->stream>>>(m, A->rowptr, A->colval, cnt,
                                                                    p->rows);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_error(e, "column index");
  }
  cudaFree(cnt);
  if (rc != GG_OK) return rc;
  // pieces of the long rows (host table from the row pointers) and the product buffer
  std::vector<int32_t> rp((size_t)m + 1);
  GG_CUDA(cudaMemcpy(rp.data(), A->rowptr, (m + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost));
  std::vector<int4> pcs;
  std::vector<int32_t> first((size_t)(m > 0 ? m : 1), -1);
  for (int64_t r = 0; r < m; ++r) {
    const int32_t k0 = rp[(size_t)r] - 1, k1 = rp[(size_t)r + 1] - 1;
    if (k1 - k0 <= kSpvShort) continue;
    first[(size_t)r] = (int32_t)pcs.size();
    for (int32_t k = k0; k < k1; k += kSpvPiece)
      pcs.push_back(make_int4((int32_t)r, k, k1 - k < kSpvPiece ? k1 : k + kSpvPiece, 0));
  }
  p->npieces = (int64_t)pcs.size();
  const size_t np = pcs.size() > 0 ? pcs.size() : 1;
  GG_CUDA(cudaMalloc((void**)&p->pieces, np * sizeof(int4)));
  GG_CUDA(cudaMalloc((void**)&p->pcnt, np * sizeof(int32_t)));
  GG_CUDA(cudaMalloc((void**)&p->first_piece, first.size() * sizeof(int32_t)));
  GG_CUDA(cudaMalloc(&p->prod, (size_t)(nnz > 0 ? nnz : 1) * 8));
  if (!pcs.empty())
    GG_CUDA(cudaMemcpy(p->pieces, pcs.data(), pcs.size() * sizeof(int4), cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemcpy(p->first_piece, first.data(), first.size() * sizeof(int32_t),
                     cudaMemcpyHostToDevice));
  p->indexed = true;
  return GG_OK;
}

template <int TC>
static SRGen<TC> spv_semiring(gg_mat* A, int mul, int add, int accum, void* y, int ty,
                              const void* x, int tx) {
  typedef typename CType<TC>::T T;
  SRGen<TC> sr;
  sr.mul = mul;
  sr.add = add;
  sr.accum = accum;
  sr.tv = A->dtype;
  sr.tx = tx;
  sr.ty = ty;
  sr.neutral_v = neutral_of<T>(add);
  sr.has_absorb = absorb_of<T>(add, &sr.absorb_v);
  sr.nz = A->nzval;
  sr.x = x;
  sr.y = y;
  sr.ldb = 0;
  sr.ldc = 0;
  sr.layout = GG_COL_MAJOR;
  return sr;
}

// the pull phases over a row list (device count ctr[0] when rows == nullptr)
template <int TC, bool kSparse>
static int spv_pull(gg_ctx* ctx, gg_mat* A, const SRGen<TC>& sr, const int32_t* rows,
                    int64_t nrows) {
  SpvPlan* p = A->spv;
  const int64_t bound = rows ? nrows : A->m;
  const int64_t m = A->m;
  if (bound > 0) {
    k_spv_pull<TC, kSparse><<<spv_grid(ctx, bound), 256, 0, ctx->stream>>>(
        sr, A->rowptr, A->colval, rows ? rows : p->tlist, rows ? nullptr : p->ctr, nrows,
        rows ? 1 : 0, m, p->xbits, p->llist, p->ctr);
    GG_CUDA(cudaGetLastError());
    if (kSparse) {
      // long rows: present products compacted per piece by many warps, then folded in
      // order by a warp per row (a hub is not walked by one warp entry by entry)
      typedef typename SRGen<TC>::T T;
      if (p->npieces > 0) {
        k_spv_compact<TC><<<spv_grid(ctx, p->npieces * 32), 256, 0, ctx->stream>>>(
            sr, p->pieces, p->npieces, A->colval, p->tbits, p->xbits, p->pcnt,
            static_cast<T*>(p->prod));
        GG_CUDA(cudaGetLastError());
        k_spv_fold_long<TC><<<spv_grid(ctx, bound * 32), 256, 0, ctx->stream>>>(
            sr, A->rowptr, p->llist, p->ctr, p->first_piece, p->pcnt, static_cast<const T*>(p->prod));
        GG_CUDA(cudaGetLastError());
      }
      trace_count(ctx, 3);
      return GG_OK;
    }
    k_spv_pull_long<TC, kSparse><<<spv_grid(ctx, bound * 32), 256, 0, ctx->stream>>>(
        sr, A->rowptr, A->colval, p->llist, p->ctr, p->xbits);
    GG_CUDA(cudaGetLastError());
  }
  trace_count(ctx, 2);
  return GG_OK;
}

template <int TC>
static int spmspv_t(gg_ctx* ctx, gg_mat* A, int mul, int add, int accum, void* y, int ty,
                    const int32_t* x_ind, const void* x_val, int tx, int64_t x_nnz,
                    int32_t* y_ind, int64_t* y_nnz) {
  SpvPlan* p = A->spv;
  const int64_t m = A->m, n = A->n;
  GG_CUDA(cudaMemsetAsync(p->ctr, 0, 4 * sizeof(unsigned), ctx->stream));
  if (x_nnz > 0) {
    k_spv_scatter<<<spv_grid(ctx, x_nnz), 256, 0, ctx->stream>>>(
        x_ind, static_cast<const char*>(x_val), dtype_size(tx), x_nnz, n, p->xs, p->xbits, p->ctr);
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(p->h_ctr, p->ctr, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost,
                            ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (p->h_ctr[2]) {
      k_spv_unscatter<<<spv_grid(ctx, x_nnz), 256, 0, ctx->stream>>>(x_ind, x_nnz, n, p->xbits);
      GG_CUDA(cudaGetLastError());
      GG_CUDA(cudaStreamSynchronize(ctx->stream));
      return set_error(GG_ERR_ARGUMENT, "x.nzind must be strictly increasing and inside 1:%lld",
                       (long long)n);
    }
    const int tr = trace_main_begin(ctx);
    k_spv_push<<<spv_grid(ctx, x_nnz * 32), 256, 0, ctx->stream>>>(x_ind, x_nnz, p->colptr,
                                                                   p->rows, p->tbits, p->tlist,
                                                                   p->ctr, p->lcol);
    GG_CUDA(cudaGetLastError());
    k_spv_push_long<<<spv_grid(ctx, (int64_t)ctx->num_sms * 2048), 256, 0, ctx->stream>>>(
        p->lcol, p->colptr, p->rows, p->tbits, p->tlist, p->ctr);
    GG_CUDA(cudaGetLastError());
    trace_count(ctx, 3);
    GG_CHECK((spv_pull<TC, true>(ctx, A, spv_semiring<TC>(A, mul, add, accum, y, ty, p->xs, tx),
                                 nullptr, 0)));
    trace_main_end(ctx, tr);
    const int64_t nwords = (m + 31) / 32;
    if (y_ind) {
      const int64_t nb = (nwords + kEmitWords - 1) / kEmitWords;
      if (nb > 0) {
        k_spv_bcount<<<(unsigned)nb, kEmitWords, 0, ctx->stream>>>(p->tbits, nwords, p->bsum);
        k_spv_bscan<<<1, 32, 0, ctx->stream>>>(p->bsum, nb);
        k_spv_emit<<<(unsigned)nb, kEmitWords, 0, ctx->stream>>>(p->tbits, nwords, p->bsum, y_ind);
        GG_CUDA(cudaGetLastError());
        trace_count(ctx, 3);
      }
    } else if (m > 0) {
      k_spv_unmark<<<spv_grid(ctx, m), 256, 0, ctx->stream>>>(p->tlist, p->ctr, p->tbits);
      GG_CUDA(cudaGetLastError());
      trace_count(ctx, 1);
    }
    k_spv_unscatter<<<spv_grid(ctx, x_nnz), 256, 0, ctx->stream>>>(x_ind, x_nnz, n, p->xbits);
    GG_CUDA(cudaGetLastError());
    trace_count(ctx, 1);
  }
  GG_CUDA(cudaMemcpyAsync(p->h_ctr, p->ctr, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (y_nnz) *y_nnz = x_nnz > 0 ? (int64_t)p->h_ctr[0] : 0;
  return GG_OK;
}

template <int TC>
static int spmv_rows_t(gg_ctx* ctx, gg_mat* A, int mul, int add, int accum, void* y, int ty,
                       const void* x, int tx, const int32_t* rows, int64_t nrows) {
  SpvPlan* p = A->spv;
  GG_CUDA(cudaMemsetAsync(p->ctr, 0, 4 * sizeof(unsigned), ctx->stream));
  const int tr = trace_main_begin(ctx);
  GG_CHECK((spv_pull<TC, false>(ctx, A, spv_semiring<TC>(A, mul, add, accum, y, ty, x, tx), rows,
                                nrows)));
  trace_main_end(ctx, tr);
  GG_CUDA(cudaMemcpyAsync(p->h_ctr, p->ctr, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (p->h_ctr[2])
    return set_error(GG_ERR_BOUNDS, "row index outside 1:%lld", (long long)A->m);
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_spmspv(gg_ctx* ctx, const gg_mat* A_, int mul, int add, int accum, void* y, int y_dtype,
              int64_t y_len, const int32_t* x_ind, const void* x_val, int x_dtype,
              int64_t x_nnz, int64_t x_len, int32_t* y_ind, int64_t* y_nnz) {
  if (!ctx || !A_) return set_error(GG_ERR_ARGUMENT, "ctx / A is NULL");
  gg_mat* A = const_cast<gg_mat*>(A_);
  if (A->format != GG_FMT_CSR)
    return set_error(GG_ERR_UNSUPPORTED, "gpu_spmspv! takes a SparseGPUMatrixCSR");
  // the dimension checks of gpu_spmspv! (src/spmspv.jl:31-37)
  if (A->n != x_len) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  if (y_len != A->m) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  if (x_nnz < 0 || x_nnz > x_len)
    return set_error(GG_ERR_ARGUMENT, "x holds %lld entries for length %lld", (long long)x_nnz,
                     (long long)x_len);
  int tc = 0;
  GG_CHECK(check_semiring(A->dtype, x_dtype, y_dtype, mul, add, accum, &tc));
  if (x_nnz > 0 && (!x_ind || !x_val)) return set_error(GG_ERR_ARGUMENT, "NULL sparse vector");
  if (A->m > 0 && !y) return set_error(GG_ERR_ARGUMENT, "NULL vector");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_CHECK(ensure_spv(ctx, A, true));
  switch (tc) {
    case GG_BOOL: return spmspv_t<GG_BOOL>(ctx, A, mul, add, accum, y, y_dtype, x_ind, x_val, x_dtype, x_nnz, y_ind, y_nnz);
    case GG_INT32: return spmspv_t<GG_INT32>(ctx, A, mul, add, accum, y, y_dtype, x_ind, x_val, x_dtype, x_nnz, y_ind, y_nnz);
    case GG_INT64: return spmspv_t<GG_INT64>(ctx, A, mul, add, accum, y, y_dtype, x_ind, x_val, x_dtype, x_nnz, y_ind, y_nnz);
    case GG_FLOAT32: return spmspv_t<GG_FLOAT32>(ctx, A, mul, add, accum, y, y_dtype, x_ind, x_val, x_dtype, x_nnz, y_ind, y_nnz);
    default: return spmspv_t<GG_FLOAT64>(ctx, A, mul, add, accum, y, y_dtype, x_ind, x_val, x_dtype, x_nnz, y_ind, y_nnz);
  }
}

int gg_spmv_rows(gg_ctx* ctx, const gg_mat* A_, int mul, int add, int accum, void* y,
                 int y_dtype, int64_t y_len, const void* x, int x_dtype, int64_t x_len,
                 const int32_t* rows, int64_t nrows) {
  if (!ctx || !A_) return set_error(GG_ERR_ARGUMENT, "ctx / A is NULL");
  gg_mat* A = const_cast<gg_mat*>(A_);
  if (A->format != GG_FMT_CSR)
    return set_error(GG_ERR_UNSUPPORTED, "the row-list SpMV takes a SparseGPUMatrixCSR");
  if (A->n != x_len) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  if (y_len != A->m) return set_error(GG_ERR_DIMENSION, "Matrix dimensions must agree");
  if (nrows < 0) return set_error(GG_ERR_ARGUMENT, "negative row count");
  int tc = 0;
  GG_CHECK(check_semiring(A->dtype, x_dtype, y_dtype, mul, add, accum, &tc));
  if (nrows == 0) return GG_OK;
  if (!rows || !y || (A->n > 0 && !x)) return set_error(GG_ERR_ARGUMENT, "NULL vector");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_CHECK(ensure_spv(ctx, A, false));
  switch (tc) {
    case GG_BOOL: return spmv_rows_t<GG_BOOL>(ctx, A, mul, add, accum, y, y_dtype, x, x_dtype, rows, nrows);
    case GG_INT32: return spmv_rows_t<GG_INT32>(ctx, A, mul, add, accum, y, y_dtype, x, x_dtype, rows, nrows);
    case GG_INT64: return spmv_rows_t<GG_INT64>(ctx, A, mul, add, accum, y, y_dtype, x, x_dtype, rows, nrows);
    case GG_FLOAT32: return spmv_rows_t<GG_FLOAT32>(ctx, A, mul, add, accum, y, y_dtype, x, x_dtype, rows, nrows);
    default: return spmv_rows_t<GG_FLOAT64>(ctx, A, mul, add, accum, y, y_dtype, x, x_dtype, rows, nrows);
  }
}

}  // extern "C"
