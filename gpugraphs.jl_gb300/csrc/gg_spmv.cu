// gg_spmv.cu -- semiring SpMV over CSR and SELL (gpu_spmv!, src/spmv/CSR.jl and
// src/spmv/SELL.jl of GPUGraphs.jl).
//
// Kernels
//  * k_csr_rowblock<SR>: unmasked CSR.  One warp per regular row block (<= 256
//    stored entries): the warp computes mul(A[k], x[col[k]]) for the whole block
//    with coalesced loads into shared memory, then every lane folds one row from
//    shared memory in storage order -- the reference's sequential order, so these
//    rows are bit-identical to it.  Long rows are cut into 2048-entry segments;
//    each segment is reduced by one warp (lane partials + shuffle tree) and the warp
//    that finishes a row's last segment combines the partials in order.  One launch
//    covers both kinds of work item.
//    Mask / range variants use the same kernel with a row filter, so every row with
//    at most 256 entries is folded in storage order whatever the variant.
//  * k_csr_first_hit<TC>: add == GPUGraphs_any with a mask on CSR: the first stored
//    column whose x is nonzero (any_dense_masked_csr_spmv_kernel!, CSR.jl:147-171).
//  * k_sell<SR>: one thread per stored SELL row walking its slice with stride C
//    (slice-column-major, so a warp reads C consecutive words), stopping at the
//    first -1 padding column like sell_spmv_kernel! (SELL.jl:31-63).
#include <vector>

#include "gg_semiring.cuh"

namespace gg {

static const unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned group_mask(int G) {
  if (G >= 32) return kFull;
  int lane = threadIdx.x & 31;
  return ((1u << G) - 1u) << (lane & ~(G - 1));
}

template <typename T>
__device__ __forceinline__ T shfl_xor_m(unsigned mask, T v, int off, int width) {
  return __shfl_xor_sync(mask, v, off, width);
}
template <>
__device__ __forceinline__ uint8_t shfl_xor_m<uint8_t>(unsigned mask, uint8_t v, int off,
                                                       int width) {
  return static_cast<uint8_t>(__shfl_xor_sync(mask, static_cast<int>(v), off, width));
}

// ---------------------------------------------------------------------------------
// row-block kernel (unmasked CSR)
// ---------------------------------------------------------------------------------
static const int kRBWarps = 8;  // warps per CTA

// Row filter of the masked / range variants (CSR.jl:117-144, :224-313): a row is
// computed when it lies in [lo, hi) (0-based) and mask[row] != 0.
struct RowFilter {
  const void* mask;
  int tmask;
  int64_t lo, hi;
  __device__ __forceinline__ bool keep(int64_t r) const {
    if (r < lo || r >= hi) return false;
    return !mask || !raw_is_zero(load_raw(mask, tmask, r), tmask);
  }
};

// row of stored entry k inside rows [r0, r1) (binary search; only index operators
// that read the row id need it during staging)
__device__ __forceinline__ int64_t row_of(const int32_t* rowptr, int32_t r0, int32_t r1, int32_t k) {
  int32_t lo = r0, hi = r1 - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(rowptr + mid) - 1 <= k) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <class SR, bool kFiltered, bool kNeedsRow>
__global__ void __launch_bounds__(kRBWarps * 32)
    k_csr_rowblock(SR sr, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
                   const int2* __restrict__ blocks, int64_t nblocks, const int4* __restrict__ segs,
                   int64_t nsegs, const int32_t* __restrict__ long_first_seg,
                   const int32_t* __restrict__ long_rows, unsigned int* long_count,
                   typename SR::T* partials, RowFilter flt) {
  typedef typename SR::T T;
  __shared__ T stage[kRBWarps][kBlockNnz];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * kRBWarps;
  T* st = stage[warp];
  for (int64_t item = (int64_t)blockIdx.x * kRBWarps + warp; item < nblocks + nsegs; item += nw) {
    if (item < nblocks) {
      const int2 b = blocks[item];
      if (kFiltered && (b.y <= flt.lo || b.x >= flt.hi)) continue;
      const int32_t k0 = __ldg(rowptr + b.x) - 1;
      const int32_t k1 = __ldg(rowptr + b.y) - 1;
      // stage products: 8 independent coalesced loads in flight per lane
      T v[kBlockNnz / 32];
#pragma unroll
      for (int u = 0; u < kBlockNnz / 32; ++u) {
        const int32_t k = k0 + u * 32 + lane;
        if (k < k1)
          v[u] = sr.mulk(k, __ldcs(colval + k), kNeedsRow ? row_of(rowptr, b.x, b.y, k) + 1 : 0);
      }
#pragma unroll
      for (int u = 0; u < kBlockNnz / 32; ++u) {
        const int32_t k = k0 + u * 32 + lane;
        if (k < k1) st[u * 32 + lane] = v[u];
      }
      __syncwarp();
      for (int32_t r = b.x + lane; r < b.y; r += 32) {
        if (kFiltered && !flt.keep(r)) continue;
        const int32_t s = __ldg(rowptr + r) - 1 - k0;
        const int32_t e = __ldg(rowptr + r + 1) - 1 - k0;
        T acc = sr.neutral();
        for (int32_t i = s; i < e; ++i) {
          acc = sr.addv(acc, st[i]);
          if (SR::kHasAbsorbCheck && sr.is_absorb(acc)) break;
        }
        sr.write(r, acc);
      }
      __syncwarp();
    } else {
      const int64_t si = item - nblocks;
      const int4 sg = segs[si];  // row, k_begin, k_end, long-row index
      if (kFiltered && !flt.keep(sg.x)) continue;
      T acc = sr.neutral();
      for (int32_t base = sg.y; base < sg.z; base += 32 * 4) {
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int32_t k = base + u * 32 + lane;
          v[u] = (k < sg.z) ? sr.mulk(k, __ldcs(colval + k), sg.x + 1) : sr.neutral();
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) acc = sr.addv(acc, v[u]);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc = sr.addv(acc, shfl_xor_m<T>(kFull, acc, off, 32));
      unsigned prev = 0;
      if (lane == 0) {
        partials[si] = acc;
        __threadfence();
        prev = atomicAdd(long_count + sg.w, 1u);
      }
      prev = __shfl_sync(kFull, prev, 0);
      const int32_t f0 = long_first_seg[sg.w], f1 = long_first_seg[sg.w + 1];
      if (prev == (unsigned)(f1 - f0 - 1)) {  // this warp completed the row
        __threadfence();
        if (lane == 0) {
          T tot = sr.neutral();
          for (int32_t q = f0; q < f1; ++q) tot = sr.addv(tot, __ldcg(partials + q));
          sr.write(long_rows[sg.w], tot);
          long_count[sg.w] = 0;  // ready for the next launch
        }
      }
    }
  }
}

// first frontier column in storage order (CSR, add == any, mask)
template <int TC>
__global__ void k_csr_first_hit(SRGen<TC> sr, const int32_t* __restrict__ rowptr,
                                const int32_t* __restrict__ colval, int64_t nrows,
                                const void* mask, int tmask, int G) {
  typedef typename CType<TC>::T T;
  const unsigned gm = group_mask(G);
  const int lg = threadIdx.x & (G - 1);
  const int gbase = (threadIdx.x & 31) & ~(G - 1);
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
  for (int64_t r = gid; r < nrows; r += ng) {
    if (raw_is_zero(load_raw(mask, tmask, r), tmask)) continue;
    const int32_t k0 = rowptr[r] - 1, k1 = rowptr[r + 1] - 1;
    for (int32_t base = k0; base < k1; base += G) {
      const int32_t k = base + lg;
      bool hit = false;
      int32_t col = 0;
      Raw b;
      b.i = 0;
      b.d = 0;
      if (k < k1) {
        col = colval[k];
        b = load_raw(sr.x, sr.tx, col - 1);
        hit = !raw_is_zero(b, sr.tx);
      }
      const unsigned bal = (__ballot_sync(gm, hit) >> gbase) & ((G >= 32) ? kFull : ((1u << G) - 1u));
      if (bal) {
        if (lg == __ffs(bal) - 1) {
          Raw a = load_raw(sr.nz, sr.tv, k);
          T mres = apply_op<TC>(sr.mul, raw_to<TC>(a, sr.tv), raw_to<TC>(b, sr.tx), b, sr.tx, r + 1,
                                col, col, 1);
          sr.write(r, mres);
        }
        break;
      }
    }
  }
}

// ---------------------------------------------------------------------------------
// SELL: one thread per stored row
// ---------------------------------------------------------------------------------
template <class SR>
__global__ void k_sell(SR sr, const int32_t* __restrict__ slice_ptr,
                       const int32_t* __restrict__ colval, const int32_t* __restrict__ perm,
                       int64_t C, int64_t sr_lo, int64_t sr_hi, int64_t range_lo, int64_t range_hi,
                       const void* mask, int tmask) {
  typedef typename SR::T T;
  for (int64_t t = sr_lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < sr_hi;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / C, o = t - s * C;
    const int64_t r1 = perm ? (int64_t)perm[t] : t + 1;  // original row, 1-based
    if (range_lo > 0 && (r1 < range_lo || r1 > range_hi)) continue;
    if (mask && raw_is_zero(load_raw(mask, tmask, r1 - 1), tmask)) continue;
    const int64_t i0 = (int64_t)slice_ptr[s] - 1 + o, i1 = (int64_t)slice_ptr[s + 1] - 1;
    T acc = sr.neutral();
    for (int64_t i = i0; i < i1; i += C) {
      const int32_t col = __ldcs(colval + i);
      if (col == -1) break;
      acc = sr.addv(acc, sr.mulk(i, col, r1));
    }
    sr.write(r1 - 1, acc);
  }
}

// ---------------------------------------------------------------------------------
// analysis: row blocks and long-row segments (built once per matrix, on first use)
// ---------------------------------------------------------------------------------
int build_row_blocks(gg_ctx* ctx, gg_mat* A) {
  if (A->blocks) return GG_OK;
  const int64_t m = A->m;
  std::vector<int32_t> rp(m + 1);
  GG_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr, (m + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int2> blocks;
  std::vector<int4> segs;
  std::vector<int32_t> first_seg, long_rows;
  blocks.reserve(m / 8 + 16);
  int64_t r = 0;
  while (r < m) {
    int64_t len = rp[r + 1] - rp[r];
    if (len > kBlockNnz) {
      int32_t li = (int32_t)long_rows.size();
      long_rows.push_back((int32_t)r);
      first_seg.push_back((int32_t)segs.size());
      for (int64_t kb = rp[r] - 1; kb < rp[r + 1] - 1; kb += kSegNnz) {
        int64_t ke = kb + kSegNnz < rp[r + 1] - 1 ? kb + kSegNnz : rp[r + 1] - 1;
        segs.push_back(make_int4((int)r, (int)kb, (int)ke, li));
      }
      ++r;
      continue;
    }
    int64_t first = r, cnt = 0;
    while (r < m && r - first < kBlockRows) {
      int64_t l = rp[r + 1] - rp[r];
      if (l > kBlockNnz || cnt + l > kBlockNnz) break;
      cnt += l;
      ++r;
    }
    blocks.push_back(make_int2((int)first, (int)r));
  }
  first_seg.push_back((int32_t)segs.size());

  RowBlocks* rb = new RowBlocks();
  rb->nblocks = (int64_t)blocks.size();
  rb->nsegs = (int64_t)segs.size();
  rb->nlong = (int64_t)long_rows.size();
  rb->partial_bytes = rb->nsegs * 8;
  cudaError_t e = cudaSuccess;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(dst, bytes > 0 ? bytes : 16);
    if (e == cudaSuccess && bytes > 0)
      e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  };
  up((void**)&rb->blocks, blocks.data(), blocks.size() * sizeof(int2));
  up((void**)&rb->segs, segs.data(), segs.size() * sizeof(int4));
  up((void**)&rb->long_first_seg, first_seg.data(), first_seg.size() * sizeof(int32_t));
  up((void**)&rb->long_rows, long_rows.data(), long_rows.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&rb->long_count, (rb->nlong + 1) * sizeof(unsigned));
  if (e == cudaSuccess)
    e = cudaMemsetAsync(rb->long_count, 0, (rb->nlong + 1) * sizeof(unsigned), ctx->stream);
  if (e == cudaSuccess) e = cudaMalloc(&rb->partials, rb->partial_bytes > 0 ? rb->partial_bytes : 16);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(rb->blocks);
    cudaFree(rb->segs);
    cudaFree(rb->long_first_seg);
    cudaFree(rb->long_rows);
    cudaFree(rb->long_count);
    cudaFree(rb->partials);
    delete rb;
    return cuda_error(e, "row-block analysis");
  }
  A->blocks = rb;
  return GG_OK;
}

static int grid_for(gg_ctx* ctx, int64_t threads, int block) {
  int64_t g = (threads + block - 1) / block;
  int64_t cap = (int64_t)ctx->num_sms * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

static int group_width(const gg_mat* A) {
  double avg = A->m > 0 ? (double)A->nnz / (double)A->m : 0.0;
  int G = 1;
  while (G < 32 && G < avg) G <<= 1;
  return G;
}

template <class SR, bool kFiltered, bool kNeedsRow>
int launch_rowblock_t(gg_ctx* ctx, gg_mat* A, const SR& sr, const RowFilter& flt) {
  GG_CHECK(build_row_blocks(ctx, A));
  RowBlocks* rb = A->blocks;
  const int64_t items = rb->nblocks + rb->nsegs;
  if (items == 0) return GG_OK;
  int64_t grid = (items + kRBWarps - 1) / kRBWarps;
  const int64_t cap = (int64_t)ctx->num_sms * 8;  // 8 CTAs x 8 warps = 64 warps per SM
  if (grid > cap) grid = cap;
  k_csr_rowblock<SR, kFiltered, kNeedsRow><<<(int)grid, kRBWarps * 32, 0, ctx->stream>>>(
      sr, A->rowptr, A->colval, rb->blocks, rb->nblocks, rb->segs, rb->nsegs, rb->long_first_seg,
      rb->long_rows, rb->long_count, static_cast<typename SR::T*>(rb->partials), flt);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

template <class SR>
int launch_rowblock(gg_ctx* ctx, gg_mat* A, const SR& sr, const void* mask = nullptr,
                    int tmask = 0, int64_t lo = 0, int64_t hi = 0, bool needs_row = false) {
  RowFilter flt;
  flt.mask = mask;
  flt.tmask = tmask;
  flt.lo = lo > 0 ? lo - 1 : 0;
  flt.hi = lo > 0 ? hi : A->m;
  const bool filtered = mask != nullptr || lo > 0;
  if (needs_row) {
    if (filtered) return launch_rowblock_t<SR, true, true>(ctx, A, sr, flt);
    return launch_rowblock_t<SR, false, true>(ctx, A, sr, flt);
  }
  if (filtered) return launch_rowblock_t<SR, true, false>(ctx, A, sr, flt);
  return launch_rowblock_t<SR, false, false>(ctx, A, sr, flt);
}

template <int TC>
static int spmv_generic(gg_ctx* ctx, gg_mat* A, int mul, int add, int accum, void* y, int ty,
                        const void* x, int tx, const void* mask, int tmask, int64_t lo,
                        int64_t hi) {
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
  const int64_t m = A->m;
  if (A->format == GG_FMT_SELL) {
    sr.has_absorb = false;  // the SELL kernels never stop early (SELL.jl:54-60)
    int64_t s_lo = 0, s_hi = m;
    if (lo > 0) {
      // stored rows of original rows lo..hi lie in the sigma windows covering them
      const int64_t w = A->sigma > 1 ? A->sigma : 1;
      s_lo = ((lo - 1) / w) * w;
      s_hi = ((hi + w - 1) / w) * w;
      if (s_hi > m) s_hi = m;
    }
    if (s_hi <= s_lo) return GG_OK;
    k_sell<SRGen<TC>><<<grid_for(ctx, s_hi - s_lo, 256), 256, 0, ctx->stream>>>(
        sr, A->slice_ptr, A->colval, A->sigma > 1 ? A->perm : nullptr, A->slice_size, s_lo, s_hi,
        lo, hi, mask, tmask);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  const int G = group_width(A);
  if (add == GG_OP_ANY && mask != nullptr && lo == 0) {
    k_csr_first_hit<TC><<<grid_for(ctx, m * G, 256), 256, 0, ctx->stream>>>(
        sr, A->rowptr, A->colval, m, mask, tmask, G);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  return launch_rowblock(ctx, A, sr, mask, tmask, lo, hi, mul == GG_OP_FIRSTI);
}

// dispatch of gg_spmv after validation (gg_api.cu); tc = accumulator type
int spmv_dispatch(gg_ctx* ctx, gg_mat* A, int tc, int mul, int add, int accum, void* y, int ty,
                  const void* x, int tx, const void* mask, int tmask, int64_t lo, int64_t hi) {
  if (A->m == 0) return GG_OK;
  const bool plain = (mask == nullptr && lo == 0);
  if (plain && A->dtype == GG_FLOAT32 && tx == GG_FLOAT32 && ty == GG_FLOAT32 &&
      mul == GG_OP_MUL && add == GG_OP_ADD && accum == GG_OP_SECOND) {
    SRPlusTimesF32 sr;
    sr.nz = static_cast<const float*>(A->nzval);
    sr.x = static_cast<const float*>(x);
    sr.y = static_cast<float*>(y);
    if (A->format == GG_FMT_CSR) return launch_rowblock(ctx, A, sr);
    k_sell<SRPlusTimesF32><<<grid_for(ctx, A->m, 256), 256, 0, ctx->stream>>>(
        sr, A->slice_ptr, A->colval, A->sigma > 1 ? A->perm : nullptr, A->slice_size, 0, A->m, 0,
        0, nullptr, 0);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  switch (tc) {
    case GG_BOOL: return spmv_generic<GG_BOOL>(ctx, A, mul, add, accum, y, ty, x, tx, mask, tmask, lo, hi);
    case GG_INT32: return spmv_generic<GG_INT32>(ctx, A, mul, add, accum, y, ty, x, tx, mask, tmask, lo, hi);
    case GG_INT64: return spmv_generic<GG_INT64>(ctx, A, mul, add, accum, y, ty, x, tx, mask, tmask, lo, hi);
    case GG_FLOAT32: return spmv_generic<GG_FLOAT32>(ctx, A, mul, add, accum, y, ty, x, tx, mask, tmask, lo, hi);
    default: return spmv_generic<GG_FLOAT64>(ctx, A, mul, add, accum, y, ty, x, tx, mask, tmask, lo, hi);
  }
}

}  // namespace gg
