// gg_spmv.cu -- semiring SpMV over CSR and SELL (gpu_spmv!, src/spmv/CSR.jl and
// src/spmv/SELL.jl of GPUGraphs.jl).
//
// Kernels
//  * k_csr_rowblock<SR>: any semiring / element type, optional row filter (mask,
//    range).  Short rows (<= 32 entries) are grouped into blocks of <= 256 entries;
//    one warp computes mul(A[k], x[col[k]]) for a block with coalesced loads into
//    shared memory, then every lane folds one row from shared memory in storage
//    order -- the reference's sequential order, so these rows are bit-identical to
//    it, early exit included.  Longer rows are reduced by one warp per segment
//    (<= 4096 entries; lane partials + shuffle tree); for rows of several segments
//    the warp that finishes the last one combines the partials in order.  Mask and
//    range variants use the same kernel with a row filter.
//  * k_spmv_pipe<SR>: the same work items for the fixed-type plus-times Float32
//    semiring, software pipelined (next block's loads in flight during the current
//    block's gathers), A streamed past L1, long segments read with 128-bit loads.
//    Used for CSR matrices of fewer than 65536 rows; larger ones run plus-times on a
//    SELL-32 copy with rows sorted by length (built once per matrix).
//  * k_csr_first_hit<TC>: add == GPUGraphs_any with a mask on CSR: the first stored
//    column whose x is nonzero (any_dense_masked_csr_spmv_kernel!, CSR.jl:147-171).
//  * k_sell<SR>: one thread per (stored SELL row, chunk of <= 128 slice columns)
//    walking with stride C (slice-column-major, so a warp reads C consecutive
//    words), stopping at the first -1 padding column like sell_spmv_kernel!
//    (SELL.jl:31-63); rows of multi-chunk slices are combined by k_sell_combine.
//  * k_sell_hot: the same for plus-times Float32 over frequency-relabelled columns,
//    with the 32768 most gathered x values in shared memory.
#include <algorithm>
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
template <typename T>
__device__ __forceinline__ T shfl_idx_m(unsigned mask, T v, int src) {
  return __shfl_sync(mask, v, src);
}
template <>
__device__ __forceinline__ uint8_t shfl_idx_m<uint8_t>(unsigned mask, uint8_t v, int src) {
  return static_cast<uint8_t>(__shfl_sync(mask, static_cast<int>(v), src));
}
template <>
__device__ __forceinline__ uint8_t shfl_xor_m<uint8_t>(unsigned mask, uint8_t v, int off,
                                                       int width) {
  return static_cast<uint8_t>(__shfl_xor_sync(mask, static_cast<int>(v), off, width));
}

// ---------------------------------------------------------------------------------
// storage-order refold with the reference's early exit (csr_spmv_kernel!,
// src/spmv/CSR.jl:47-52) for rows reduced in parallel
//
// A parallel (tree-ordered) fold of a floating-point row differs from the sequential
// fold with its stop at the absorbing value only through NaN: a NaN or -Inf term
// after the sum reached +Inf (GPUGraphs_add), or a NaN after -Inf / +Inf (min /
// max).  Without the stop those give NaN; any other non-finite or finite result is
// the same.  So a row whose parallel result is NaN is folded again, by the whole
// warp: lanes compute 32 products at once (coalesced loads) and the sum is taken in
// storage order through shuffles, stopping where the reference stops.  Integer and
// Bool accumulators never compare unequal to themselves, so they skip this.
// ---------------------------------------------------------------------------------
template <class SR>
__device__ __forceinline__ typename SR::T warp_refold_row(const SR& sr, const int32_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ colval,
                                                          int64_t row0, int lane) {
  typedef typename SR::T T;
  const int32_t kb = __ldg(rowptr + row0) - 1, ke = __ldg(rowptr + row0 + 1) - 1;
  T acc = sr.neutral();
  bool done = false;
  for (int32_t base = kb; base < ke && !done; base += 32) {
    const int32_t k = base + lane;
    T p = sr.neutral();
    if (k < ke) p = sr.mulk(k, __ldg(colval + k), row0 + 1);
    const int cnt = ke - base < 32 ? ke - base : 32;
    for (int j = 0; j < cnt; ++j) {
      acc = sr.addv(acc, shfl_idx_m<T>(kFull, p, j));
      if (sr.is_absorb(acc)) {
        done = true;
        break;
      }
    }
  }
  return acc;
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
                   const int4* __restrict__ blocks, int64_t nblocks, const int4* __restrict__ segs,
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
      const int4 b = blocks[item];
      if (kFiltered && (b.y <= flt.lo || b.x >= flt.hi)) continue;
      const int32_t k0 = b.z, k1 = b.w;
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
      const int4 sg = segs[si];  // partial slot, k_begin, k_end, long-row index
      const int32_t row = long_rows[sg.w];
      if (kFiltered && !flt.keep(row)) continue;
      T acc = sr.neutral();
      for (int32_t base = sg.y; base < sg.z; base += 32 * 4) {
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int32_t k = base + u * 32 + lane;
          v[u] = (k < sg.z) ? sr.mulk(k, __ldcs(colval + k), row + 1) : sr.neutral();
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) acc = sr.addv(acc, v[u]);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc = sr.addv(acc, shfl_xor_m<T>(kFull, acc, off, 32));
      const int32_t f0 = long_first_seg[sg.w], f1 = long_first_seg[sg.w + 1];
      if (f1 - f0 == 1) {  // the whole row in one segment
        if (acc != acc) acc = warp_refold_row(sr, rowptr, colval, row, lane);
        if (lane == 0) sr.write(row, acc);
        continue;
      }
      unsigned prev = 0;
      if (lane == 0) {
        partials[sg.x] = acc;
        __threadfence();
        prev = atomicAdd(long_count + sg.w, 1u);
      }
      prev = __shfl_sync(kFull, prev, 0);
      if (prev == (unsigned)(f1 - f0 - 1)) {  // this warp completed the row
        __threadfence();
        T tot = sr.neutral();
        if (lane == 0) {
          for (int32_t q = f0; q < f1; ++q) tot = sr.addv(tot, __ldcg(partials + q));
          long_count[sg.w] = 0;  // ready for the next launch
        }
        tot = shfl_idx_m<T>(kFull, tot, 0);
        if (tot != tot) tot = warp_refold_row(sr, rowptr, colval, row, lane);
        if (lane == 0) sr.write(row, tot);
      }
    }
  }
}

// ---------------------------------------------------------------------------------
// pipelined row-block kernel for fixed-type semirings (no mask / range)
//
// Same work items as k_csr_rowblock, with the memory chain shortened and overlapped:
// block descriptors carry their entry range; each warp issues the column / value
// loads of its next block before gathering x for the current one, and prefetches
// the rowptr pair of the current block's first 32 rows.  Long-row segments are read
// with 128-bit loads, double buffered.  Rows of regular blocks are still folded in
// storage order.
// ---------------------------------------------------------------------------------
static const int kPipeWarps = 8;
static const int kPU = kBlockNnz / 32;  // entries per lane of a regular block

template <class SR>
struct BlockRegs {
  int32_t col[kPU];
  float val[kPU];
  int32_t rp0, rp1;  // rowptr[r0 + lane], rowptr[r0 + lane + 1]
};

template <class SR>
__device__ __forceinline__ void load_block(const SR& sr, const int32_t* __restrict__ rowptr,
                                           const int32_t* __restrict__ colval, const int4& d,
                                           int lane, BlockRegs<SR>& R) {
#pragma unroll
  for (int u = 0; u < kPU; ++u) {
    const int32_t k = d.z + u * 32 + lane;
    if (k < d.w) {
      R.col[u] = ld_stream(colval + k);
      R.val[u] = sr.a(k);
    }
  }
  if (d.x + lane < d.y) {
    R.rp0 = __ldg(rowptr + d.x + lane);
    R.rp1 = __ldg(rowptr + d.x + lane + 1);
  }
}

template <class SR>
__global__ void __launch_bounds__(kPipeWarps * 32)
    k_spmv_pipe(SR sr, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colval,
                const int4* __restrict__ blocks, int64_t nblocks, const int4* __restrict__ segs,
                int64_t nsegs, const int32_t* __restrict__ long_first_seg,
                const int32_t* __restrict__ long_rows, unsigned int* long_count,
                typename SR::T* partials) {
  typedef typename SR::T T;
  __shared__ T stage[kPipeWarps][kBlockNnz];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * kPipeWarps;
  const int64_t gw = (int64_t)blockIdx.x * kPipeWarps + warp;
  T* st = stage[warp];
  const int4 empty = make_int4(0, 0, 0, 0);

  // ---- regular blocks ----
  int64_t it = gw;
  int4 dc = it < nblocks ? blocks[it] : empty;
  int4 dn = it + nw < nblocks ? blocks[it + nw] : empty;
  BlockRegs<SR> cur, nxt;
  load_block(sr, rowptr, colval, dc, lane, cur);
  while (it < nblocks) {
    const int64_t itn = it + nw;
    const int4 dnn = itn + nw < nblocks ? blocks[itn + nw] : empty;
    // gathers for the current block (its columns are already in registers)
    T p[kPU];
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      const int32_t k = dc.z + u * 32 + lane;
      if (k < dc.w) p[u] = sr.mul(cur.val[u], sr.xg(cur.col[u]));
    }
    // loads of the next block go out while the gathers are in flight
    load_block(sr, rowptr, colval, dn, lane, nxt);
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      const int32_t k = dc.z + u * 32 + lane;
      if (k < dc.w) st[u * 32 + lane] = p[u];
    }
    __syncwarp();
    for (int32_t r = dc.x + lane; r < dc.y; r += 32) {
      const int32_t s = (r == dc.x + lane ? cur.rp0 : __ldg(rowptr + r)) - 1 - dc.z;
      const int32_t e = (r == dc.x + lane ? cur.rp1 : __ldg(rowptr + r + 1)) - 1 - dc.z;
      // Fold in storage order.  Without NaN / -Inf terms, a sum that reaches +Inf
      // stays +Inf, which equals the reference's stop at the absorbing +Inf
      // (CSR.jl:49-51); a NaN result is folded again with that stop.
      T acc = sr.neutral();
#pragma unroll 4
      for (int32_t i = s; i < e; ++i) acc = sr.addv(acc, st[i]);
      if (acc != acc) {
        acc = sr.neutral();
        for (int32_t i = s; i < e; ++i) {
          acc = sr.addv(acc, st[i]);
          if (sr.is_absorb(acc)) break;
        }
      }
      sr.write(r, acc);
    }
    __syncwarp();
    it = itn;
    dc = dn;
    dn = dnn;
    cur = nxt;
  }

  // ---- long-row segments: 128-bit loads, next chunk prefetched ----
  for (int64_t si = gw; si < nsegs; si += nw) {
    const int4 sg = segs[si];  // partial slot, k_begin, k_end, long-row index
    const int32_t row = long_rows[sg.w];
    T acc = sr.neutral();
    const int32_t kb = sg.y, ke = sg.z;
    int32_t ka = (kb + 3) & ~3;  // first 16-byte aligned entry
    if (ka > ke) ka = ke;
    if (kb + lane < ka) acc = sr.addv(acc, sr.mul(sr.a(kb + lane), sr.xg(ld_stream(colval + kb + lane))));
    // body in chunks of 256 entries: 2 x (int4 + float4) per lane
    int32_t k = ka;
    const int32_t kend = ka + ((ke - ka) & ~255);
    int4 c0, c1;
    float4 v0, v1;
    if (k < kend) {
      c0 = ld_stream4(colval + k + lane * 4);
      c1 = ld_stream4(colval + k + 128 + lane * 4);
      v0 = sr.a4(k + lane * 4);
      v1 = sr.a4(k + 128 + lane * 4);
    }
    while (k < kend) {
      const int32_t kn = k + 256;
      int4 nc0 = c0, nc1 = c1;
      float4 nv0 = v0, nv1 = v1;
      if (kn < kend) {
        nc0 = ld_stream4(colval + kn + lane * 4);
        nc1 = ld_stream4(colval + kn + 128 + lane * 4);
        nv0 = sr.a4(kn + lane * 4);
        nv1 = sr.a4(kn + 128 + lane * 4);
      }
      const float x0 = sr.xg(c0.x), x1 = sr.xg(c0.y), x2 = sr.xg(c0.z), x3 = sr.xg(c0.w);
      const float x4 = sr.xg(c1.x), x5 = sr.xg(c1.y), x6 = sr.xg(c1.z), x7 = sr.xg(c1.w);
      acc = sr.addv(acc, sr.mul(v0.x, x0));
      acc = sr.addv(acc, sr.mul(v0.y, x1));
      acc = sr.addv(acc, sr.mul(v0.z, x2));
      acc = sr.addv(acc, sr.mul(v0.w, x3));
      acc = sr.addv(acc, sr.mul(v1.x, x4));
      acc = sr.addv(acc, sr.mul(v1.y, x5));
      acc = sr.addv(acc, sr.mul(v1.z, x6));
      acc = sr.addv(acc, sr.mul(v1.w, x7));
      c0 = nc0; c1 = nc1; v0 = nv0; v1 = nv1;
      k = kn;
    }
    for (int32_t kk = kend + lane; kk < ke; kk += 32)
      acc = sr.addv(acc, sr.mul(sr.a(kk), sr.xg(ld_stream(colval + kk))));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc = sr.addv(acc, shfl_xor_m<T>(kFull, acc, off, 32));
    const int32_t f0 = long_first_seg[sg.w], f1 = long_first_seg[sg.w + 1];
    if (f1 - f0 == 1) {  // the whole row in one segment
      if (acc != acc) acc = warp_refold_row(sr, rowptr, colval, row, lane);
      if (lane == 0) sr.write(row, acc);
      continue;
    }
    unsigned prev = 0;
    if (lane == 0) {
      partials[sg.x] = acc;
      __threadfence();
      prev = atomicAdd(long_count + sg.w, 1u);
    }
    prev = __shfl_sync(kFull, prev, 0);
    if (prev == (unsigned)(f1 - f0 - 1)) {
      __threadfence();
      T tot = sr.neutral();
      if (lane == 0) {
        for (int32_t q = f0; q < f1; ++q) tot = sr.addv(tot, __ldcg(partials + q));
        long_count[sg.w] = 0;
      }
      tot = __shfl_sync(kFull, tot, 0);
      if (tot != tot) tot = warp_refold_row(sr, rowptr, colval, row, lane);
      if (lane == 0) sr.write(row, tot);
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
// SELL: one thread per (stored row, chunk of its slice).  Every thread walks at most
// kSellChunk columns with stride C, so hub slices no longer serialise on one thread;
// a row spread over several chunks is combined in chunk order by k_sell_combine.
// ---------------------------------------------------------------------------------
template <class SR>
__global__ void k_sell(SR sr, const int32_t* __restrict__ slice_ptr,
                       const int32_t* __restrict__ colval, const int32_t* __restrict__ perm,
                       int64_t C, int64_t m, const int4* __restrict__ items, int64_t nitems,
                       typename SR::T* partials, int64_t range_lo, int64_t range_hi,
                       const void* mask, int tmask) {
  typedef typename SR::T T;
  const int64_t total = nitems * C;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t it = t / C, o = t - it * C;
    const int4 d = items[it];  // slice, first column, end column, partial index
    const int64_t srow = (int64_t)d.x * C + o;
    if (srow >= m) continue;
    const int64_t r1 = perm ? (int64_t)perm[srow] : srow + 1;  // original row, 1-based
    if (range_lo > 0 && (r1 < range_lo || r1 > range_hi)) continue;
    if (mask && raw_is_zero(load_raw(mask, tmask, r1 - 1), tmask)) continue;
    int64_t i = (int64_t)slice_ptr[d.x] - 1 + o + (int64_t)d.y * C;
    T acc = sr.neutral();
    int32_t j = d.y;
    bool done = false;
    for (; j + 8 <= d.z && !done; j += 8, i += 8 * C) {
      int32_t c[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) c[u] = ld_stream(colval + i + u * C);
      T p[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) p[u] = (c[u] != -1) ? sr.mulk(i + u * C, c[u], r1) : sr.neutral();
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (c[u] == -1) { done = true; break; }
        acc = sr.addv(acc, p[u]);
      }
    }
    for (; j < d.z && !done; ++j, i += C) {
      const int32_t col = ld_stream(colval + i);
      if (col == -1) break;
      acc = sr.addv(acc, sr.mulk(i, col, r1));
    }
    if (d.w < 0) sr.write(r1 - 1, acc);
    else partials[(int64_t)d.w * C + o] = acc;
  }
}

// one warp per (multi-chunk slice, row): lanes fold the chunk partials lane-strided,
// then a shuffle tree.  A row of <= kSellChunk entries has one non-neutral partial,
// so its value is unchanged (x + 0 == x; the partials are never -0.0).
template <class SR>
__global__ void k_sell_combine(SR sr, const int32_t* __restrict__ perm, int64_t C, int64_t m,
                               const int4* __restrict__ multi, int64_t nmulti,
                               const typename SR::T* __restrict__ partials, int64_t range_lo,
                               int64_t range_hi, const void* mask, int tmask) {
  typedef typename SR::T T;
  const int lane = threadIdx.x & 31;
  const int64_t total = nmulti * C;
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < total;
       t += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t q = t / C, o = t - q * C;
    const int4 d = multi[q];  // slice, first partial, chunks
    const int64_t srow = (int64_t)d.x * C + o;
    if (srow >= m) continue;
    const int64_t r1 = perm ? (int64_t)perm[srow] : srow + 1;
    if (range_lo > 0 && (r1 < range_lo || r1 > range_hi)) continue;
    if (mask && raw_is_zero(load_raw(mask, tmask, r1 - 1), tmask)) continue;
    T acc = sr.neutral();
    for (int32_t c = lane; c < d.z; c += 32) acc = sr.addv(acc, partials[(int64_t)(d.y + c) * C + o]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc = sr.addv(acc, shfl_xor_m<T>(kFull, acc, off, 32));
    if (lane == 0) sr.write(r1 - 1, acc);
  }
}

// ---------------------------------------------------------------------------------
// SELL plus-times Float32 over relabelled columns with the hot part of x in shared
// memory.  After relabelling by frequency, columns 1..hot are the most gathered
// ones (about half of the entries of an R-MAT graph fall in the first 32768); each
// CTA stages them once and serves those gathers from shared memory, so the L1 tag
// stage -- one distinct line per cycle, the limit of scattered gathers -- sees only
// the cold ones.  Same work items and fold order as k_sell.
// ---------------------------------------------------------------------------------
static const int kHotCols = 32768;     // default hot x values in shared memory
static const int kHotColsMax = 53248;  // 208 KB: the most a 1024-thread CTA may stage
static const int kHotThreads = 1024;

__global__ void __launch_bounds__(kHotThreads, 1)
    k_sell_hot(const float* __restrict__ nz, const float* __restrict__ xr, float* __restrict__ y,
               const int32_t* __restrict__ slice_ptr, const int32_t* __restrict__ colval,
               const int32_t* __restrict__ perm, int64_t C, int64_t m,
               const int4* __restrict__ items, int64_t nitems, float* partials, int hot) {
  extern __shared__ float sx[];
  for (int i = threadIdx.x; i < hot; i += blockDim.x) sx[i] = __ldg(xr + i);
  __syncthreads();
  const int64_t total = nitems * C;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t it = t / C, o = t - it * C;
    const int4 d = items[it];  // slice, first column, end column, partial index
    const int64_t srow = (int64_t)d.x * C + o;
    if (srow >= m) continue;
    const int64_t r1 = perm ? (int64_t)perm[srow] : srow + 1;
    // positions fit in Int32 (n_stored < 2^31 is checked when the SELL copy is built)
    const int32_t Ci = (int32_t)C;
    int32_t pos = slice_ptr[d.x] - 1 + (int32_t)o + d.y * Ci;  // entry (row o, column j)
    // Padding columns (-1) contribute +0.0, which leaves the sum unchanged (the sum
    // starts at +0.0 and is never -0.0), so the row is folded in storage order with
    // no early exit; column / value loads of the next 8 entries are issued before the
    // gathers of the current 8.
    float acc = 0.0f;
    int32_t c[8];
    float a[8];
    int32_t j = d.y;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool in = j + u < d.z;
      c[u] = in ? ld_stream(colval + pos + u * Ci) : -1;
      a[u] = in ? ld_stream(nz + pos + u * Ci) : 0.0f;
    }
    while (j < d.z) {
      const int32_t jn = j + 8;
      const int32_t pn = pos + 8 * Ci;
      int32_t cn[8];
      float an[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = jn + u < d.z;
        cn[u] = in ? ld_stream(colval + pn + u * Ci) : -1;
        an[u] = in ? ld_stream(nz + pn + u * Ci) : 0.0f;
      }
      float p[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int32_t col = c[u];
        float xv = 0.0f;
        if (col > 0) xv = col <= hot ? sx[col - 1] : __ldg(xr + (col - 1));
        p[u] = __fmul_rn(a[u], xv);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) acc = __fadd_rn(acc, p[u]);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        c[u] = cn[u];
        a[u] = an[u];
      }
      j = jn;
      pos = pn;
    }
    if (d.w < 0) __stcs(y + (r1 - 1), acc);
    else partials[(int64_t)d.w * C + o] = acc;
  }
}

void free_sell_plan(SellPlan* P) {
  if (!P) return;
  cudaFree(P->items);
  cudaFree(P->multi);
  cudaFree(P->partials);
  cudaFree(P->pitems);
  cudaFree(P->narrow);
  cudaFree(P->wide);
  cudaFree(P->pitems256);
  cudaFree(P->multi256);
  delete P;
}

int build_sell_plan(gg_ctx* ctx, gg_mat* A) {
  if (A->sellplan) return GG_OK;
  return build_sell_plan_from(ctx, A, 0, &A->sellplan);
}

// work items of the slices s0, s0 + 1, ... (s0 > 0: the rows before slice s0 are
// computed elsewhere, e.g. the hub rows of gg_spmv_hub.cu)
int build_sell_plan_from(gg_ctx* ctx, const gg_mat* A, int64_t s0, SellPlan** out) {
  const int64_t ns = A->nslices, C = A->slice_size;
  std::vector<int32_t> sp(ns + 1);
  GG_CUDA(cudaMemcpyAsync(sp.data(), A->slice_ptr, (ns + 1) * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int4> items, multi, pitems, narrow, wide;
  int32_t np = 0;
  // narrow-slice groups of the warp kernel (C == 32 only)
  int64_t g_first = -1, g_cols = 0, g_count = 0;
  uint32_t g_widths = 0;
  auto flush_group = [&]() {
    if (g_count > 0)
      pitems.push_back(make_int4(sp[g_first] - 1, (int)(g_first * C), -(int)g_count, (int)g_widths));
    g_first = -1;
    g_cols = 0;
    g_count = 0;
    g_widths = 0;
  };
  for (int64_t s = s0; s < ns; ++s) {
    const int64_t L = C > 0 ? ((int64_t)sp[s + 1] - sp[s]) / C : 0;
    if (C == 32 && L <= kNarrowCols) {
      if (g_count == 8 || g_cols + L > kNarrowCols) flush_group();
      if (g_count == 0) g_first = s;
      g_widths |= (uint32_t)L << (4 * g_count);
      g_cols += L;
      ++g_count;
    } else {
      flush_group();
    }
    if (L <= kSellChunk) {
      items.push_back(make_int4((int)s, 0, (int)L, -1));
      if (!(C == 32 && L <= kNarrowCols)) pitems.push_back(make_int4(sp[s] - 1, (int)(s * C), (int)L, -1));
      continue;
    }
    const int32_t nch = (int32_t)((L + kSellChunk - 1) / kSellChunk);
    (nch <= kNarrowChunks ? narrow : wide).push_back(make_int4((int)s, np, nch, 0));
    multi.push_back(make_int4((int)s, np, nch, 0));
    for (int32_t c = 0; c < nch; ++c) {
      const int64_t jb = (int64_t)c * kSellChunk;
      const int64_t je = jb + kSellChunk < L ? jb + kSellChunk : L;
      items.push_back(make_int4((int)s, (int)jb, (int)je, np + c));
      pitems.push_back(make_int4((int)(sp[s] - 1 + jb * C), (int)(s * C), (int)(je - jb), np + c));
    }
    np += nch;
  }
  flush_group();
  SellPlan* P = new SellPlan();
  P->npitems = (int64_t)pitems.size();
  P->nitems = (int64_t)items.size();
  P->nmulti = (int64_t)multi.size();
  P->nnarrow = (int64_t)narrow.size();
  P->nwide = (int64_t)wide.size();
  cudaError_t e = cudaMalloc((void**)&P->items, (items.size() + 1) * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->multi, (multi.size() + 1) * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc(&P->partials, ((int64_t)np * C + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->pitems, (pitems.size() + 1) * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->narrow, (narrow.size() + 1) * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->wide, (wide.size() + 1) * sizeof(int4));
  if (e == cudaSuccess && !narrow.empty())
    e = cudaMemcpyAsync(P->narrow, narrow.data(), narrow.size() * sizeof(int4), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess && !wide.empty())
    e = cudaMemcpyAsync(P->wide, wide.data(), wide.size() * sizeof(int4), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess && !pitems.empty())
    e = cudaMemcpyAsync(P->pitems, pitems.data(), pitems.size() * sizeof(int4),
                        cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && !items.empty())
    e = cudaMemcpyAsync(P->items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess && !multi.empty())
    e = cudaMemcpyAsync(P->multi, multi.data(), multi.size() * sizeof(int4), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    free_sell_plan(P);
    return cuda_error(e, "SELL analysis");
  }
  *out = P;
  return GG_OK;
}

template <class SR>
static int launch_sell(gg_ctx* ctx, gg_mat* A, const SR& sr, const void* mask, int tmask,
                       int64_t lo, int64_t hi, const int32_t* colval_override = nullptr);

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
  std::vector<int4> blocks;
  std::vector<int4> segs;
  std::vector<int32_t> first_seg, long_rows;
  blocks.reserve(m / 8 + 16);
  const int64_t max_rows = A->block_rows > 0 ? A->block_rows : kBlockRows;
  int64_t r = 0;
  while (r < m) {
    int64_t len = rp[r + 1] - rp[r];
    if (len > kShortRow) {
      int32_t li = (int32_t)long_rows.size();
      long_rows.push_back((int32_t)r);
      first_seg.push_back((int32_t)segs.size());
      for (int64_t kb = rp[r] - 1; kb < rp[r + 1] - 1; kb += kSegNnz) {
        int64_t ke = kb + kSegNnz < rp[r + 1] - 1 ? kb + kSegNnz : rp[r + 1] - 1;
        segs.push_back(make_int4((int)segs.size(), (int)kb, (int)ke, li));
      }
      ++r;
      continue;
    }
    int64_t first = r, cnt = 0;
    while (r < m && r - first < max_rows) {
      int64_t l = rp[r + 1] - rp[r];
      if (l > kShortRow || cnt + l > kBlockNnz) break;
      cnt += l;
      ++r;
    }
    blocks.push_back(make_int4((int)first, (int)r, rp[first] - 1, rp[r] - 1));
  }
  first_seg.push_back((int32_t)segs.size());
  // largest segments first: with the kernels' round-robin assignment this balances
  // the warps (longest-processing-time order); partial slots stay in row order
  std::stable_sort(segs.begin(), segs.end(),
                   [](const int4& a, const int4& b) { return (a.z - a.y) > (b.z - b.y); });

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
  up((void**)&rb->blocks, blocks.data(), blocks.size() * sizeof(int4));
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
  static int per_sm = 0;
  if (per_sm == 0) {
    GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, k_csr_rowblock<SR, kFiltered, kNeedsRow>, kRBWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
  }
  int64_t grid = (items + kRBWarps - 1) / kRBWarps;
  const int64_t cap = (int64_t)ctx->num_sms * per_sm;  // one resident wave
  if (grid > cap) grid = cap;
  const int tr = trace_main_begin(ctx);
  k_csr_rowblock<SR, kFiltered, kNeedsRow><<<(int)grid, kRBWarps * 32, 0, ctx->stream>>>(
      sr, A->rowptr, A->colval, rb->blocks, rb->nblocks, rb->segs, rb->nsegs, rb->long_first_seg,
      rb->long_rows, rb->long_count, static_cast<typename SR::T*>(rb->partials), flt);
  trace_main_end(ctx, tr);
  trace_count(ctx, 1);
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
    return launch_sell(ctx, A, sr, mask, tmask, lo, hi);
  }
  const int G = group_width(A);
  if (add == GG_OP_ANY && mask != nullptr && lo == 0) {
    const int tr = trace_main_begin(ctx);
    k_csr_first_hit<TC><<<grid_for(ctx, m * G, 256), 256, 0, ctx->stream>>>(
        sr, A->rowptr, A->colval, m, mask, tmask, G);
    trace_main_end(ctx, tr);
    trace_count(ctx, 1);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  return launch_rowblock(ctx, A, sr, mask, tmask, lo, hi, mul == GG_OP_FIRSTI);
}

// ---------------------------------------------------------------------------------
// column relabelling by frequency (plus-times Float32 path)
// ---------------------------------------------------------------------------------
__global__ void k_col_count(const int32_t* __restrict__ colval, int64_t len, int32_t* cnt) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < len;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = colval[k];
    if (c > 0) atomicAdd(cnt + (c - 1), 1);
  }
}

__global__ void k_col_relabel(const int32_t* __restrict__ colval, int64_t len,
                              const int32_t* __restrict__ rank, int32_t* out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < len;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = colval[k];
    out[k] = c > 0 ? rank[c - 1] + 1 : c;
  }
}

__global__ void k_gather_x(const float* __restrict__ x, const int32_t* __restrict__ inv,
                           int64_t n, float* xr) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    xr[i] = __ldg(x + inv[i]);
}

// Builds the relabelling once per matrix.  It is kept only when the column
// frequencies are skewed (the 1% most frequent columns hold over a quarter of the
// entries) and x is larger than L1 could hold anyway; otherwise the natural order
// (e.g. the locality of a grid) is better.
static int build_colperm(gg_ctx* ctx, gg_mat* A) {
  if (A->colperm) return GG_OK;
  ColPerm* P = new ColPerm();
  A->colperm = P;
  const int64_t n = A->n;
  const int64_t len = A->format == GG_FMT_CSR ? A->nnz : A->n_stored;
  if (n < (1 << 16) || A->nnz == 0) return GG_OK;
  int32_t* cnt = nullptr;
  GG_CUDA(cudaMalloc((void**)&cnt, n * sizeof(int32_t)));
  GG_CUDA(cudaMemsetAsync(cnt, 0, n * sizeof(int32_t), ctx->stream));
  k_col_count<<<grid_for(ctx, len, 256), 256, 0, ctx->stream>>>(A->colval, len, cnt);
  std::vector<int32_t> hc(n);
  cudaError_t e = cudaMemcpyAsync(hc.data(), cnt, n * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(cnt);
    return cuda_error(e, "column counts");
  }
  std::vector<uint64_t> key(n);
  for (int64_t c = 0; c < n; ++c) key[c] = ((uint64_t)(uint32_t)(~(uint32_t)hc[c]) << 32) | (uint64_t)c;
  std::sort(key.begin(), key.end());
  int64_t top = 0;
  const int64_t ntop = n / 100;
  for (int64_t i = 0; i < ntop; ++i) top += hc[key[i] & 0xffffffffu];
  if (top * 4 <= A->nnz) {  // not skewed: keep the natural column order
    cudaFree(cnt);
    return GG_OK;
  }
  std::vector<int32_t> inv(n), rank(n);
  for (int64_t i = 0; i < n; ++i) {
    inv[i] = (int32_t)(key[i] & 0xffffffffu);
    rank[inv[i]] = (int32_t)i;
  }
  e = cudaMemcpyAsync(cnt, rank.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->colval_r, (len > 0 ? len : 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->inv, n * sizeof(int32_t));
  // xr padded with zeros to whole column windows (the bulk copies of gg_spmv_hub.cu
  // read complete windows)
  const int64_t npad = (n + kHwCols - 1) / kHwCols * kHwCols;
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->xr, npad * sizeof(float));
  if (e == cudaSuccess && npad > n)
    e = cudaMemsetAsync(P->xr + n, 0, (npad - n) * sizeof(float), ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->inv, inv.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    k_col_relabel<<<grid_for(ctx, len, 256), 256, 0, ctx->stream>>>(A->colval, len, cnt, P->colval_r);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(cnt);
  if (e != cudaSuccess) return cuda_error(e, "column relabelling");
  P->enabled = true;
  return GG_OK;
}

template <class SR>
static int launch_sell(gg_ctx* ctx, gg_mat* A, const SR& sr, const void* mask, int tmask,
                       int64_t lo, int64_t hi, const int32_t* colval_override) {
  GG_CHECK(build_sell_plan(ctx, A));
  SellPlan* P = A->sellplan;
  const int64_t C = A->slice_size;
  typedef typename SR::T T;
  if (P->nitems > 0) {
    const int tr = trace_main_begin(ctx);
    k_sell<SR><<<grid_for(ctx, P->nitems * C, 256), 256, 0, ctx->stream>>>(
        sr, A->slice_ptr, colval_override ? colval_override : A->colval,
        A->sigma > 1 ? A->perm : nullptr, C, A->m, P->items,
        P->nitems, static_cast<T*>(P->partials), lo, hi, mask, tmask);
    trace_main_end(ctx, tr);
    trace_count(ctx, 1);
  }
  if (P->nmulti > 0) {
    k_sell_combine<SR><<<grid_for(ctx, P->nmulti * C * 32, 256), 256, 0, ctx->stream>>>(
        sr, A->sigma > 1 ? A->perm : nullptr, C, A->m, P->multi, P->nmulti,
        static_cast<const T*>(P->partials), lo, hi, mask, tmask);
    trace_count(ctx, 1);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// Plus-times Float32 combine of SELL-32 slices of at most kNarrowChunks chunks, one
// thread per row, in exactly the order of k_sell_combine: there lane l folds the
// chunks c = l mod 32 (here at most one each) and lane 0 ends with the butterfly
// sum, i.e. a pairwise tree over the lanes' values in bit-reversed lane order.
__global__ void k_sell_combine_narrow(const int4* __restrict__ narrow, int64_t nnarrow,
                                      const float* __restrict__ partials,
                                      const int32_t* __restrict__ perm, int64_t m,
                                      float* __restrict__ y) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnarrow * 32;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int4 d = narrow[t >> 5];  // slice, first partial, chunks
    const int o = (int)(t & 31);
    const int64_t srow = (int64_t)d.x * 32 + o;
    if (srow >= m) continue;
    float v[kNarrowChunks];
#pragma unroll
    for (int c = 0; c < kNarrowChunks; ++c)
      v[c] = c < d.z ? __fadd_rn(0.0f, partials[(int64_t)(d.y + c) * 32 + o]) : 0.0f;
    float stk[5];
    int lvl[5];
    int top = 0;
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      const int l = (int)(__brev((unsigned)k) >> 27);
      float s = l < kNarrowChunks ? v[l] : 0.0f;
      int lv = 0;
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        if (top > 0 && lvl[top - 1] == lv) {
          s = __fadd_rn(stk[top - 1], s);
          --top;
          ++lv;
        }
      }
      stk[top] = s;
      lvl[top] = lv;
      ++top;
    }
    const int32_t r1 = perm ? perm[srow] : (int32_t)(srow + 1);
    __stcs(y + (r1 - 1), stk[0]);
  }
}

// SELL-32 variant: one warp per work item (lane = row of the slice), with the item's
// first position, first stored row, width and partial slot precomputed, and the next
// item's descriptor loaded while the current one runs -- rows of one or two entries
// (most rows of a power-law graph) no longer pay a chain of dependent descriptor
// loads before their first column load.
__global__ void __launch_bounds__(kHotThreads, 1)
    k_sell_hot32(const float* __restrict__ nz, const float* __restrict__ xr, float* __restrict__ y,
                 const int32_t* __restrict__ colval, const int32_t* __restrict__ perm, int64_t m,
                 const int4* __restrict__ pitems, int64_t nitems, float* partials, int hot) {
  extern __shared__ float sx[];
  for (int i = threadIdx.x; i < hot; i += blockDim.x) sx[i] = __ldg(xr + i);
  __syncthreads();
  const uint64_t pol_s = l2_evict_first(), pol_x = l2_evict_last();
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int4 dn = gw < nitems ? __ldg(pitems + gw) : make_int4(0, 0, 0, -1);
  for (int64_t it = gw; it < nitems; it += nw) {
    const int4 d = dn;  // first position, first stored row, columns, partial
    if (it + nw < nitems) dn = __ldg(pitems + it + nw);
    if (d.z < 0) {
      // group of -d.z narrow slices (widths in 4-bit fields of d.w), <= 8 columns in
      // all: load every entry at once, then fold slice by slice in column order
      const int ns = -d.z;
      const uint32_t widths = (uint32_t)d.w;
      int total = 0;
      for (int t = 0; t < ns; ++t) total += (widths >> (4 * t)) & 15u;
      int32_t c[kNarrowCols];
      float a[kNarrowCols];
#pragma unroll
      for (int u = 0; u < kNarrowCols; ++u) {
        const bool in = u < total;
        c[u] = in ? ld_stream_p(colval + d.x + u * 32 + lane, pol_s) : -1;
        a[u] = in ? ld_stream_p(nz + d.x + u * 32 + lane, pol_s) : 0.0f;
      }
      float p[kNarrowCols];
#pragma unroll
      for (int u = 0; u < kNarrowCols; ++u) {
        const int32_t col = c[u];
        float xv = 0.0f;
        if (col > 0) xv = col <= hot ? sx[col - 1] : ld_keep(xr + (col - 1), pol_x);
        p[u] = __fmul_rn(a[u], xv);
      }
      int u0 = 0;
      for (int t = 0; t < ns; ++t) {
        const int w = (int)((widths >> (4 * t)) & 15u);
        float acc = 0.0f;
#pragma unroll
        for (int u = 0; u < kNarrowCols; ++u)
          if (u >= u0 && u < u0 + w) acc = __fadd_rn(acc, p[u]);
        u0 += w;
        const int64_t srow = (int64_t)d.y + t * 32 + lane;
        if (srow < m) {
          const int32_t r1 = perm ? __ldg(perm + srow) : (int32_t)(srow + 1);
          __stcs(y + (r1 - 1), acc);
        }
      }
      continue;
    }
    const int64_t srow = (int64_t)d.y + lane;
    const bool live = srow < m;
    const int32_t r1 = (live && perm) ? __ldg(perm + srow) : (int32_t)(srow + 1);
    int32_t pos = d.x + lane;
    // padding columns (-1) add +0.0: storage-order fold without an early exit
    float acc = 0.0f;
    int32_t c[8];
    float a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool in = live && u < d.z;
      c[u] = in ? ld_stream_p(colval + pos + u * 32, pol_s) : -1;
      a[u] = in ? ld_stream_p(nz + pos + u * 32, pol_s) : 0.0f;
    }
    for (int32_t j = 0; j < d.z; j += 8) {
      const int32_t pn = pos + 8 * 32;
      int32_t cn[8];
      float an[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = live && j + 8 + u < d.z;
        cn[u] = in ? ld_stream_p(colval + pn + u * 32, pol_s) : -1;
        an[u] = in ? ld_stream_p(nz + pn + u * 32, pol_s) : 0.0f;
      }
      float p[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int32_t col = c[u];
        float xv = 0.0f;
        if (col > 0) xv = col <= hot ? sx[col - 1] : ld_keep(xr + (col - 1), pol_x);
        p[u] = __fmul_rn(a[u], xv);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) acc = __fadd_rn(acc, p[u]);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        c[u] = cn[u];
        a[u] = an[u];
      }
      pos = pn;
    }
    if (!live) continue;
    if (d.w < 0) __stcs(y + (r1 - 1), acc);
    else partials[(int64_t)d.w * 32 + lane] = acc;
  }
}

// plus-times Float32 SELL over relabelled columns (k_sell_hot + chunk combination)
static int launch_sell_hot(gg_ctx* ctx, gg_mat* A, const SRPlusTimesF32& sr,
                           const int32_t* colval) {
  GG_CHECK(build_sell_plan(ctx, A));
  const int64_t C = A->slice_size;
  // sell_variant 2 on a SELL-32 layout: the hub rows from shared-memory column windows
  // (gg_spmv_hub.cu) when the analysis found dense enough hub groups; the SELL-32
  // kernel then runs the other rows only
  bool hub = false;
  if (C == 32 && A->sell_variant == 2) {
    GG_CHECK(build_hubwin_plan(ctx, A));
    hub = A->hubwin->enabled;
  }
  SellPlan* P = hub ? A->hubwin->rest : A->sellplan;
  const int hot_cap = A->hot_cols > 0 ? (A->hot_cols < kHotColsMax ? A->hot_cols : kHotColsMax)
                                      : kHotCols;
  const int hot = (int)std::min<int64_t>(A->n, hot_cap);
  static bool attr_set[64] = {false};
  if (ctx->device < 64 && !attr_set[ctx->device]) {
    GG_CUDA(cudaFuncSetAttribute(k_sell_hot, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kHotColsMax * (int)sizeof(float)));
    GG_CUDA(cudaFuncSetAttribute(k_sell_hot32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kHotColsMax * (int)sizeof(float)));
    attr_set[ctx->device] = true;
  }
  if (P->nitems > 0 && C == 32 && A->sell_variant == 1) {
    GG_CHECK(launch_sell_tma(ctx, A, sr.nz, sr.x, sr.y, colval));  // brackets its own kernel
  } else if (P->nitems > 0 || hub) {
    const int tr = trace_main_begin(ctx);
    if (C == 32 && P->npitems > 0)
      k_sell_hot32<<<ctx->num_sms, kHotThreads, hot * sizeof(float), ctx->stream>>>(
          sr.nz, sr.x, sr.y, colval, A->sigma > 1 ? A->perm : nullptr, A->m, P->pitems, P->npitems,
          static_cast<float*>(P->partials), hot);
    else if (C != 32)
      k_sell_hot<<<ctx->num_sms, kHotThreads, hot * sizeof(float), ctx->stream>>>(
          sr.nz, sr.x, sr.y, A->slice_ptr, colval, A->sigma > 1 ? A->perm : nullptr, C, A->m,
          P->items, P->nitems, static_cast<float*>(P->partials), hot);
    if (hub) GG_CHECK(launch_hubwin(ctx, A, sr.x, sr.y));  // counts its own launches
    trace_main_end(ctx, tr);
    trace_count(ctx, P->npitems > 0 || C != 32 ? 1 : 0);
  }
  // SELL-32: narrow chunked slices a thread per row, the wide ones a warp per row
  const bool split = C == 32;
  if (split && P->nnarrow > 0) {
    k_sell_combine_narrow<<<grid_for(ctx, P->nnarrow * 32, 256), 256, 0, ctx->stream>>>(
        P->narrow, P->nnarrow, static_cast<const float*>(P->partials),
        A->sigma > 1 ? A->perm : nullptr, A->m, sr.y);
    trace_count(ctx, 1);
  }
  const int4* cl = split ? P->wide : P->multi;
  const int64_t ncl = split ? P->nwide : P->nmulti;
  if (ncl > 0) {
    k_sell_combine<SRPlusTimesF32><<<grid_for(ctx, ncl * C * 32, 256), 256, 0, ctx->stream>>>(
        sr, A->sigma > 1 ? A->perm : nullptr, C, A->m, cl, ncl,
        static_cast<const float*>(P->partials), 0, 0, nullptr, 0);
    trace_count(ctx, 1);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ---------------------------------------------------------------------------------
// One-column plus-times SpMM y = A x over the SELL-32 copy of a large CSR handle, in
// the SpMM's fold order: a row of at most kSegMM entries is folded in storage order
// from 0; a longer row in pieces of kSegMM entries (its 256-column chunks in the
// slice-column-major copy, since the copy keeps every row's entries in order), each
// folded from 0, then added in order with the stop at +Inf (k_spmm_combine); a piece
// whose fold ends NaN is folded again with that stop.  So the results equal the
// one-column kernels of gg_spmm.cu and every column of the 32-column SpMM bit for bit
// while the loads are those of the headline SpMV (a lane per row, one 128-byte line
// per warp load, the hottest x values in shared memory).
// ---------------------------------------------------------------------------------
static int build_col1_plan(gg_ctx* ctx, gg_mat* S) {
  GG_CHECK(build_sell_plan(ctx, S));
  SellPlan* P = S->sellplan;
  if (P->npitems256 >= 0) return GG_OK;
  const int64_t ns = S->nslices;
  std::vector<int32_t> sp(ns + 1);
  GG_CUDA(cudaMemcpyAsync(sp.data(), S->slice_ptr, (ns + 1) * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int4> pitems, multi;
  int32_t np = 0;
  int64_t g_first = -1, g_cols = 0, g_count = 0;
  uint32_t g_widths = 0;
  auto flush_group = [&]() {
    if (g_count > 0)
      pitems.push_back(make_int4(sp[g_first] - 1, (int)(g_first * 32), -(int)g_count, (int)g_widths));
    g_first = -1;
    g_cols = 0;
    g_count = 0;
    g_widths = 0;
  };
  for (int64_t s = 0; s < ns; ++s) {
    const int64_t L = ((int64_t)sp[s + 1] - sp[s]) / 32;
    if (L <= kNarrowCols) {
      if (g_count == 8 || g_cols + L > kNarrowCols) flush_group();
      if (g_count == 0) g_first = s;
      g_widths |= (uint32_t)L << (4 * g_count);
      g_cols += L;
      ++g_count;
      continue;
    }
    flush_group();
    if (L <= kSegMM) {
      pitems.push_back(make_int4(sp[s] - 1, (int)(s * 32), (int)L, -1));
      continue;
    }
    const int32_t nch = (int32_t)((L + kSegMM - 1) / kSegMM);
    multi.push_back(make_int4((int)(s * 32), np, nch, 0));
    for (int32_t c = 0; c < nch; ++c) {
      const int64_t jb = (int64_t)c * kSegMM;
      const int64_t je = jb + kSegMM < L ? jb + kSegMM : L;
      pitems.push_back(make_int4((int)(sp[s] - 1 + jb * 32), (int)(s * 32), (int)(je - jb), np + c));
    }
    np += nch;
  }
  flush_group();
  cudaError_t e = cudaMalloc((void**)&P->pitems256, (pitems.size() + 1) * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->multi256, (multi.size() + 1) * sizeof(int4));
  if (e == cudaSuccess && !pitems.empty())
    e = cudaMemcpyAsync(P->pitems256, pitems.data(), pitems.size() * sizeof(int4),
                        cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && !multi.empty())
    e = cudaMemcpyAsync(P->multi256, multi.data(), multi.size() * sizeof(int4),
                        cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(P->pitems256);
    cudaFree(P->multi256);
    P->pitems256 = P->multi256 = nullptr;
    return cuda_error(e, "one-column SpMM plan");
  }
  P->npitems256 = (int64_t)pitems.size();
  P->nmulti256 = (int64_t)multi.size();
  P->npart256 = np;
  return GG_OK;
}

// x value of relabelled column col (1-based): shared memory for the hot ones
__device__ __forceinline__ float col1_x(const float* sx, const float* __restrict__ xr, int32_t col,
                                        int hot, uint64_t pol_x) {
  return col <= hot ? sx[col - 1] : ld_keep(xr + (col - 1), pol_x);
}

__global__ void __launch_bounds__(kHotThreads, 1)
    k_col1_sell(const float* __restrict__ nz, const float* __restrict__ xr, float* __restrict__ y,
                const int32_t* __restrict__ colval, const int32_t* __restrict__ perm, int64_t m,
                const int4* __restrict__ pitems, int64_t nitems, float* partials, int hot) {
  extern __shared__ float sx[];
  for (int i = threadIdx.x; i < hot; i += blockDim.x) sx[i] = __ldg(xr + i);
  __syncthreads();
  const uint64_t pol_s = l2_evict_first(), pol_x = l2_evict_last();
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
      float p[kNarrowCols];
#pragma unroll
      for (int u = 0; u < kNarrowCols; ++u) {
        p[u] = 0.0f;
        if (u < total) {
          const int32_t col = ld_stream_p(colval + d.x + u * 32 + lane, pol_s);
          const float a = ld_stream_p(nz + d.x + u * 32 + lane, pol_s);
          if (col > 0) p[u] = __fmul_rn(a, col1_x(sx, xr, col, hot, pol_x));
        }
      }
      int u0 = 0;
      for (int t = 0; t < ns; ++t) {
        const int w = (int)((widths >> (4 * t)) & 15u);
        float acc = 0.0f;
#pragma unroll
        for (int u = 0; u < kNarrowCols; ++u)
          if (u >= u0 && u < u0 + w) acc = __fadd_rn(acc, p[u]);
        if (acc != acc) {  // NaN: the sequential fold with the stop at +Inf
          acc = 0.0f;
          for (int u = u0; u < u0 + w; ++u) {
            acc = __fadd_rn(acc, p[u]);
            if (acc == __int_as_float(0x7f800000)) break;
          }
        }
        u0 += w;
        const int64_t srow = (int64_t)d.y + t * 32 + lane;
        if (srow < m) __stcs(y + (__ldg(perm + srow) - 1), acc);
      }
      continue;
    }
    const int64_t srow = (int64_t)d.y + lane;
    const bool live = srow < m;
    const int32_t pos0 = d.x + lane;
    int32_t pos = pos0;
    float acc = 0.0f;
    int32_t c[8];
    float a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool in = live && u < d.z;
      c[u] = in ? ld_stream_p(colval + pos + u * 32, pol_s) : -1;
      a[u] = in ? ld_stream_p(nz + pos + u * 32, pol_s) : 0.0f;
    }
    for (int32_t j = 0; j < d.z; j += 8) {
      const int32_t pn = pos + 8 * 32;
      int32_t cn[8];
      float an[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = live && j + 8 + u < d.z;
        cn[u] = in ? ld_stream_p(colval + pn + u * 32, pol_s) : -1;
        an[u] = in ? ld_stream_p(nz + pn + u * 32, pol_s) : 0.0f;
      }
      float p[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) p[u] = c[u] > 0 ? __fmul_rn(a[u], col1_x(sx, xr, c[u], hot, pol_x)) : 0.0f;
#pragma unroll
      for (int u = 0; u < 8; ++u) acc = __fadd_rn(acc, p[u]);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        c[u] = cn[u];
        a[u] = an[u];
      }
      pos = pn;
    }
    if (!live) continue;
    if (acc != acc) {  // NaN: this row's piece again, in storage order, stopping at +Inf
      acc = 0.0f;
      for (int32_t j = 0; j < d.z; ++j) {
        const int32_t col = colval[pos0 + j * 32];
        if (col <= 0) break;  // padding: the row ended
        acc = __fadd_rn(acc, __fmul_rn(nz[pos0 + j * 32], col1_x(sx, xr, col, hot, pol_x)));
        if (acc == __int_as_float(0x7f800000)) break;
      }
    }
    if (d.w < 0) __stcs(y + (__ldg(perm + srow) - 1), acc);
    else partials[(int64_t)d.w * 32 + lane] = acc;
  }
}

// rows of slices cut into several chunks: the pieces added in order, stopping at +Inf
// (k_spmm_combine's order; chunks past a row's end hold +0.0, which changes no sum)
__global__ void k_col1_combine(const int4* __restrict__ multi, int64_t nmulti,
                               const float* __restrict__ partials, const int32_t* __restrict__ perm,
                               int64_t m, float* __restrict__ y) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nmulti * 32;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int4 d = multi[t >> 5];  // first stored row, first partial, chunks
    const int o = (int)(t & 31);
    const int64_t srow = (int64_t)d.x + o;
    if (srow >= m) continue;
    // the chunks' partials 8 at a time (a hub slice has hundreds of chunks), folded in
    // order up to the stop at +Inf
    float acc = 0.0f;
    bool stop = false;
    for (int c = 0; c < d.z && !stop; c += 8) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = c + u < d.z ? partials[(int64_t)(d.y + c + u) * 32 + o] : 0.0f;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (c + u < d.z && !stop) {
          acc = __fadd_rn(acc, v[u]);
          stop = acc == __int_as_float(0x7f800000);
        }
      }
    }
    y[perm[srow] - 1] = acc;
  }
}

// y = A x, one column, for a CSR handle of >= 65536 rows (gg_spmm with k == 1); the
// relabelled x and the piece partials live in the context's scratch arena
int launch_col1_sell(gg_ctx* ctx, gg_mat* A, const float* x, float* y) {
  if (!A->sell_copy) {
    GG_CHECK(gg_sell_create(ctx, A, 32, A->m, &A->sell_copy));
    A->sell_copy->sell_variant = A->sell_variant;
    A->sell_copy->hot_cols = A->hot_cols;
  }
  gg_mat* S = A->sell_copy;
  GG_CHECK(build_colperm(ctx, S));
  GG_CHECK(build_col1_plan(ctx, S));
  const SellPlan* P = S->sellplan;
  const int64_t n = A->n;
  const size_t xr_bytes = ((size_t)n * sizeof(float) + 255) & ~(size_t)255;
  GG_CHECK(ensure_scratch(ctx, xr_bytes + (size_t)(P->npart256 * 32 + 1) * sizeof(float)));
  float* xr_buf = static_cast<float*>(ctx->scratch);
  float* partials = reinterpret_cast<float*>(static_cast<char*>(ctx->scratch) + xr_bytes);
  const float* xr = x;
  const int32_t* colval = S->colval;
  if (S->colperm->enabled) {
    k_gather_x<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(x, S->colperm->inv, n, xr_buf);
    trace_count(ctx, 1);
    xr = xr_buf;
    colval = S->colperm->colval_r;
  }
  const int hot_cap = S->hot_cols > 0 ? (S->hot_cols < kHotColsMax ? S->hot_cols : kHotColsMax)
                                      : kHotCols;
  const int hot = (int)std::min<int64_t>(n, hot_cap);
  static bool attr_set[64] = {false};
  if (ctx->device < 64 && !attr_set[ctx->device]) {
    GG_CUDA(cudaFuncSetAttribute(k_col1_sell, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kHotColsMax * (int)sizeof(float)));
    attr_set[ctx->device] = true;
  }
  if (P->npitems256 > 0) {
    const int tr = trace_main_begin(ctx);
    k_col1_sell<<<ctx->num_sms, kHotThreads, hot * sizeof(float), ctx->stream>>>(
        static_cast<const float*>(S->nzval), xr, y, colval, S->perm, S->m, P->pitems256,
        P->npitems256, partials, hot);
    trace_main_end(ctx, tr);
    trace_count(ctx, 1);
  }
  if (P->nmulti256 > 0) {
    k_col1_combine<<<grid_for(ctx, P->nmulti256 * 32, 256), 256, 0, ctx->stream>>>(
        P->multi256, P->nmulti256, partials, S->perm, S->m, y);
    trace_count(ctx, 1);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// plus-times Float32 y = A x over a CSR handle with the row-block pipeline kernel
// (colval: the handle's own or relabelled column labels); trace_main brackets the
// kernel as the call's main kernel
int launch_pipe_f32(gg_ctx* ctx, gg_mat* A, const float* nz, const float* x, float* y,
                    const int32_t* colval, bool trace_main) {
  GG_CHECK(build_row_blocks(ctx, A));
  RowBlocks* rb = A->blocks;
  const int64_t items = rb->nblocks > rb->nsegs ? rb->nblocks : rb->nsegs;
  if (items == 0) return GG_OK;
  static int per_sm = 0;
  if (per_sm == 0) {
    GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, k_spmv_pipe<SRPlusTimesF32>, kPipeWarps * 32, 0));
    if (per_sm < 1) per_sm = 1;
  }
  SRPlusTimesF32 sr;
  sr.nz = nz;
  sr.x = x;
  sr.y = y;
  int64_t grid = (items + kPipeWarps - 1) / kPipeWarps;
  const int64_t cap = (int64_t)ctx->num_sms * per_sm;  // one resident wave
  if (grid > cap) grid = cap;
  const int tr = trace_main ? trace_main_begin(ctx) : -1;
  k_spmv_pipe<SRPlusTimesF32><<<(int)grid, kPipeWarps * 32, 0, ctx->stream>>>(
      sr, A->rowptr, colval, rb->blocks, rb->nblocks, rb->segs, rb->nsegs,
      rb->long_first_seg, rb->long_rows, rb->long_count, static_cast<float*>(rb->partials));
  trace_main_end(ctx, tr);
  trace_count(ctx, 1);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ---------------------------------------------------------------------------------
// A CSR handle whose plus-times product ran on its SELL-32 copy or its column-window
// tiles: those kernels fold without the stop at +Inf (the SELL reference kernel has
// none), so every row whose result is NaN is folded again over the handle's own CSR
// in storage order with the stop (csr_spmv_kernel!, src/spmv/CSR.jl:47-52).  One warp
// per 32 rows reads their results (one coalesced load) and refolds its NaN rows
// together (warp_refold_row).  Inputs without NaN / -Inf cost one read of y.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_refold_nan_rows(SRPlusTimesF32 sr, const int32_t* __restrict__ rowptr,
                      const int32_t* __restrict__ colval, int64_t m) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32 < m; w += nw) {
    const int64_t r = w * 32 + lane;
    const float v = r < m ? __ldcs(sr.y + r) : 0.0f;
    unsigned bad = __ballot_sync(kFull, v != v);
    while (bad) {
      const int b = __ffs(bad) - 1;
      bad &= bad - 1;
      const int64_t row = w * 32 + b;
      const float acc = warp_refold_row(sr, rowptr, colval, row, lane);
      if (lane == 0) sr.y[row] = acc;
    }
  }
}

static int launch_refold_nan_rows(gg_ctx* ctx, const gg_mat* A, const float* x, float* y) {
  SRPlusTimesF32 sr;
  sr.nz = static_cast<const float*>(A->nzval);
  sr.x = x;
  sr.y = y;
  const int64_t warps = (A->m + 31) / 32;
  int64_t grid = (warps + 7) / 8;
  const int64_t cap = (int64_t)ctx->num_sms * 8;
  if (grid > cap) grid = cap;
  k_refold_nan_rows<<<(int)grid, 256, 0, ctx->stream>>>(sr, A->rowptr, A->colval, A->m);
  trace_count(ctx, 1);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
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
    if (A->format == GG_FMT_CSR && A->tuned_spmv == 3) {
      // column-window tiles (gg_spmv_win.cu), when the column frequencies are skewed
      // enough for shared-memory windows to pay; otherwise the SELL copy below
      GG_CHECK(build_win_plan(ctx, A));
      if (A->winplan->enabled) {
        A->last_layout = 3;
        GG_CHECK(launch_spmv_win(ctx, A, sr.x, sr.y));
        return launch_refold_nan_rows(ctx, A, sr.x, sr.y);
      }
    }
    const bool use_copy = A->tuned_spmv == 2 || ((A->tuned_spmv == 0 || A->tuned_spmv == 3) &&
                                                 A->m >= (1 << 16));
    if (A->format == GG_FMT_CSR && use_copy) {
      // plus-times over a large CSR runs on a SELL-32 copy with rows sorted by length
      // (built once; gg_tune may pick another C and sigma): slices of equal-length
      // rows give every thread the same work
      if (!A->sell_copy) {
        GG_CHECK(gg_sell_create(ctx, A, 32, A->m, &A->sell_copy));
        A->sell_copy->sell_variant = A->sell_variant;  // choices applied before the copy
        A->sell_copy->hot_cols = A->hot_cols;
      }
      A->last_layout = 2;
      GG_CHECK(spmv_dispatch(ctx, A->sell_copy, tc, mul, add, accum, y, ty, x, tx, mask, tmask,
                             lo, hi));
      return launch_refold_nan_rows(ctx, A, sr.x, sr.y);
    }
    GG_CHECK(build_colperm(ctx, A));
    const int32_t* colval = A->colval;
    if (A->colperm->enabled) {
      k_gather_x<<<grid_for(ctx, A->n, 256), 256, 0, ctx->stream>>>(
          static_cast<const float*>(x), A->colperm->inv, A->n, A->colperm->xr);
      trace_count(ctx, 1);
      sr.x = A->colperm->xr;
      colval = A->colperm->colval_r;
    }
    if (A->format == GG_FMT_CSR) {
      A->last_layout = 1;
      return launch_pipe_f32(ctx, A, sr.nz, sr.x, sr.y, colval, true);
    }
    A->last_layout = 2;
    if (A->colperm->enabled) return launch_sell_hot(ctx, A, sr, colval);
    return launch_sell(ctx, A, sr, nullptr, 0, 0, 0, colval);
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
