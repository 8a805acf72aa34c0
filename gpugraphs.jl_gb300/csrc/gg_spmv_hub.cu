// gg_spmv_hub.cu -- the hub rows of a plus-times Float32 SpMV over a sorted SELL-32
// copy, folded from shared-memory column windows.
//
// Why: the SELL-32 kernel (k_sell_hot32) serves the gathers of the 32768 most
// frequent columns from shared memory; every other gather is its own 32-byte request
// to L2, and that request rate bounds the kernel (half of the HBM peak on R-MAT).  On
// a power-law graph most of those cold gathers come from the long rows: at R-MAT
// scale 22 the rows of more than 128 entries hold 73% of the entries and three
// quarters of the cold gathers.  Those rows (the first np stored rows of the copy,
// which is sorted by row length) are taken out of the SELL-32 kernel and folded here:
// the x values of each window of kHwCols consecutive column ranks are copied into
// shared memory once per group of up to pg rows (a 32 KB bulk copy), and every entry
// of the group's rows inside the window is served from there.  The remaining rows
// keep the SELL-32 kernel, which now meets about a quarter of the cold gathers.
//
// Layout (HubWinPlan in gg_common.cuh): row i of a group is accumulator slot i in
// shared memory and belongs to warp i mod 32, so a row is only ever updated by one
// warp and no atomics are needed.  For every (group, warp, window) the warp's runs (a
// row's entries inside the window, storage order) of more than kHwRunMin entries are
// run items (stored contiguously, the lanes take 4 entries each with 16-byte loads);
// the other rows form SELL-32 slices (lane = row, sorted by entry count in the window,
// padded with a zero slot), column offsets in 16 bits.  A slice of more than
// kHwNarrow entry rows is a quad slice (each lane's entries in groups of 4, 16-byte
// loads); narrower slices are packed kHwNarrow entry rows per item, across up to
// kHwBufs consecutive windows of one unit (loaded at once, like the narrow groups of
// k_sell_hot32).  A heavy window is split over several units by group warp.
//
// Kernel (k_hubwin): one 1024-thread CTA per SM walks its units (group and group-warp
// range, window range, partial slot; assigned longest first to the least loaded CTA).
// Windows pass through a ring of kHwBufs buffers: the copy of window j completes on
// mbarrier j mod kHwBufs, and the last warp to leave window j issues the copy of
// window j + kHwBufs (the sequence runs on across the CTA's units).  A warp waits for
// every window before it leaves it, so the arrivals counted for a buffer always belong
// to one window.  Warps never wait for one another inside a unit.  A row's fold is sequential: slot value,
// then its entries in storage order, window after window; the unit's slots go to its
// partial, and k_hw_combine adds a row's partials in window order.  Every sum is
// formed in one fixed order, so repeated calls give identical bits.  Every wait is
// bounded (the context's poll limit; then the error flag, a drain of the copies in
// flight and an orderly return).
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "gg_semiring.cuh"
#include "gg_tma.cuh"

namespace gg {

static const int kHwThreads = 1024;
static const int kHwWarps = kHwThreads / 32;
static const int kHwBufs = 4;                  // window buffers in the ring
static const int kHwStride = kHwCols + 4;      // floats per buffer: window + zero slot
static const int kHwMaxRows = 16384;           // accumulator slots (rows) per group
static const int kHwNarrow = 8;                // entry rows of a narrow item
static const int kHwRunMin = 32;               // longer runs are run items (lanes over entries)
static const unsigned kHwPolls = 1u << 22;
// a group is folded from windows only while its entries per staged x value reach this
#ifndef GG_HW_DENSITY
#define GG_HW_DENSITY 8.0
#endif
static const double kHwDensity = GG_HW_DENSITY;
static const int kHwUnitsPerSm = 3;
static const double kHwWinCost = 150.0;  // a window's copy and waits, in entry rows

static size_t hw_smem(int pg) {
  return (size_t)kHwBufs * kHwStride * 4 + (size_t)pg * 4 + 16 * 4 + 8 * kHwBufs;
}

__device__ __forceinline__ uint16_t hw_ld_u16(const uint16_t* p, uint64_t pol) {
  unsigned short r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.u16 %0, [%1], %2;"
      : "=h"(r)
      : "l"(p), "l"(pol));
  return r;
}

// try_wait with a suspend-time hint: a waiting warp sleeps until the phase completes
// (or about 1 us passes) instead of spinning on the issue slots the working warps need
__device__ __forceinline__ bool hw_try_wait_sleep(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity), "r"(1000u)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint2 hw_ld_u2(const uint16_t* p, uint64_t pol) {
  uint2 r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.v2.u32 {%0,%1}, [%2], %3;"
      : "=r"(r.x), "=r"(r.y)
      : "l"(p), "l"(pol));
  return r;
}

__device__ __forceinline__ float4 hw_ld_f4(const float* p, uint64_t pol) {
  float4 r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
      : "l"(p), "l"(pol));
  return r;
}

__device__ __forceinline__ bool hw_wait(uint32_t bar, uint32_t parity, unsigned limit) {
  for (unsigned p = 0; p < limit; ++p)
    if (hw_try_wait_sleep(bar, parity)) return true;
  return false;
}

// window of position q in this CTA's window sequence (its units, each contributing
// its windows in order)
__device__ bool hw_seq_window(const int4* __restrict__ units, const int32_t* __restrict__ cptr,
                              int64_t q, int* w) {
  for (int u = cptr[blockIdx.x]; u < cptr[blockIdx.x + 1]; ++u) {
    const int4 U = units[u];
    const int64_t len = U.z - U.y;
    if (q < len) {
      *w = U.y + (int)q;
      return true;
    }
    q -= len;
  }
  return false;
}

// scnt: [0, kHwBufs) arrivals per buffer, [kHwBufs] abort, [kHwBufs + 1 + b] fills
// issued into buffer b
__device__ void hw_issue(const float* __restrict__ xr, float* bufs, uint32_t bar0, volatile int* scnt,
                         const int4* __restrict__ units, const int32_t* __restrict__ cptr, int64_t q) {
  int w;
  if (!hw_seq_window(units, cptr, q, &w)) return;
  const int b = (int)(q % kHwBufs);
  mbar_expect_tx(bar0 + 8 * b, kHwCols * 4);
  bulk_g2s(smem_u32(bufs + b * kHwStride), xr + (int64_t)w * kHwCols, kHwCols * 4, bar0 + 8 * b);
  scnt[kHwBufs + 1 + b] += 1;
}

// one work item of a warp, its first window in ring buffer qf mod kHwBufs:
//  * a slice of one window: d.z = width, d.w = 0, entries from d.x, slot lanes from d.y;
//  * up to kHwNarrow entry rows of consecutive narrow slices of this warp, possibly of
//    up to kHwBufs consecutive windows: d.z = INT_MIN | entry rows << 8, d.w = one
//    bit per entry row that starts a slice (bits 0-7) and the entry row's window
//    offset (2 bits each from bit 8);
//  * a run of one row in one window: d.w = -1, d.z entries stored contiguously from
//    d.x, slot d.y; entry j is folded by lane j mod 32 (in order), then a butterfly
//    sum is added to the slot.
__device__ __forceinline__ void hw_item(const int4 d, const uint16_t* __restrict__ col,
                                        const float* __restrict__ val,
                                        const uint16_t* __restrict__ rowid, const float* bufs,
                                        int64_t qf, float* ys, int lane, uint64_t pol) {
  if (d.w == -1) {
    // run: lane l folds entries 4l .. 4l + 3 of every 128 (16-byte value loads; the
    // run is padded to a multiple of 4 with zero-slot entries)
    const float* xs = bufs + (int)(qf % kHwBufs) * kHwStride;
    float acc = 0.0f;
    const int32_t end = d.x + d.z;
    int32_t pos = d.x + lane * 4;
    uint2 cv = make_uint2(0, 0);
    float4 av = make_float4(0.f, 0.f, 0.f, 0.f);
    if (pos < end) {
      cv = hw_ld_u2(col + pos, pol);
      av = hw_ld_f4(val + pos, pol);
    } else {
      cv = make_uint2(kHwCols | (kHwCols << 16), kHwCols | (kHwCols << 16));
    }
    for (int32_t b = d.x; b < end; b += 128) {
      const int32_t pn = pos + 128;
      uint2 cn = make_uint2(kHwCols | (kHwCols << 16), kHwCols | (kHwCols << 16));
      float4 an = make_float4(0.f, 0.f, 0.f, 0.f);
      if (pn < end) {
        cn = hw_ld_u2(col + pn, pol);
        an = hw_ld_f4(val + pn, pol);
      }
      acc = __fadd_rn(acc, __fmul_rn(av.x, xs[cv.x & 0xffffu]));
      acc = __fadd_rn(acc, __fmul_rn(av.y, xs[cv.x >> 16]));
      acc = __fadd_rn(acc, __fmul_rn(av.z, xs[cv.y & 0xffffu]));
      acc = __fadd_rn(acc, __fmul_rn(av.w, xs[cv.y >> 16]));
      cv = cn;
      av = an;
      pos = pn;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    if (lane == 0) ys[d.y] = __fadd_rn(ys[d.y], acc);
    return;
  }
  if (d.w == -2) {
    // quad slice: lane = row, d.z steps of 4 entries per lane stored [step][lane][4]
    const float* xs = bufs + (int)(qf % kHwBufs) * kHwStride;
    const uint16_t r = hw_ld_u16(rowid + d.y + lane, pol);
    float acc = r != 0xffff ? ys[r] : 0.0f;
    int32_t pos = d.x + lane * 4;
    uint2 cv = hw_ld_u2(col + pos, pol);
    float4 av = hw_ld_f4(val + pos, pol);
    for (int32_t st = 0; st < d.z; ++st) {
      const int32_t pn = pos + 128;
      uint2 cn = cv;
      float4 an = av;
      if (st + 1 < d.z) {
        cn = hw_ld_u2(col + pn, pol);
        an = hw_ld_f4(val + pn, pol);
      }
      acc = __fadd_rn(acc, __fmul_rn(av.x, xs[cv.x & 0xffffu]));
      acc = __fadd_rn(acc, __fmul_rn(av.y, xs[cv.x >> 16]));
      acc = __fadd_rn(acc, __fmul_rn(av.z, xs[cv.y & 0xffffu]));
      acc = __fadd_rn(acc, __fmul_rn(av.w, xs[cv.y >> 16]));
      cv = cn;
      av = an;
      pos = pn;
    }
    if (r != 0xffff) ys[r] = acc;
    return;
  }
  if (d.z < 0) {
    // entry row u: bit u of d.w starts a new slice (row lanes), bits 8 + 2u.. the
    // window offset; slices are consecutive in the slot-lane array from d.y
    const int total = (d.z >> 8) & 15;
    const uint32_t bnd = (uint32_t)d.w & 0xffu, offs = (uint32_t)d.w >> 8;
    uint16_t c[kHwNarrow], r[kHwNarrow];
    float a[kHwNarrow];
#pragma unroll
    for (int u = 0; u < kHwNarrow; ++u) {
      const bool in = u < total;
      c[u] = in ? hw_ld_u16(col + d.x + u * 32 + lane, pol) : (uint16_t)kHwCols;
      a[u] = in ? ld_stream_p(val + d.x + u * 32 + lane, pol) : 0.0f;
      const int t = __popc(bnd & ((2u << u) - 1u)) - 1;  // slice of entry row u
      r[u] = (in && ((bnd >> u) & 1u)) ? hw_ld_u16(rowid + d.y + t * 32 + lane, pol) : (uint16_t)0xffff;
    }
    float p[kHwNarrow];
#pragma unroll
    for (int u = 0; u < kHwNarrow; ++u)
      p[u] = __fmul_rn(a[u], bufs[(int)((qf + ((offs >> (2 * u)) & 3u)) % kHwBufs) * kHwStride + c[u]]);
    uint16_t rc = 0xffff;
    float acc = 0.0f;
#pragma unroll
    for (int u = 0; u < kHwNarrow; ++u) {
      if (u < total) {
        if ((bnd >> u) & 1u) {  // warp-uniform: the next slice starts
          if (u > 0) {
            if (rc != 0xffff) ys[rc] = acc;
            __syncwarp();  // a row may recur in a later slice (a later window), another lane
          }
          rc = r[u];
          acc = rc != 0xffff ? ys[rc] : 0.0f;
        }
        acc = __fadd_rn(acc, p[u]);
      }
    }
    if (rc != 0xffff) ys[rc] = acc;
    return;
  }
  const float* xs = bufs + (int)(qf % kHwBufs) * kHwStride;
  const uint16_t r = hw_ld_u16(rowid + d.y + lane, pol);
  float acc = r != 0xffff ? ys[r] : 0.0f;
  int32_t pos = d.x + lane;
  uint16_t c[8];
  float a[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const bool in = u < d.z;
    c[u] = in ? hw_ld_u16(col + pos + u * 32, pol) : (uint16_t)kHwCols;
    a[u] = in ? ld_stream_p(val + pos + u * 32, pol) : 0.0f;
  }
  for (int32_t j = 0; j < d.z; j += 8) {
    const int32_t pn = pos + 8 * 32;
    uint16_t cn[8];
    float an[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool in = j + 8 + u < d.z;
      cn[u] = in ? hw_ld_u16(col + pn + u * 32, pol) : (uint16_t)kHwCols;
      an[u] = in ? ld_stream_p(val + pn + u * 32, pol) : 0.0f;
    }
    float p[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) p[u] = __fmul_rn(a[u], xs[c[u]]);
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (j + u < d.z) acc = __fadd_rn(acc, p[u]);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      c[u] = cn[u];
      a[u] = an[u];
    }
    pos = pn;
  }
  if (r != 0xffff) ys[r] = acc;
}

// windows an item reads: its first and, for a narrow item, up to kHwBufs - 1 more
__device__ __forceinline__ int hw_span(const int4 d) {
  if (d.z >= 0 || d.w < 0) return 1;
  const int total = (d.z >> 8) & 15;
  return 1 + (int)(((uint32_t)d.w >> (8 + 2 * (total - 1))) & 3u);
}

// leave window q (sequence position) for this warp; the last warp out refills its
// buffer with window q + kHwBufs once the copy it held has landed
__device__ __forceinline__ void hw_arrive(int64_t q, int64_t total, const float* __restrict__ xr,
                                          float* bufs, uint32_t bar0, volatile int* scnt,
                                          const int4* __restrict__ units,
                                          const int32_t* __restrict__ cptr, int lane,
                                          unsigned polls, unsigned* err) {
  __syncwarp();
  if (lane == 0) {
    const int b = (int)(q % kHwBufs);
    __threadfence_block();
    if (atomicAdd((int*)scnt + b, 1) == kHwWarps - 1) {
      scnt[b] = 0;
      if (q + kHwBufs < total && scnt[kHwBufs] == 0) {
        if (hw_wait(bar0 + 8 * b, (uint32_t)((q / kHwBufs) & 1), polls)) {
          fence_proxy_async();
          hw_issue(xr, bufs, bar0, scnt, units, cptr, q + kHwBufs);
        } else {
          scnt[kHwBufs] = 1;
          if (err) atomicExch(err, 1u);
        }
      }
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kHwThreads, 1)
    k_hubwin(const float* __restrict__ xr, const uint16_t* __restrict__ col,
             const float* __restrict__ val, const uint16_t* __restrict__ rowid,
             const int4* __restrict__ items, const int32_t* __restrict__ itemptr,
             const int4* __restrict__ units, const int32_t* __restrict__ cptr, int nwin, int pg,
             float* __restrict__ partials, unsigned* err, unsigned polls) {
  extern __shared__ __align__(128) unsigned char smem[];
  float* bufs = reinterpret_cast<float*>(smem);
  float* ys = bufs + kHwBufs * kHwStride;
  volatile int* scnt = reinterpret_cast<volatile int*>(ys + pg);
  uint64_t* sbar = reinterpret_cast<uint64_t*>(ys + pg + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bar0 = smem_u32(sbar);
  if (tid == 0) {
    for (int b = 0; b < kHwBufs; ++b) mbar_init(bar0 + 8 * b, 1);
    for (int i = 0; i < 16; ++i) scnt[i] = 0;
  }
  if (tid < kHwBufs * 4) bufs[(tid >> 2) * kHwStride + kHwCols + (tid & 3)] = 0.0f;  // zero slots
  fence_mbar_init();
  __syncthreads();
  int64_t total = 0;  // windows of this CTA's units
  const int u0 = cptr[blockIdx.x], u1 = cptr[blockIdx.x + 1];
  for (int u = u0; u < u1; ++u) total += units[u].z - units[u].y;
  if (tid == 0) {
    fence_proxy_async();
    for (int64_t q = 0; q < kHwBufs && q < total; ++q) hw_issue(xr, bufs, bar0, scnt, units, cptr, q);
  }
  const uint64_t pol = l2_evict_first();
  int64_t qu = 0;  // sequence position of the unit's first window
  for (int u = u0; u < u1; ++u) {
    const int4 U = units[u];  // packed group / warp range, first window, end window, slot
    const int g = U.x & 0xffff, gw0 = (U.x >> 16) & 31, lg = (U.x >> 21) & 7;
    // the unit's group warps gw0 .. gw0 + 2^lg - 1 (all 32 for a window range; a
    // heavy single window is split over several units by group warp): CTA warp i takes
    // every (32 >> lg)-th item of group warp gw0 + i mod 2^lg
    const int gw = gw0 + (warp & ((1 << lg) - 1));
    const int io = warp >> lg, ist = kHwWarps >> lg;
    const int nw = U.z - U.y;
    for (int i = tid; i < pg; i += kHwThreads) ys[i] = 0.0f;
    __syncthreads();
    const int32_t* ip = itemptr + ((int64_t)g * kHwWarps + gw) * nwin + U.y;
    const int32_t iend = ip[nw];
    int32_t it = ip[0] + io;
    // windows of the unit (relative) this warp has waited for / left.  A warp leaves a
    // window only after waiting for it: the copy of window q is issued once every warp
    // has left window q - kHwBufs, so no warp can leave window q while another is still
    // in q - kHwBufs (their arrivals share one counter per buffer), and every wait is on
    // the phase right after the last one this warp saw.
    int wcur = 0, waited = 0, arrived = 0;
    int ok = scnt[kHwBufs] == 0;
    auto wait_next = [&]() {
      if (ok) {
        const int64_t qw = qu + waited;
        if (lane == 0) ok = hw_wait(bar0 + 8 * (int)(qw % kHwBufs), (uint32_t)((qw / kHwBufs) & 1), polls);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok && lane == 0 && scnt[kHwBufs] == 0) {
          scnt[kHwBufs] = 1;
          if (err) atomicExch(err, 1u);
        }
      }
      ++waited;
    };
    auto leave_next = [&]() {
      if (waited == arrived) wait_next();
      hw_arrive(qu + arrived, total, xr, bufs, bar0, scnt, units, cptr, lane, polls, err);
      ++arrived;
    };
    int4 d = it < iend ? __ldg(items + it) : make_int4(0, 0, 0, 0);
    int32_t wend = ip[1];  // first item of the window after wcur
    while (it < iend) {
      const int4 dn = it + ist < iend ? __ldg(items + it + ist) : d;  // next descriptor ahead
      while (it >= wend) wend = ip[++wcur + 1];  // the item's first window
      while (arrived < wcur) leave_next();  // windows this warp is done with
      const int need = wcur + hw_span(d);  // at most kHwBufs windows past the last left
      while (waited < need) wait_next();
      if (ok && scnt[kHwBufs] == 0) {
        hw_item(d, col, val, rowid, bufs, qu + wcur, ys, lane, pol);
        __syncwarp();  // the next item may update a row of this one from another lane
      }
      it += ist;
      d = dn;
    }
    while (arrived < nw) leave_next();
    qu += nw;
    __syncthreads();
    // the unit's rows (slot i belongs to group warp i mod 32) into its partial
    float* out = partials + (int64_t)U.w * pg;
    const int nsel = 1 << lg;
    for (int i = tid; i < pg; i += kHwThreads)
      if (((i & 31) - gw0) >= 0 && ((i & 31) - gw0) < nsel) __stcg(out + i, ys[i]);
    __syncthreads();
  }
  if (tid == 0) {
    // let every copy land before the CTA's shared memory goes away (a window no warp
    // read, or any after a wait ran out, may still be in flight)
    for (int b = 0; b < kHwBufs; ++b) {
      const int f = scnt[kHwBufs + 1 + b];
      if (f > 0) hw_wait(bar0 + 8 * b, (uint32_t)((f - 1) & 1), kHwPolls);
    }
  }
}

// y of the hub rows: a row's unit partials added in window order
__global__ void k_hw_combine(int64_t np, int pg, const int32_t* __restrict__ gptr,
                             const float* __restrict__ partials, const int32_t* __restrict__ perm,
                             float* __restrict__ y) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)(p / pg), pl = (int)(p - (int64_t)g * pg);
    const int k0 = gptr[g], k1 = gptr[g + 1];
    float s = partials[(int64_t)k0 * pg + pl];
    for (int k = k0 + 1; k < k1; ++k) s = __fadd_rn(s, partials[(int64_t)k * pg + pl]);
    const int32_t r1 = perm ? perm[p] : (int32_t)(p + 1);
    __stcs(y + (r1 - 1), s);
  }
}

// ---------------------------------------------------------------------------------
// layout build (once per matrix)
// ---------------------------------------------------------------------------------

// entries of stored rows [0, nc): the first padding slot of the row (rows are packed
// to the left of their slice, padding -1)
__global__ void k_hw_rowlen(int64_t nc, const int32_t* __restrict__ slice_ptr,
                            const int32_t* __restrict__ colval, int32_t* len) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nc;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = p >> 5, o = p & 31;
    const int64_t base = (int64_t)slice_ptr[s] - 1 + o;
    int64_t lo = 0, hi = ((int64_t)slice_ptr[s + 1] - slice_ptr[s]) / 32;  // first -1 in [lo, hi]
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (colval[base + mid * 32] < 0) hi = mid;
      else lo = mid + 1;
    }
    len[p] = (int32_t)lo;
  }
}

// sort keys of the hub entries: (group, warp, window, slot), value = SELL position;
// a row's entries are emitted in storage order (the sort is stable)
__global__ void k_hw_keys(int64_t np, int pg, int64_t nwin, const int32_t* __restrict__ slice_ptr,
                          const int32_t* __restrict__ colval_r, const int32_t* __restrict__ len,
                          const int64_t* __restrict__ pptr, uint64_t* keys, int32_t* vals) {
  const int lane = threadIdx.x & 31;
  for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < np;
       p += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t g = p / pg, pl = p - g * pg;
    const int64_t base = (int64_t)slice_ptr[p >> 5] - 1 + (p & 31);
    const int32_t L = len[p];
    const int64_t o = pptr[p];
    const uint64_t seg0 = (uint64_t)(g * kHwWarps + (pl & 31)) * (uint64_t)nwin;
    for (int32_t j = lane; j < L; j += 32) {
      const int64_t pos = base + (int64_t)j * 32;
      const int64_t rank = (int64_t)colval_r[pos] - 1;
      keys[o + j] = (seg0 + (uint64_t)(rank / kHwCols)) * (uint64_t)pg + (uint64_t)pl;
      vals[o + j] = (int32_t)pos;
    }
  }
}

// per run (distinct (group, warp, window, slot)): segment key in the high 32 bits,
// the count descending in the low 32 (a row may hold repeated columns, so a count is
// not bounded by the window width)
__global__ void k_hw_key2(int64_t nr, int pg, const uint64_t* __restrict__ ukey,
                          const int32_t* __restrict__ cnt, uint64_t* key2, int32_t* idx) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nr;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t seg = ukey[i] / (uint64_t)pg;
    key2[i] = (seg << 32) | (uint64_t)(0xffffffffu - (uint32_t)cnt[i]);
    idx[i] = (int32_t)i;
  }
}

__global__ void k_hw_segid(int64_t nr, const uint64_t* __restrict__ key2, uint64_t* segid) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nr;
       i += (int64_t)gridDim.x * blockDim.x)
    segid[i] = key2[i] >> 32;
}

// runs of more than kHwRunMin entries at the head of every segment (the runs of a
// segment are sorted by count, descending): they become run items
__global__ void k_hw_nwide(int64_t nseg, const int32_t* __restrict__ segcnt,
                           const int32_t* __restrict__ seg_run0, const int32_t* __restrict__ order,
                           const int32_t* __restrict__ cnt, int32_t* nwide) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nseg;
       c += (int64_t)gridDim.x * blockDim.x) {
    int32_t k = 0;
    while (k < segcnt[c] && cnt[order[seg_run0[c] + k]] > kHwRunMin) ++k;
    nwide[c] = k;
  }
}

// count and slot of every wide run, in segment order
__global__ void k_hw_wideinfo(int64_t nseg, const int32_t* __restrict__ nwide,
                              const int32_t* __restrict__ wide0, const int32_t* __restrict__ seg_run0,
                              const int32_t* __restrict__ order, const int32_t* __restrict__ cnt,
                              const uint64_t* __restrict__ ukey, int pg, int2* info) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nseg;
       c += (int64_t)gridDim.x * blockDim.x)
    for (int32_t k = 0; k < nwide[c]; ++k) {
      const int32_t r = order[seg_run0[c] + k];
      info[wide0[c] + k] = make_int2(cnt[r], (int)(ukey[r] % (uint64_t)pg));
    }
}

// width of every slice: the largest count among its (at most 32) runs, the segment's
// runs after its wide ones
__global__ void k_hw_widths(int64_t nseg, const int32_t* __restrict__ segcnt,
                            const int32_t* __restrict__ nwide, const int32_t* __restrict__ seg_run0,
                            const int32_t* __restrict__ slice0, const int32_t* __restrict__ order,
                            const int32_t* __restrict__ cnt, int32_t* width) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nseg;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r0 = seg_run0[c] + nwide[c], nrun = segcnt[c] - nwide[c];
    for (int32_t j = 0; j * 32 < nrun; ++j) {
      int32_t mx = 0;
      for (int32_t l = j * 32; l < nrun && l < j * 32 + 32; ++l) mx = max(mx, cnt[order[r0 + l]]);
      width[slice0[c] + j] = mx;
    }
  }
}

// entries of every run: a wide run contiguously at its own offset, any other into its
// slice lane (thread per run, runs in segment order)
__global__ void k_hw_fill(int64_t nr, int64_t nseg, int pg, int64_t nwin,
                          const int32_t* __restrict__ seg_run0, const int32_t* __restrict__ nwide,
                          const int32_t* __restrict__ wide0, const int32_t* __restrict__ woff,
                          const int32_t* __restrict__ slice0, const int32_t* __restrict__ soff,
                          const int32_t* __restrict__ width,
                          const int32_t* __restrict__ order, const uint64_t* __restrict__ ukey,
                          const int32_t* __restrict__ cnt, const int32_t* __restrict__ start,
                          const int32_t* __restrict__ spos, const int32_t* __restrict__ colval_r,
                          const float* __restrict__ nz, uint16_t* col, float* val, uint16_t* rowid) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nr;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = nseg - 1;  // last segment whose first run is <= i
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (seg_run0[mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    const int64_t k = i - seg_run0[lo];
    const int32_t r = order[i];
    const uint64_t uk = ukey[r];
    const int64_t w = (int64_t)((uk / (uint64_t)pg) % (uint64_t)nwin);
    int64_t off, step;
    if (k < nwide[lo]) {
      off = woff[wide0[lo] + k];
      step = 1;
    } else {
      const int64_t kk = k - nwide[lo];
      const int64_t slice = slice0[lo] + (kk >> 5);
      const int lane = (int)(kk & 31);
      rowid[slice * 32 + lane] = (uint16_t)(uk % (uint64_t)pg);
      if (width[slice] > kHwNarrow) {  // quad slice: [step][lane][4]
        off = (int64_t)soff[slice] + lane * 4;
        step = -1;
      } else {
        off = (int64_t)soff[slice] + lane;
        step = 32;
      }
    }
    const int32_t c = cnt[r], s0 = start[r];
    for (int32_t j = 0; j < c; ++j) {
      const int32_t e = spos[s0 + j];
      const int64_t at = step < 0 ? off + (int64_t)(j >> 2) * 128 + (j & 3) : off + j * step;
      col[at] = (uint16_t)(colval_r[e] - 1 - w * kHwCols);
      val[at] = nz[e];
    }
  }
}

__global__ void k_hw_fill_u16(uint16_t* p, int64_t n, uint16_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

static int hw_grid(gg_ctx* ctx, int64_t threads) {
  int64_t g = (threads + 255) / 256;
  const int64_t cap = (int64_t)ctx->num_sms * 16;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

static int bits_for(uint64_t v) {
  int b = 1;
  while (b < 64 && (v >> b) != 0) ++b;
  return b;
}

void free_hubwin_plan(gg_mat* A) {
  HubWinPlan* P = A->hubwin;
  if (!P) return;
  cudaFree(P->col);
  cudaFree(P->val);
  cudaFree(P->rowid);
  cudaFree(P->items);
  cudaFree(P->itemptr);
  cudaFree(P->units);
  cudaFree(P->cptr);
  cudaFree(P->gptr);
  cudaFree(P->partials);
  free_sell_plan(P->rest);
  delete P;
  A->hubwin = nullptr;
}

// temporaries of the build, freed on every return path
struct HwTemp {
  std::vector<void*> p;
  ~HwTemp() {
    for (void* q : p) cudaFree(q);
  }
  template <typename T>
  cudaError_t alloc(T** out, int64_t n) {
    *out = nullptr;
    cudaError_t e = cudaMalloc((void**)out, (size_t)(n > 0 ? n : 1) * sizeof(T));
    if (e == cudaSuccess) p.push_back((void*)*out);
    return e;
  }
};

static int build_hubwin_plan_impl(gg_ctx* ctx, gg_mat* S);

// The layout is an optional speed-up: when the device has no room for it (the build
// sorts the hub entries with about 24 bytes of temporaries each), the SELL-32 kernel
// runs every row instead of the call failing.
int build_hubwin_plan(gg_ctx* ctx, gg_mat* S) {
  if (S->hubwin) return GG_OK;
  const int rc = build_hubwin_plan_impl(ctx, S);
  if (rc == GG_OK || rc != GG_ERR_OOM) return rc;
  free_hubwin_plan(S);
  S->hubwin = new HubWinPlan();  // disabled
  return GG_OK;
}

static int build_hubwin_plan_impl(gg_ctx* ctx, gg_mat* S) {
  HubWinPlan* P = new HubWinPlan();
  S->hubwin = P;  // disabled unless completed below
  if (S->format != GG_FMT_SELL || S->slice_size != 32 || S->dtype != GG_FLOAT32 ||
      S->m < (1 << 16) || !S->colperm || !S->colperm->enabled || S->nnz == 0)
    return GG_OK;
  const int64_t ns = S->nslices, n = S->n;
  std::vector<int32_t> sp(ns + 1);
  GG_CUDA(cudaMemcpyAsync(sp.data(), S->slice_ptr, (ns + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  int64_t nslc = 0;  // leading slices wider than kSellChunk
  while (nslc < ns && ((int64_t)sp[nslc + 1] - sp[nslc]) / 32 > kSellChunk) ++nslc;
  const int64_t nc = std::min<int64_t>(nslc * 32, S->m);
  if (nc < 32) return GG_OK;
  HwTemp T;
  int32_t* dlen = nullptr;
  GG_CUDA(T.alloc(&dlen, nc));
  k_hw_rowlen<<<hw_grid(ctx, nc), 256, 0, ctx->stream>>>(nc, S->slice_ptr, S->colval, dlen);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> len(nc);
  GG_CUDA(cudaMemcpyAsync(len.data(), dlen, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  // hub rows: the sorted prefix of rows longer than kSellChunk, in groups of pg rows,
  // while a group has at least kHwDensity entries per x value a window stages
  int64_t nlong = 0;
  while (nlong < nc && len[nlong] > kSellChunk) ++nlong;
  nlong = nlong / 32 * 32;
  const int pg = kHwMaxRows;
  const int64_t nwin = (n + kHwCols - 1) / kHwCols;
  int64_t np = 0, ep = 0;
  while (np < nlong) {
    const int64_t g1 = std::min<int64_t>(np + pg, nlong);
    int64_t e = 0;
    for (int64_t p = np; p < g1; ++p) e += len[p];
    if ((double)e < kHwDensity * (double)nwin * kHwCols) break;
    np = g1;
    ep += e;
  }
  if (np == 0 || ep >= ((int64_t)1 << 31) - 4096) return GG_OK;
  const int ngroups = (int)((np + pg - 1) / pg);
  const uint64_t kmax = (uint64_t)ngroups * kHwWarps * (uint64_t)nwin * (uint64_t)pg;
  if (ngroups >= 0xffff || bits_for(kmax) > 62 || (uint64_t)ngroups * kHwWarps * (uint64_t)nwin >= ((uint64_t)1 << 31))
    return GG_OK;
  std::vector<int64_t> pptr(np + 1);
  pptr[0] = 0;
  for (int64_t p = 0; p < np; ++p) pptr[p + 1] = pptr[p] + len[p];
  // 1. keys (group, warp, window, slot) of every hub entry, stably sorted
  int64_t* dpptr = nullptr;
  uint64_t *keys = nullptr, *keys2 = nullptr;
  int32_t *vals = nullptr, *vals2 = nullptr;
  GG_CUDA(T.alloc(&dpptr, np + 1));
  GG_CUDA(T.alloc(&keys, ep));
  GG_CUDA(T.alloc(&keys2, ep));
  GG_CUDA(T.alloc(&vals, ep));
  GG_CUDA(T.alloc(&vals2, ep));
  GG_CUDA(cudaMemcpyAsync(dpptr, pptr.data(), (np + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                          ctx->stream));
  k_hw_keys<<<hw_grid(ctx, np * 32), 256, 0, ctx->stream>>>(np, pg, nwin, S->slice_ptr,
                                                             S->colperm->colval_r, dlen, dpptr, keys, vals);
  GG_CUDA(cudaGetLastError());
  const int kbits = bits_for(kmax);
  // cub temporary storage, grown as the steps need
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  auto need_tmp = [&](size_t b) -> cudaError_t {
    if (b <= tmp_bytes) return cudaSuccess;
    char* t = nullptr;
    cudaError_t e = T.alloc(&t, (int64_t)b);
    if (e == cudaSuccess) {
      tmp = t;
      tmp_bytes = b;
    }
    return e;
  };
  size_t tb = 0;
  GG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, vals2, (int)ep, 0, kbits,
                                          ctx->stream));
  GG_CUDA(need_tmp(tb));
  tb = tmp_bytes;
  GG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, vals2, (int)ep, 0, kbits,
                                          ctx->stream));
  // 2. runs of equal key (a row's entries inside one window) and their starts
  uint64_t* ukey = nullptr;
  int32_t *rcnt = nullptr, *rstart = nullptr, *dnr = nullptr;
  GG_CUDA(T.alloc(&ukey, ep));
  GG_CUDA(T.alloc(&rcnt, ep));
  GG_CUDA(T.alloc(&rstart, ep));
  GG_CUDA(T.alloc(&dnr, 2));
  tb = 0;
  GG_CUDA(cub::DeviceRunLengthEncode::Encode(nullptr, tb, keys2, ukey, rcnt, dnr, (int)ep, ctx->stream));
  GG_CUDA(need_tmp(tb));
  tb = tmp_bytes;
  GG_CUDA(cub::DeviceRunLengthEncode::Encode(tmp, tb, keys2, ukey, rcnt, dnr, (int)ep, ctx->stream));
  int32_t hnr = 0;
  GG_CUDA(cudaMemcpyAsync(&hnr, dnr, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  const int64_t nr = hnr;
  tb = 0;
  GG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, rcnt, rstart, (int)nr, ctx->stream));
  GG_CUDA(need_tmp(tb));
  tb = tmp_bytes;
  GG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, rcnt, rstart, (int)nr, ctx->stream));
  // 3. runs in slice order: segment (group, warp, window), count descending (keys /
  //    vals of step 1 serve as scratch from here on; vals2 keeps the sorted positions)
  uint64_t* k2 = keys;
  int32_t* idx = vals;
  int32_t* order = nullptr;
  uint64_t* k2sorted = nullptr;
  GG_CUDA(T.alloc(&order, nr));
  GG_CUDA(T.alloc(&k2sorted, nr));
  k_hw_key2<<<hw_grid(ctx, nr), 256, 0, ctx->stream>>>(nr, pg, ukey, rcnt, k2, idx);
  GG_CUDA(cudaGetLastError());
  const int k2bits = bits_for(kmax / (uint64_t)pg) + 32;
  tb = 0;
  GG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, k2, k2sorted, idx, order, (int)nr, 0, k2bits,
                                          ctx->stream));
  GG_CUDA(need_tmp(tb));
  tb = tmp_bytes;
  GG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, k2, k2sorted, idx, order, (int)nr, 0, k2bits,
                                          ctx->stream));
  // segments: runs per (group, warp, window)
  uint64_t* segid = keys2;  // reuse (the sorted entry keys are no longer needed)
  k_hw_segid<<<hw_grid(ctx, nr), 256, 0, ctx->stream>>>(nr, k2sorted, segid);
  GG_CUDA(cudaGetLastError());
  uint64_t* useg = nullptr;
  int32_t* segcnt = nullptr;
  GG_CUDA(T.alloc(&useg, nr));
  GG_CUDA(T.alloc(&segcnt, nr));
  tb = 0;
  GG_CUDA(cub::DeviceRunLengthEncode::Encode(nullptr, tb, segid, useg, segcnt, dnr, (int)nr, ctx->stream));
  GG_CUDA(need_tmp(tb));
  tb = tmp_bytes;
  GG_CUDA(cub::DeviceRunLengthEncode::Encode(tmp, tb, segid, useg, segcnt, dnr, (int)nr, ctx->stream));
  int32_t hns = 0;
  GG_CUDA(cudaMemcpyAsync(&hns, dnr, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  const int64_t nseg = hns;
  std::vector<uint64_t> hseg(nseg);
  std::vector<int32_t> hsegcnt(nseg);
  GG_CUDA(cudaMemcpyAsync(hseg.data(), useg, nseg * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(hsegcnt.data(), segcnt, nseg * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> hrun0(nseg);
  {
    int64_t runs = 0;
    for (int64_t c = 0; c < nseg; ++c) {
      hrun0[c] = (int32_t)runs;
      runs += hsegcnt[c];
    }
  }
  int32_t *drun0 = nullptr, *dnwide = nullptr;
  GG_CUDA(T.alloc(&drun0, nseg));
  GG_CUDA(T.alloc(&dnwide, nseg));
  GG_CUDA(cudaMemcpyAsync(drun0, hrun0.data(), nseg * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
  k_hw_nwide<<<hw_grid(ctx, nseg), 256, 0, ctx->stream>>>(nseg, segcnt, drun0, order, rcnt, dnwide);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> hnwide(nseg);
  GG_CUDA(cudaMemcpyAsync(hnwide.data(), dnwide, nseg * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> hslice0(nseg), hwide0(nseg);
  int64_t nslices = 0, nwruns = 0;
  for (int64_t c = 0; c < nseg; ++c) {
    hslice0[c] = (int32_t)nslices;
    hwide0[c] = (int32_t)nwruns;
    nslices += (hsegcnt[c] - hnwide[c] + 31) / 32;
    nwruns += hnwide[c];
  }
  if (nslices * 32 >= ((int64_t)1 << 31)) return GG_OK;
  int32_t *dslice0 = nullptr, *dwide0 = nullptr, *dwidth = nullptr;
  int2* dwinfo = nullptr;
  GG_CUDA(T.alloc(&dslice0, nseg));
  GG_CUDA(T.alloc(&dwide0, nseg));
  GG_CUDA(T.alloc(&dwidth, nslices));
  GG_CUDA(T.alloc(&dwinfo, nwruns));
  GG_CUDA(cudaMemcpyAsync(dslice0, hslice0.data(), nseg * sizeof(int32_t), cudaMemcpyHostToDevice,
                          ctx->stream));
  GG_CUDA(cudaMemcpyAsync(dwide0, hwide0.data(), nseg * sizeof(int32_t), cudaMemcpyHostToDevice,
                          ctx->stream));
  k_hw_widths<<<hw_grid(ctx, nseg), 256, 0, ctx->stream>>>(nseg, segcnt, dnwide, drun0, dslice0, order,
                                                          rcnt, dwidth);
  k_hw_wideinfo<<<hw_grid(ctx, nseg), 256, 0, ctx->stream>>>(nseg, dnwide, dwide0, drun0, order, rcnt,
                                                            ukey, pg, dwinfo);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> width(nslices);
  std::vector<int2> winfo(nwruns);
  GG_CUDA(cudaMemcpyAsync(width.data(), dwidth, nslices * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GG_CUDA(cudaMemcpyAsync(winfo.data(), dwinfo, nwruns * sizeof(int2), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  // 4. host: the cost of every (group, window), the units, then the entry offsets of
  //    the runs and slices and the work items per (group, warp, window)
  const int64_t nsegall = (int64_t)ngroups * kHwWarps * nwin;
  std::vector<double> cost((size_t)ngroups * nwin, 0.0);
  for (int64_t c = 0; c < nseg; ++c) {
    const int64_t sid = (int64_t)hseg[c];
    const int64_t g = sid / (kHwWarps * nwin), w = sid % nwin;
    double& cw = cost[g * nwin + w];  // in entry rows (32 entries) of work
    for (int64_t k = hwide0[c]; k < hwide0[c] + hnwide[c]; ++k) cw += winfo[k].x / 32.0 + 4.0;
    for (int64_t sl = hslice0[c]; sl < hslice0[c] + (hsegcnt[c] - hnwide[c] + 31) / 32; ++sl)
      cw += width[sl] + 2.0;
  }
  // units: each group's windows cut into ranges of about equal cost (every window
  // also costs its copy and the warps' waits on it), about kHwUnitsPerSm per SM in
  // all; a window costlier than that is a unit of its own, split by group warp
  double tot = 0.0;
  for (auto& v : cost) v += kHwWinCost, tot += v;
  const double target = tot / ((double)ctx->num_sms * kHwUnitsPerSm);
  std::vector<int4> units;
  std::vector<double> ucost;
  std::vector<int32_t> gptr(ngroups + 1);
  std::vector<int32_t> wunit((size_t)ngroups * nwin);  // the unit range holding (group, window)
  int nslot = 0;
  for (int g = 0; g < ngroups; ++g) {
    gptr[g] = nslot;
    int64_t wb = 0;
    double acc = 0.0;
    auto flush = [&](int64_t we) {
      if (we > wb) {
        for (int64_t w = wb; w < we; ++w) wunit[g * nwin + w] = nslot;
        units.push_back(make_int4(g | (5 << 21), (int)wb, (int)we, nslot++));
        ucost.push_back(acc);
      }
      wb = we;
      acc = 0.0;
    };
    for (int64_t w = 0; w < nwin; ++w) {
      const double cw = cost[g * nwin + w];
      if (cw > target) {
        flush(w);
        int lg = 5;
        while (lg > 0 && cw / (double)(1 << (5 - lg)) > target) --lg;
        wunit[g * nwin + w] = nslot;
        for (int k = 0; k < (1 << (5 - lg)); ++k) {
          units.push_back(make_int4(g | ((k << lg) << 16) | (lg << 21), (int)w, (int)(w + 1), nslot));
          ucost.push_back(cw / (double)(1 << (5 - lg)));
        }
        ++nslot;
        wb = w + 1;
        continue;
      }
      acc += cw;
      if (acc >= target) flush(w + 1);
    }
    flush(nwin);
  }
  gptr[ngroups] = nslot;
  // items of every (group, warp) in window order: runs and wide slices one each;
  // narrow slices packed kHwNarrow entry rows at a time, across up to kHwBufs
  // consecutive windows of one unit
  std::vector<int32_t> soff(nslices), woff(nwruns);
  std::vector<int4> items;
  std::vector<int32_t> itemptr(nsegall + 1, 0);
  int64_t eoff = 0, c = 0;
  // an open narrow item holds its place in the list from its first slice on, so it
  // precedes the items of the later windows it reaches into
  int gfirst = -1, gcount = 0, gtotal = 0;
  int64_t gwin = -1, gunit = -1, gidx = -1;
  uint32_t gbnd = 0, goffs = 0;
  auto flush = [&]() {
    if (gcount > 0)
      items[gidx] = make_int4(soff[gfirst], gfirst * 32, (int)(0x80000000u | ((uint32_t)gtotal << 8)),
                              (int)(gbnd | (goffs << 8)));
    gfirst = -1;
    gcount = 0;
    gtotal = 0;
    gbnd = 0;
    goffs = 0;
  };
  for (int64_t sid = 0; sid < nsegall; ++sid) {
    const int64_t g = sid / (kHwWarps * nwin), w = sid % nwin;
    if (w == 0) flush();  // next (group, warp)
    const int64_t un = wunit[g * nwin + w];
    if (gcount > 0 && (un != gunit || w - gwin >= kHwBufs)) flush();
    itemptr[sid] = (int32_t)items.size();
    if (c >= nseg || hseg[c] != (uint64_t)sid) continue;
    // runs: one item each, the warp's lanes over the run's entries
    if (hnwide[c] > 0) flush();
    for (int64_t k = hwide0[c]; k < hwide0[c] + hnwide[c]; ++k) {
      woff[k] = (int32_t)eoff;
      items.push_back(make_int4((int)eoff, winfo[k].y, winfo[k].x, -1));
      eoff += (winfo[k].x + 3) / 4 * 4;  // 4-entry aligned starts
    }
    const int64_t s0 = hslice0[c], s1 = s0 + (hsegcnt[c] - hnwide[c] + 31) / 32;
    for (int64_t sl = s0; sl < s1; ++sl) {
      const int wd = width[sl];
      soff[sl] = (int32_t)eoff;
      eoff += (int64_t)wd * 32;
      if (wd <= kHwNarrow) {
        if (gcount == kHwNarrow || gtotal + wd > kHwNarrow) flush();
        if (gcount == 0) {
          gfirst = (int)sl;
          gwin = w;
          gunit = un;
          gidx = (int64_t)items.size();
          items.push_back(make_int4(0, 0, 0, 0));
        }
        gbnd |= 1u << gtotal;
        for (int u = gtotal; u < gtotal + wd; ++u) goffs |= (uint32_t)(w - gwin) << (2 * u);
        gtotal += wd;
        ++gcount;
      } else {
        // quad slice: each lane's entries in groups of 4, [step][lane][4]
        flush();
        const int w4 = (wd + 3) / 4;
        eoff += (int64_t)w4 * 128 - (int64_t)wd * 32;
        items.push_back(make_int4(soff[sl], (int)(sl * 32), w4, -2));
      }
    }
    ++c;
  }
  flush();
  itemptr[nsegall] = (int32_t)items.size();
  if (eoff >= ((int64_t)1 << 31) - 4096) return GG_OK;
  // units to CTAs: most expensive first, each to the least loaded CTA; a CTA runs its
  // units in that order
  const int grid = (int)std::min<int64_t>(ctx->num_sms, (int64_t)units.size());
  std::vector<int> uo(units.size());
  for (size_t i = 0; i < uo.size(); ++i) uo[i] = (int)i;
  std::stable_sort(uo.begin(), uo.end(), [&](int a, int b) { return ucost[a] > ucost[b]; });
  std::vector<std::vector<int>> per(grid);
  {
    std::vector<std::pair<double, int>> heap;
    for (int b = 0; b < grid; ++b) heap.push_back({0.0, b});
    auto cmp = [](const std::pair<double, int>& x, const std::pair<double, int>& y) {
      return x.first > y.first || (x.first == y.first && x.second > y.second);
    };
    std::make_heap(heap.begin(), heap.end(), cmp);
    for (int i : uo) {
      std::pop_heap(heap.begin(), heap.end(), cmp);
      auto& top = heap.back();
      per[top.second].push_back(i);
      top.first += ucost[i];
      std::push_heap(heap.begin(), heap.end(), cmp);
    }
  }
  std::vector<int4> units_sorted;
  std::vector<int32_t> cptr(grid + 1, 0);
  for (int b = 0; b < grid; ++b) {
    cptr[b] = (int32_t)units_sorted.size();
    for (int i : per[b]) units_sorted.push_back(units[i]);
  }
  cptr[grid] = (int32_t)units_sorted.size();
  // 5. device layout
  int32_t *dsoff = nullptr, *dwoff = nullptr;
  GG_CUDA(T.alloc(&dsoff, nslices));
  GG_CUDA(T.alloc(&dwoff, nwruns));
  GG_CUDA(cudaMemcpyAsync(dsoff, soff.data(), nslices * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(dwoff, woff.data(), nwruns * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
  cudaError_t e = cudaMalloc((void**)&P->col, (size_t)(eoff > 0 ? eoff : 1) * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->val, (size_t)(eoff > 0 ? eoff : 1) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->rowid, (size_t)(nslices > 0 ? nslices : 1) * 32 * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->items, (items.size() + 1) * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->itemptr, (nsegall + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->units, (units.size() + 1) * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->cptr, (grid + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->gptr, (ngroups + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&P->partials, (size_t)nslot * pg * sizeof(float));
  if (e != cudaSuccess) {
    free_hubwin_plan(S);
    S->hubwin = new HubWinPlan();
    return cuda_error(e, "hub-row window layout");
  }
  k_hw_fill_u16<<<hw_grid(ctx, eoff), 256, 0, ctx->stream>>>(P->col, eoff, (uint16_t)kHwCols);
  GG_CUDA(cudaMemsetAsync(P->val, 0, (size_t)eoff * sizeof(float), ctx->stream));
  GG_CUDA(cudaMemsetAsync(P->rowid, 0xff, (size_t)nslices * 32 * sizeof(uint16_t), ctx->stream));
  GG_CUDA(cudaMemcpyAsync(P->items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice,
                          ctx->stream));
  GG_CUDA(cudaMemcpyAsync(P->itemptr, itemptr.data(), (nsegall + 1) * sizeof(int32_t),
                          cudaMemcpyHostToDevice, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(P->cptr, cptr.data(), (grid + 1) * sizeof(int32_t), cudaMemcpyHostToDevice,
                          ctx->stream));
  GG_CUDA(cudaMemcpyAsync(P->units, units_sorted.data(), units.size() * sizeof(int4),
                          cudaMemcpyHostToDevice, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(P->gptr, gptr.data(), (ngroups + 1) * sizeof(int32_t), cudaMemcpyHostToDevice,
                          ctx->stream));
  k_hw_fill<<<hw_grid(ctx, nr), 256, 0, ctx->stream>>>(
      nr, nseg, pg, nwin, drun0, dnwide, dwide0, dwoff, dslice0, dsoff, dwidth, order, ukey, rcnt, rstart,
      vals2, S->colperm->colval_r, static_cast<const float*>(S->nzval), P->col, P->val, P->rowid);
  GG_CUDA(cudaGetLastError());
  SellPlan* rest = nullptr;
  GG_CHECK(build_sell_plan_from(ctx, S, np / 32, &rest));  // synchronises the stream
  P->rest = rest;
  P->np = np;
  P->pg = pg;
  P->ngroups = ngroups;
  P->nwin = nwin;
  P->nunits = (int64_t)units.size();
  P->grid = grid;
  P->nitems = (int64_t)items.size();
  P->nslices = nslices;
  P->nentries = eoff;
  P->enabled = true;
  return GG_OK;
}

int launch_hubwin(gg_ctx* ctx, gg_mat* S, const float* xr, float* y) {
  HubWinPlan* P = S->hubwin;
  const size_t smem = hw_smem(P->pg);
  static bool attr_set[64] = {false};
  if (ctx->device < 64 && !attr_set[ctx->device]) {
    GG_CUDA(cudaFuncSetAttribute(k_hubwin, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)hw_smem(kHwMaxRows)));
    attr_set[ctx->device] = true;
  }
  k_hubwin<<<P->grid, kHwThreads, smem, ctx->stream>>>(xr, P->col, P->val, P->rowid, P->items, P->itemptr,
                                                        P->units, P->cptr, (int)P->nwin, P->pg,
                                                        P->partials, ctx->d_err, copy_polls(ctx));
  k_hw_combine<<<hw_grid(ctx, P->np), 256, 0, ctx->stream>>>(P->np, P->pg, P->gptr, P->partials,
                                                             S->sigma > 1 ? S->perm : nullptr, y);
  trace_count(ctx, 2);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

extern "C" int64_t gg_spmv_hub_rows(const gg_mat* A) {
  if (!A) return 0;
  const gg_mat* S = A->format == GG_FMT_CSR ? A->sell_copy : A;
  return (S && S->hubwin && S->hubwin->enabled) ? S->hubwin->np : 0;
}
