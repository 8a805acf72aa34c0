/*
 * gen.c -- CPU copy of the seeded synthetic graph generators and of the CSR
 * assembly rule, used to check the CUDA generators and to build inputs for the CPU
 * baseline.  TEST INFRASTRUCTURE ONLY (see oracle.c).
 *
 * Generator definition (shared with gpugraphs.jl_gb300/csrc/gg_gen.cu):
 *   splitmix64(z): z += 0x9E3779B97F4A7C15; z = (z ^ z>>30) * 0xBF58476D1CE4E5B9;
 *                  z = (z ^ z>>27) * 0x94D049BB133111EB; return z ^ z>>31
 *   draw(seed, e, j) = splitmix64(splitmix64(seed) + 64*e + j)       (mod 2^64)
 *   u01_f32(r) = (r >> 40) * 2^-24,  u01_f64(r) = (r >> 11) * 2^-53
 *   R-MAT edge e: for level l < scale, u = u01_f64(draw(e, l)); quadrant (0,0) if
 *     u < t1, (0,1) if u < t2, (1,0) if u < t3, else (1,1); src = 2 src + row bit,
 *     dst = 2 dst + column bit (t1 = a, t2 = a+b, t3 = a+b+c).
 *   Erdos-Renyi edge e: src = ((draw(e,0) >> 32) * n) >> 32, dst likewise with draw(e,1).
 *   Grid H x W, 4-neighbour: horizontal edge e = i*(W-1)+j joins (i,j)-(i,j+1),
 *     vertical edge e = H*(W-1) + i*W + j joins (i,j)-(i+1,j); vertex id i*W+j.
 *   Weight of edge e from r = draw(e, 63): kind 0 Bool true; 1 u01_f32(r) (Float32);
 *     2 1 + ((r >> 32) mod 255) (Int32); 3 (float)(1 + 9*u01_f64(r)) (Float32).
 *   Dense vector element i: u01_f32(draw(seed, i, 0)).
 * CSR assembly: entries in generation order (edge e, then its mirror when
 * symmetrising), self-loops optionally dropped, stable sort by (row, column), the
 * first entry of each duplicate (row, column) kept.  All ids 1-based in the output.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static inline uint64_t draw(uint64_t base, uint64_t e, uint64_t j) {
  return splitmix64(base + 64ULL * e + j);
}

static inline float u01_f32(uint64_t r) { return (float)(r >> 40) * (1.0f / 16777216.0f); }
static inline double u01_f64(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

static void weight(int kind, uint64_t r, void* w, int64_t e) {
  switch (kind) {
    case 0: ((uint8_t*)w)[e] = 1; break;
    case 1: ((float*)w)[e] = u01_f32(r); break;
    case 2: ((int32_t*)w)[e] = 1 + (int32_t)((r >> 32) % 255ULL); break;
    default: ((float*)w)[e] = (float)(1.0 + 9.0 * u01_f64(r)); break;
  }
}

void orc_gen_rmat(int scale, int64_t nedges, double t1, double t2, double t3, uint64_t seed,
                  int wkind, int32_t* src, int32_t* dst, void* w) {
  uint64_t base = splitmix64(seed);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nedges; ++e) {
    uint64_t s = 0, d = 0;
    for (int l = 0; l < scale; ++l) {
      double u = u01_f64(draw(base, (uint64_t)e, (uint64_t)l));
      int rb, cb;
      if (u < t1) { rb = 0; cb = 0; }
      else if (u < t2) { rb = 0; cb = 1; }
      else if (u < t3) { rb = 1; cb = 0; }
      else { rb = 1; cb = 1; }
      s = 2 * s + (uint64_t)rb;
      d = 2 * d + (uint64_t)cb;
    }
    src[e] = (int32_t)(s + 1);
    dst[e] = (int32_t)(d + 1);
    weight(wkind, draw(base, (uint64_t)e, 63), w, e);
  }
}

void orc_gen_er(int64_t n, int64_t nedges, uint64_t seed, int wkind, int32_t* src,
                int32_t* dst, void* w) {
  uint64_t base = splitmix64(seed);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nedges; ++e) {
    uint64_t r0 = draw(base, (uint64_t)e, 0), r1 = draw(base, (uint64_t)e, 1);
    src[e] = (int32_t)((((r0 >> 32) * (uint64_t)n) >> 32) + 1);
    dst[e] = (int32_t)((((r1 >> 32) * (uint64_t)n) >> 32) + 1);
    weight(wkind, draw(base, (uint64_t)e, 63), w, e);
  }
}

/* number of undirected grid edges: H*(W-1) + (H-1)*W */
void orc_gen_grid(int64_t H, int64_t W, uint64_t seed, int wkind, int32_t* src, int32_t* dst,
                  void* w) {
  uint64_t base = splitmix64(seed);
  int64_t nh = H * (W - 1), nv = (H - 1) * W;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nh + nv; ++e) {
    int64_t i, j, a, b;
    if (e < nh) { i = e / (W - 1); j = e % (W - 1); a = i * W + j; b = a + 1; }
    else { int64_t f = e - nh; i = f / W; j = f % W; a = i * W + j; b = a + W; }
    src[e] = (int32_t)(a + 1);
    dst[e] = (int32_t)(b + 1);
    weight(wkind, draw(base, (uint64_t)e, 63), w, e);
  }
}

void orc_gen_uniform_f32(int64_t len, uint64_t seed, float* out) {
  uint64_t base = splitmix64(seed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < len; ++i) out[i] = u01_f32(draw(base, (uint64_t)i, 0));
}

typedef struct {
  int32_t col;
  int64_t ord;
  int64_t src_edge;
} ent;

static int ent_cmp(const void* a, const void* b) {
  const ent* x = (const ent*)a;
  const ent* y = (const ent*)b;
  if (x->col != y->col) return x->col < y->col ? -1 : 1;
  return x->ord < y->ord ? -1 : (x->ord > y->ord);
}

/*
 * COO (1-based, generation order) -> CSR of the n x n matrix with A[src, dst] set.
 * symmetrize: also A[dst, src]; drop_loops: skip src == dst.  Two-pass API: call
 * with colval == NULL to get the nnz after deduplication in *nnz_out, then again
 * with outputs of that size.  esz = bytes per weight (1, 4 or 8).
 */
int orc_coo_to_csr(int64_t n, int64_t ne, const int32_t* src, const int32_t* dst, const void* w,
                   int esz, int symmetrize, int drop_loops, int32_t* rowptr, int32_t* colval,
                   void* nzval, int64_t* nnz_out) {
  int64_t cap = symmetrize ? 2 * ne : ne;
  int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  for (int64_t e = 0; e < ne; ++e) {
    if (drop_loops && src[e] == dst[e]) continue;
    cnt[src[e]]++;
    if (symmetrize) cnt[dst[e]]++;
  }
  for (int64_t r = 1; r <= n; ++r) cnt[r] += cnt[r - 1];
  int64_t total = cnt[n];
  ent* ents = (ent*)malloc((size_t)(total > 0 ? total : 1) * sizeof(ent));
  int64_t* pos = (int64_t*)malloc(((size_t)n + 1) * sizeof(int64_t));
  memcpy(pos, cnt, ((size_t)n + 1) * sizeof(int64_t));
  for (int64_t e = 0; e < ne; ++e) {
    if (drop_loops && src[e] == dst[e]) continue;
    int64_t r = src[e] - 1;
    ents[pos[r]].col = dst[e]; ents[pos[r]].ord = 2 * e; ents[pos[r]].src_edge = e; pos[r]++;
    if (symmetrize) {
      r = dst[e] - 1;
      ents[pos[r]].col = src[e]; ents[pos[r]].ord = 2 * e + 1; ents[pos[r]].src_edge = e; pos[r]++;
    }
  }
  (void)cap;
  int64_t* keep = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t r = 0; r < n; ++r) {
    int64_t a = cnt[r], b = cnt[r + 1];
    if (b - a > 1) qsort(ents + a, (size_t)(b - a), sizeof(ent), ent_cmp);
    int64_t k = 0;
    for (int64_t i = a; i < b; ++i)
      if (i == a || ents[i].col != ents[i - 1].col) ++k;
    keep[r + 1] = k;
  }
  for (int64_t r = 1; r <= n; ++r) keep[r] += keep[r - 1];
  *nnz_out = keep[n];
  if (colval != NULL) {
    for (int64_t r = 0; r <= n; ++r) rowptr[r] = (int32_t)(keep[r] + 1);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t r = 0; r < n; ++r) {
      int64_t a = cnt[r], b = cnt[r + 1], o = keep[r];
      for (int64_t i = a; i < b; ++i) {
        if (i != a && ents[i].col == ents[i - 1].col) continue;
        colval[o] = ents[i].col;
        memcpy((char*)nzval + (size_t)o * (size_t)esz,
               (const char*)w + (size_t)ents[i].src_edge * (size_t)esz, (size_t)esz);
        ++o;
      }
    }
  }
  free(cnt);
  free(ents);
  free(pos);
  free(keep);
  return 0;
}
