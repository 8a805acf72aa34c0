// gg_gen.cu -- seeded synthetic graph generators (device side).
//
// Definition (identical to the CPU copy used for checking):
//   splitmix64(z): z += 0x9E3779B97F4A7C15; z = (z ^ z>>30) * 0xBF58476D1CE4E5B9;
//                  z = (z ^ z>>27) * 0x94D049BB133111EB; return z ^ z>>31
//   draw(seed, e, j) = splitmix64(splitmix64(seed) + 64*e + j)    (mod 2^64)
//   u01_f32(r) = (r >> 40) * 2^-24,  u01_f64(r) = (r >> 11) * 2^-53
//   R-MAT edge e: per level l < scale, u = u01_f64(draw(e, l)) picks quadrant
//     (0,0) u < t1, (0,1) u < t2, (1,0) u < t3, (1,1) otherwise (t1 = a, t2 = a+b,
//     t3 = a+b+c); src = 2 src + row bit, dst = 2 dst + column bit.
//   Erdos-Renyi edge e: src = ((draw(e,0) >> 32) * n) >> 32, dst from draw(e,1).
//   Grid H x W: horizontal edge e = i*(W-1)+j joins (i,j)-(i,j+1), vertical edge
//     e = H*(W-1) + i*W + j joins (i,j)-(i+1,j); vertex id i*W + j.
//   Weight of edge e from r = draw(e, 63): GG_W_PATTERN Bool true; GG_W_U01_F32
//     u01_f32(r); GG_W_INT_1_255 1 + ((r >> 32) mod 255); GG_W_F32_1_10
//     (float)(1 + 9 u01_f64(r)).
//   Dense vector element i: u01_f32(draw(seed, i, 0)).
// Vertex ids are written 1-based.
#include "gg_common.cuh"

namespace gg {

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__host__ inline uint64_t splitmix64_h(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t draw(uint64_t base, uint64_t e, uint64_t j) {
  return splitmix64(base + 64ULL * e + j);
}
__device__ __forceinline__ float u01_f32(uint64_t r) {
  return __fmul_rn((float)(r >> 40), 1.0f / 16777216.0f);
}
__device__ __forceinline__ double u01_f64(uint64_t r) {
  return __dmul_rn((double)(r >> 11), 1.0 / 9007199254740992.0);
}

__device__ __forceinline__ void put_weight(int kind, uint64_t r, void* w, int64_t e) {
  switch (kind) {
    case GG_W_PATTERN: static_cast<uint8_t*>(w)[e] = 1; break;
    case GG_W_U01_F32: static_cast<float*>(w)[e] = u01_f32(r); break;
    case GG_W_INT_1_255: static_cast<int32_t*>(w)[e] = 1 + (int32_t)((r >> 32) % 255ULL); break;
    default: static_cast<float*>(w)[e] = (float)__dadd_rn(1.0, __dmul_rn(9.0, u01_f64(r))); break;
  }
}

__global__ void k_gen_rmat(int scale, int64_t ne, double t1, double t2, double t3, uint64_t base,
                           int wkind, int32_t* src, int32_t* dst, void* w) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    uint64_t s = 0, d = 0;
    for (int l = 0; l < scale; ++l) {
      const double u = u01_f64(draw(base, (uint64_t)e, (uint64_t)l));
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
    if (w) put_weight(wkind, draw(base, (uint64_t)e, 63), w, e);
  }
}

__global__ void k_gen_er(int64_t n, int64_t ne, uint64_t base, int wkind, int32_t* src,
                         int32_t* dst, void* w) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r0 = draw(base, (uint64_t)e, 0), r1 = draw(base, (uint64_t)e, 1);
    src[e] = (int32_t)((((r0 >> 32) * (uint64_t)n) >> 32) + 1);
    dst[e] = (int32_t)((((r1 >> 32) * (uint64_t)n) >> 32) + 1);
    if (w) put_weight(wkind, draw(base, (uint64_t)e, 63), w, e);
  }
}

__global__ void k_gen_grid(int64_t H, int64_t W, uint64_t base, int wkind, int32_t* src,
                           int32_t* dst, void* w) {
  const int64_t nh = H * (W - 1), nv = (H - 1) * W;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nh + nv;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t a, b;
    if (e < nh) {
      const int64_t i = e / (W - 1), j = e % (W - 1);
      a = i * W + j;
      b = a + 1;
    } else {
      const int64_t f = e - nh, i = f / W, j = f % W;
      a = i * W + j;
      b = a + W;
    }
    src[e] = (int32_t)(a + 1);
    dst[e] = (int32_t)(b + 1);
    if (w) put_weight(wkind, draw(base, (uint64_t)e, 63), w, e);
  }
}

__global__ void k_gen_uniform_f32(int64_t len, uint64_t base, float* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = u01_f32(draw(base, (uint64_t)i, 0));
}

static int gen_grid_size(gg_ctx* ctx, int64_t work) {
  int64_t g = (work + 255) / 256;
  const int64_t cap = (int64_t)ctx->num_sms * 32;
  return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_gen_rmat_edges(gg_ctx* ctx, int scale, int64_t nedges, double a, double b, double c,
                      uint64_t seed, int weight_kind, int32_t* src, int32_t* dst, void* weights) {
  if (!ctx || !src || !dst) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (scale < 1 || scale > 30) return set_error(GG_ERR_ARGUMENT, "scale must be in 1..30");
  if (nedges <= 0) return GG_OK;
  GG_CUDA(cudaSetDevice(ctx->device));
  const double t1 = a, t2 = a + b, t3 = a + b + c;
  k_gen_rmat<<<gen_grid_size(ctx, nedges), 256, 0, ctx->stream>>>(
      scale, nedges, t1, t2, t3, splitmix64_h(seed), weight_kind, src, dst, weights);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

int gg_gen_er_edges(gg_ctx* ctx, int64_t n, int64_t nedges, uint64_t seed, int weight_kind,
                    int32_t* src, int32_t* dst, void* weights) {
  if (!ctx || !src || !dst) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (n < 1 || n > INT32_MAX) return set_error(GG_ERR_ARGUMENT, "n out of range");
  if (nedges <= 0) return GG_OK;
  GG_CUDA(cudaSetDevice(ctx->device));
  k_gen_er<<<gen_grid_size(ctx, nedges), 256, 0, ctx->stream>>>(
      n, nedges, splitmix64_h(seed), weight_kind, src, dst, weights);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

int gg_gen_grid_edges(gg_ctx* ctx, int64_t H, int64_t W, uint64_t seed, int weight_kind,
                      int32_t* src, int32_t* dst, void* weights) {
  if (!ctx || !src || !dst) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (H < 1 || W < 1 || H * W > INT32_MAX) return set_error(GG_ERR_ARGUMENT, "grid size out of range");
  const int64_t ne = H * (W - 1) + (H - 1) * W;
  if (ne <= 0) return GG_OK;
  GG_CUDA(cudaSetDevice(ctx->device));
  k_gen_grid<<<gen_grid_size(ctx, ne), 256, 0, ctx->stream>>>(H, W, splitmix64_h(seed),
                                                              weight_kind, src, dst, weights);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

int gg_gen_uniform_f32(gg_ctx* ctx, int64_t len, uint64_t seed, float* out) {
  if (!ctx || (len > 0 && !out)) return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (len <= 0) return GG_OK;
  GG_CUDA(cudaSetDevice(ctx->device));
  k_gen_uniform_f32<<<gen_grid_size(ctx, len), 256, 0, ctx->stream>>>(len, splitmix64_h(seed), out);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // extern "C"
