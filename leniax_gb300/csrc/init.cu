// Initial states generated on the device, one block per (world, init):
// leniax's initializations (initializations.py:10-116) with the Perlin noise
// of perlin.py:16-71 and make_array_compressible (loader.py:16-30).
//
// Random numbers come from a counter-based SplitMix64 hash (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", 2014) of the
// world's seed and the element index: the same construction and
// distributions as leniax, not JAX's threefry stream.
#include <algorithm>
#include <cstdarg>
#include <cstdio>

#include "common.cuh"
#include "engine.h"

using namespace lgx;

namespace {

int ifail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return api_error(code, buf);
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// uniform [0, 1) from the top 24 bits of the hash of (seed, stream, index)
__device__ __forceinline__ float uniform01(uint64_t seed, uint64_t stream, uint64_t idx) {
  const uint64_t h = splitmix64(seed ^ splitmix64(stream * 0xD1B54A32D192ED03ull + idx));
  return (float)(h >> 40) * (1.f / 16777216.f);
}

constexpr float kMaxVal = 12543.f;  // NB_CHARS^2 - 1 with NB_CHARS = 112 (constant.py:13)

__device__ __forceinline__ float compressible(float v) { return rintf(v * kMaxVal) / kMaxVal; }

__device__ __forceinline__ float perlin_fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }

struct InitArgs {
  int kind, n_worlds, nb_init, H, W, compress;
  int res0, res1, d0, d1, diff0, diff1;  // Perlin periods, cells per period, repeat offsets
  const uint64_t* seeds;
  const float* gf_m;
  float* out;
  const float* angles;  // [n_worlds, nb_init, res0, res1] or null (drawn from the seeds)
};

// Perlin value at (y, x) of init `i` (perlin.py:16-71 with leniax's
// repeat-and-slice gradient lookup, which stays valid when the shape is not a
// multiple of the periods).
__device__ __forceinline__ float perlin_at(const InitArgs& a, uint64_t seed, int world, int i, int y, int x) {
  const float gy = fmodf((float)y * ((float)a.res0 / (float)a.H), 1.f);
  const float gx = fmodf((float)x * ((float)a.res1 / (float)a.W), 1.f);
  const int y0 = y / a.d0, y1 = ((y + a.diff0) / a.d0) % a.res0;  // row a.res0 wraps to 0
  const int x0 = x / a.d1, x1 = ((x + a.diff1) / a.d1) % a.res1;
  auto grad = [&](int cy, int cx, float& c, float& s) {
    const float ang = a.angles ? __ldg(a.angles + (((size_t)world * a.nb_init + i) * a.res0 + cy) * a.res1 + cx)
                               : 6.283185307179586f * uniform01(seed, 1 + i, (uint64_t)cy * a.res1 + cx);
    sincosf(ang, &s, &c);
  };
  float c00, s00, c10, s10, c01, s01, c11, s11;
  grad(y0 % a.res0, x0 % a.res1, c00, s00);
  grad(y1, x0 % a.res1, c10, s10);
  grad(y0 % a.res0, x1, c01, s01);
  grad(y1, x1, c11, s11);
  const float n00 = gy * c00 + gx * s00;
  const float n10 = (gy - 1.f) * c10 + gx * s10;
  const float n01 = gy * c01 + (gx - 1.f) * s01;
  const float n11 = (gy - 1.f) * c11 + (gx - 1.f) * s11;
  const float t0 = perlin_fade(gy), t1 = perlin_fade(gx);
  const float n0 = n00 * (1.f - t0) + t0 * n10;
  const float n1 = n01 * (1.f - t0) + t0 * n11;
  return 1.4142135623730951f * ((1.f - t1) * n0 + t1 * n1);
}

__global__ void init_kernel(InitArgs a) {
  const int wi = blockIdx.x;  // world * nb_init + init
  const int world = wi / a.nb_init, i = wi % a.nb_init;
  const uint64_t seed = a.seeds[world];
  const long cells = (long)a.H * a.W;
  float* out = a.out + (size_t)wi * cells;
  if (a.kind == LGX_INIT_RANDOM_UNIFORM) {
    // maxval = linspace(0.4, 1, nb_init)[i]; uniform in [0, maxval)  (initializations.py:10-32)
    const float maxv = a.nb_init > 1 ? 0.4f + 0.6f * (float)i / (float)(a.nb_init - 1) : 0.4f;
    for (long c = threadIdx.x; c < cells; c += blockDim.x) {
      float v = maxv * uniform01(seed, 0x5EED0000ull + i, (uint64_t)c);
      out[c] = a.compress ? compressible(v) : v;
    }
    return;
  }
  // Perlin (initializations.py:35-77): noise, per-init min / max normalisation, scaling
  float lo = 3.4e38f, hi = -3.4e38f;
  for (long c = threadIdx.x; c < cells; c += blockDim.x) {
    const float v = perlin_at(a, seed, world, i, (int)(c / a.W), (int)(c % a.W));
    out[c] = v;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  __shared__ float smin[32], smax[32];
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    smin[threadIdx.x >> 5] = lo;
    smax[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    lo = threadIdx.x < nw ? smin[threadIdx.x] : 3.4e38f;
    hi = threadIdx.x < nw ? smax[threadIdx.x] : -3.4e38f;
    for (int o = 16; o > 0; o >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (threadIdx.x == 0) {
      smin[0] = lo;
      smax[0] = hi;
    }
  }
  __syncthreads();
  lo = smin[0];
  const float span = smax[0] - lo;
  // scaling_i = m + i / nb_init * (min(1, 3m) - m), m = gf_params[0] of the first kernel
  const float m = a.gf_m[world];
  const float scale = m + (float)i / (float)a.nb_init * (fminf(1.f, 3.f * m) - m);
  for (long c = threadIdx.x; c < cells; c += blockDim.x) {
    float v = out[c] - lo;
    v = span > 0.f ? v / span : v;
    v *= scale;
    out[c] = v;
  }
}

// cropped_perlin (initializations.py:80-116): keep the (2 kr)^2 square at
// rows / columns [24, 24 + 2 kr) of the Perlin state and centre it on a zero
// 128 x 128 world (pad_left = (128 - 2 kr) // 2).  One block per (world, init).
__global__ void crop_kernel(int H, int W, int crop, int pad_left, float* out, float* tmp, int compress) {
  const long cells = (long)H * W;
  float* o = out + (size_t)blockIdx.x * cells;
  float* t = tmp + (size_t)blockIdx.x * cells;
  for (long c = threadIdx.x; c < cells; c += blockDim.x) t[c] = o[c];
  __syncthreads();
  for (long c = threadIdx.x; c < cells; c += blockDim.x) {
    const int y = (int)(c / W), x = (int)(c % W);
    const int sy = y - pad_left, sx = x - pad_left;
    float v = 0.f;
    if (sy >= 0 && sy < crop && sx >= 0 && sx < crop) v = t[(size_t)(24 + sy) * W + 24 + sx];
    o[c] = compress ? compressible(v) : v;
  }
}

__global__ void compress_kernel(long n, float* out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = compressible(out[i]);
}

}  // namespace

extern "C" {

int lgx_init_cells_workspace_bytes(const lgx_init_job* j, size_t* bytes) {
  if (!j || !bytes) return ifail(LGX_ERR_INVALID, "lgx_init_cells_workspace_bytes: null argument");
  *bytes = j->kind == LGX_INIT_CROPPED_PERLIN ? (size_t)j->n_worlds * j->nb_init * j->H * j->W * sizeof(float) : 0;
  return LGX_OK;
}

int lgx_init_cells(const lgx_init_job* j, void* ws, size_t ws_bytes, void* stream) {
  if (!j) return ifail(LGX_ERR_INVALID, "lgx_init_cells: null job");
  if (j->kind < LGX_INIT_RANDOM_UNIFORM || j->kind > LGX_INIT_CROPPED_PERLIN)
    return ifail(LGX_ERR_UNSUPPORTED, "lgx_init_cells: unknown initialisation %d", j->kind);
  if (j->n_worlds < 1 || j->nb_init < 1 || j->H < 1 || j->W < 1)
    return ifail(LGX_ERR_INVALID, "lgx_init_cells: bad shape (%d worlds, %d inits, %dx%d)", j->n_worlds, j->nb_init,
                 j->H, j->W);
  if (!j->seeds || !j->out) return ifail(LGX_ERR_INVALID, "lgx_init_cells: null tensor");
  InitArgs a;
  a.kind = j->kind;
  a.n_worlds = j->n_worlds;
  a.nb_init = j->nb_init;
  a.H = j->H;
  a.W = j->W;
  a.compress = j->compressible;
  a.seeds = reinterpret_cast<const uint64_t*>(j->seeds);
  a.gf_m = j->gf_m;
  a.out = j->out;
  a.angles = j->angles;
  a.res0 = a.res1 = a.d0 = a.d1 = 1;
  a.diff0 = a.diff1 = 0;
  int kr = 0;
  if (j->kind != LGX_INIT_RANDOM_UNIFORM) {
    if (!j->gf_m) return ifail(LGX_ERR_INVALID, "lgx_init_cells: Perlin initialisations need gf_m");
    if (!(j->R > 0.f)) return ifail(LGX_ERR_INVALID, "lgx_init_cells: R must be > 0");
    kr = (int)ceilf(j->R);
    a.res0 = j->H / (kr * 3);
    a.res1 = j->W / (kr * 2);
    if (a.res0 < 1 || a.res1 < 1)
      return ifail(LGX_ERR_INVALID, "lgx_init_cells: world %dx%d too small for Perlin periods of R=%g", j->H, j->W,
                   (double)j->R);
    a.d0 = j->H / a.res0;
    a.d1 = j->W / a.res1;
    a.diff0 = (a.res0 + 1) * a.d0 - j->H;
    a.diff1 = (a.res1 + 1) * a.d1 - j->W;
    if (j->kind == LGX_INIT_CROPPED_PERLIN) {
      if (j->H != 128 || j->W != 128)
        return ifail(LGX_ERR_UNSUPPORTED, "lgx_init_cells: cropped_perlin is defined on 128x128 worlds");
      if (24 + 2 * kr > 128) return ifail(LGX_ERR_INVALID, "lgx_init_cells: crop of 2*ceil(R) cells exceeds the world");
      const size_t need = (size_t)j->n_worlds * j->nb_init * j->H * j->W * sizeof(float);
      if (!ws || ws_bytes < need) return ifail(LGX_ERR_WORKSPACE, "lgx_init_cells: workspace %zu < %zu", ws_bytes, need);
    }
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int blocks = j->n_worlds * j->nb_init;
  // Perlin values are compressed after cropping (or right after normalisation)
  a.compress = (j->kind == LGX_INIT_RANDOM_UNIFORM) ? j->compressible : 0;
  init_kernel<<<blocks, 256, 0, st>>>(a);
  if (j->kind == LGX_INIT_CROPPED_PERLIN) {
    const int crop = 2 * kr;
    const int pad_left = (128 - crop) / 2;
    crop_kernel<<<blocks, 256, 0, st>>>(j->H, j->W, crop, pad_left, j->out, static_cast<float*>(ws), j->compressible);
  } else if (j->kind == LGX_INIT_PERLIN && j->compressible) {
    const long n = (long)blocks * j->H * j->W;
    compress_kernel<<<(unsigned)std::min<long>((n + 255) / 256, 8192), 256, 0, st>>>(n, j->out);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ifail(LGX_ERR_CUDA, "lgx_init_cells: %s", cudaGetErrorString(e));
  return LGX_OK;
}

}  // extern "C"
