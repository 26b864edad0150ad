// On-device construction of ring kernels and their spectra, a batch at a time
// (one kernel per world of a search, each with its own R, rings and kernel
// function parameters).
//
// Per kernel, leniax's circle_2d (kernels.py:176-212) on the world grid:
//   k_radius_px = ceil(r R); centred = (i - k_radius_px) / (r R) per axis
//   d = |centred|; B = nb d; ring = min(floor(B), nb - 1)
//   K = (d < 1) * kf(params, B mod 1) * b[ring];  K /= sum(K)
// placed as get_kernels_and_mapping does (kernels.py:66-158): the
// 2 k_radius_px box padded to the world with (need // 2) cells before, then
// fftshift; the spectrum is the Hermitian half of fftn (kernels.py:145-152).
// Kernel functions: kernel_functions.py:7-250.  The 3D form takes the same
// distance over three axes.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"
#include "engine.h"
#include "fft.cuh"

using namespace lgx;

namespace {

int kfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return api_error(code, buf);
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

__device__ __forceinline__ float kernel_fn(int id, float q0, float q1, float X) {
  switch (id) {
    case LGX_KF_POLY_QUAD:  // kernel_functions.py:7-37
      return powf(4.f * X * (1.f - X), q0);
    case LGX_KF_GAUSS_BUMP:  // kernel_functions.py:40-69 (separately rounded, as numpy evaluates it)
      return expf(q0 * (q0 - 1.f / __fadd_rn(__fmul_rn(X, 1.f - X), kEps)));
    case LGX_KF_STEP:  // kernel_functions.py:72-102
      return (X >= q0 && X <= 1.f - q0) ? 1.f : 0.f;
    case LGX_KF_GAUSS: {  // kernel_functions.py:105-134
      const float o = (X - q0) / (0.3f * q0);
      return expf(-(o * o) / 2.f);
    }
    case LGX_KF_THRESHOLD:  // kernel_functions.py:137-167
      return X >= q0 ? 1.f : 0.f;
    case LGX_KF_STAIRCASE: {  // kernel_functions.py:170-208 (m = q0, s = q1)
      float o = 0.f;
      if (X >= q0 - q1 && X < q0 - q1 / 2.f) o += 0.5f;
      if (X >= q0 - q1 / 2.f && X <= q0 + q1 / 2.f) o += 1.f;
      if (X > q0 + q1 / 2.f && X <= q0 + q1) o += 0.5f;
      return o;
    }
    default: {  // LGX_KF_TRIANGLE, kernel_functions.py:211-250
      const float left = q0 - q1, right = q0 + q1;
      float o = 0.f;
      if (X >= left && X < q0) o += (X - left) / (q0 - left);
      if (X >= q0 && X <= right) o += (X - right) / (q0 - right);
      return o;
    }
  }
}

struct RingArgs {
  int nd, N, n, kf_id, nb_max;
  const float *R, *r, *b, *kfp;
  const int* nb;
  float* out;    // [n, N^nd]
  float* sums;   // [n]
  int* status;   // nonzero: a kernel box did not fit its world, or a ring count was out of range
};

// value of kernel `k` at output (fftshifted) cell `cell`
__device__ __forceinline__ float ring_value(const RingArgs& a, int k, long cell, int krp, float rR, int pad, int nb) {
  const int N = a.N;
  float s2 = 0.f;
  bool inside = true;
  long rest = cell;
  float cc[3];
  for (int ax = a.nd - 1; ax >= 0; --ax) {
    const int o = (int)(rest % N);
    rest /= N;
    const int p = (o - N / 2 + N) % N;  // unshifted padded index (fftshift rolls by N // 2)
    const int i = p - pad;
    inside = inside && i >= 0 && i < 2 * krp;
    cc[ax] = ((float)i - (float)krp) / rR;
  }
  if (!inside) return 0.f;
  // separately rounded products and sums (no FMA contraction), in numpy's
  // order, so ring and step thresholds fall on the same cells as on the host
  s2 = __fmul_rn(cc[0], cc[0]);
  for (int ax = 1; ax < a.nd; ++ax) s2 = __fadd_rn(s2, __fmul_rn(cc[ax], cc[ax]));
  const float d = sqrtf(s2);
  const float B = (float)nb * d;
  const int ring = min((int)floorf(B), nb - 1);
  const float bs = __ldg(a.b + (size_t)k * a.nb_max + ring);
  const float X = B - floorf(B);
  const float raw = kernel_fn(a.kf_id, __ldg(a.kfp + 2 * k), __ldg(a.kfp + 2 * k + 1), X);
  return (d < 1.f ? 1.f : 0.f) * raw * bs;
}

// one block per kernel: raw values + their sum (fixed reduction order)
__global__ void ring_build_kernel(RingArgs a) {
  const int k = blockIdx.x;
  const int N = a.N;
  long cells = N;
  for (int ax = 1; ax < a.nd; ++ax) cells *= N;
  const double rRd = (double)__ldg(a.r + k) * (double)__ldg(a.R + k);
  const int krp = (int)ceil(rRd);
  const float rR = (float)rRd;
  const int pad = (N - 2 * krp) / 2;
  float* out = a.out + (size_t)k * cells;
  const int nb = __ldg(a.nb + k);
  // the kernel box must fit the world (np.pad would refuse) and the ring count its b row
  if (2 * krp > N || !(rRd > 0.0) || nb < 1 || nb > a.nb_max) {
    for (long c = threadIdx.x; c < cells; c += blockDim.x) out[c] = 0.f;
    if (threadIdx.x == 0) {
      a.sums[k] = 0.f;
      atomicExch(a.status, 1);
    }
    return;
  }
  float s = 0.f;
  for (long c = threadIdx.x; c < cells; c += blockDim.x) {
    const float v = ring_value(a, k, c, krp, rR, pad, nb);
    out[c] = v;
    s += v;
  }
  s = warp_sum(s);
  __shared__ float ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    a.sums[k] = t;
  }
}

__global__ void ring_normalise_kernel(long cells, int n, float* __restrict__ out, const float* __restrict__ sums) {
  const long total = cells * n;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const float s = sums[i / cells];
    if (s != 0.f) out[i] = out[i] / s;
  }
}

// In-place complex FFT along z of every (kernel, ky, kx) line of a
// [n][N][N][N/2+1] array (groups of 4 lanes per line).
template <int N>
__global__ void __launch_bounds__(128) zline_fft_kernel(long lines, float2* __restrict__ data) {
  using GE = Geo<N, 4>;
  constexpr int P = GE::P, Q = GE::Q, G = 4, HW = N / 2 + 1;
  constexpr long PLANE = (long)N * HW;
  __shared__ float2 tw[N];
  __shared__ float2 scr[32 * GE::SCR];
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = reinterpret_cast<const float2*>(kTwiddles<N, G>.v)[i];
  __syncthreads();
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const long l = (long)blockIdx.x * 32 + grp;
  if (l >= lines) return;  // whole groups of 4 lanes leave together
  const long kern = l / PLANE, within = l % PLANE;
  float2* base = data + kern * N * PLANE + within;
  float2 v[P];
#pragma unroll
  for (int n2 = 0; n2 < P; ++n2) v[n2] = base[(long)(t + G * n2) * PLANE];
  float2 u[Q][G];
  fft_standard<GE, false, false>(v, u, scr + grp * GE::SCR, tw, t, gmask);
#pragma unroll
  for (int q = 0; q < Q; ++q)
#pragma unroll
    for (int k1 = 0; k1 < G; ++k1) base[(long)(t + G * q + P * k1) * PLANE] = u[q][k1];
}

int validate(const lgx_ring_batch* j) {
  if (!j) return kfail(LGX_ERR_INVALID, "lgx_ring_kernels: null job");
  if (j->nb_dims != 2 && j->nb_dims != 3) return kfail(LGX_ERR_INVALID, "lgx_ring_kernels: nb_dims must be 2 or 3");
  if (!nd_side_ok(j->size))
    return kfail(LGX_ERR_UNSUPPORTED, "lgx_ring_kernels: %dD worlds of side %d (the N-D engine's sides)", j->nb_dims,
                 j->size);
  if (j->n < 1) return kfail(LGX_ERR_INVALID, "lgx_ring_kernels: n must be >= 1");
  if (j->kf_id < LGX_KF_POLY_QUAD || j->kf_id > LGX_KF_TRIANGLE)
    return kfail(LGX_ERR_UNSUPPORTED, "lgx_ring_kernels: unknown kernel function id %d", j->kf_id);
  if (j->nb_max < 1) return kfail(LGX_ERR_INVALID, "lgx_ring_kernels: nb_max must be >= 1");
  if (!j->R || !j->r || !j->b || !j->nb || !j->kf_params || !j->kernel_out || !j->status)
    return kfail(LGX_ERR_INVALID, "lgx_ring_kernels: null tensor");
  return LGX_OK;
}

long cells_of(const lgx_ring_batch* j) {
  long c = 1;
  for (int i = 0; i < j->nb_dims; ++i) c *= j->size;
  return c;
}

// the register-resident spectrum of the resident / streamed sizes, else the
// N-D engine's line passes
bool fast_spectrum(const lgx_ring_batch* j) {
  return (j->nb_dims == 2 && (j->size == 32 || j->size == 64 || j->size == 128 || j->size == 256)) ||
         (j->nb_dims == 3 && (j->size == 32 || j->size == 64));
}

size_t spectrum_ws_bytes(const lgx_ring_batch* j) {
  if (fast_spectrum(j)) return al256((size_t)j->n * cells_of(j) * sizeof(float));
  const int world[3] = {j->size, j->size, j->size};
  return nd_spectrum_workspace_bytes(j->nb_dims, world, j->n);
}

}  // namespace

extern "C" {

int lgx_ring_kernels_workspace_bytes(const lgx_ring_batch* j, size_t* bytes) {
  if (!bytes) return kfail(LGX_ERR_INVALID, "lgx_ring_kernels_workspace_bytes: null output");
  *bytes = 0;
  const int v = validate(j);
  if (v != LGX_OK) return v;
  *bytes = al256((size_t)j->n * sizeof(float)) + spectrum_ws_bytes(j);
  return LGX_OK;
}

int lgx_ring_kernels(const lgx_ring_batch* j, void* ws, size_t ws_bytes, void* stream) {
  const int v = validate(j);
  if (v != LGX_OK) return v;
  size_t need = 0;
  lgx_ring_kernels_workspace_bytes(j, &need);
  if (!ws || ws_bytes < need) return kfail(LGX_ERR_WORKSPACE, "lgx_ring_kernels: workspace %zu < %zu", ws_bytes, need);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long cells = cells_of(j);
  float* sums = static_cast<float*>(ws);
  float2* spec_ws = reinterpret_cast<float2*>(static_cast<char*>(ws) + al256((size_t)j->n * sizeof(float)));
  RingArgs a;
  a.nd = j->nb_dims;
  a.N = j->size;
  a.n = j->n;
  a.kf_id = j->kf_id;
  a.nb_max = j->nb_max;
  a.R = j->R;
  a.r = j->r;
  a.b = j->b;
  a.kfp = j->kf_params;
  a.nb = j->nb;
  a.out = j->kernel_out;
  a.sums = sums;
  a.status = j->status;
  cudaError_t e = cudaMemsetAsync(j->status, 0, sizeof(int), st);
  if (e != cudaSuccess) return kfail(LGX_ERR_CUDA, "lgx_ring_kernels: %s", cudaGetErrorString(e));
  ring_build_kernel<<<j->n, 256, 0, st>>>(a);
  const long total = cells * j->n;
  ring_normalise_kernel<<<(unsigned)std::min<long>((total + 255) / 256, 8192), 256, 0, st>>>(cells, j->n,
                                                                                           j->kernel_out, sums);
  if ((e = cudaGetLastError()) != cudaSuccess) return kfail(LGX_ERR_CUDA, "lgx_ring_kernels: %s", cudaGetErrorString(e));
  if (j->k_half && !fast_spectrum(j)) {
    const int world[3] = {j->size, j->size, j->size};
    e = launch_nd_spectrum(j->nb_dims, world, j->n, j->kernel_out, reinterpret_cast<float2*>(j->k_half), spec_ws, st);
    if (e != cudaSuccess) return kfail(LGX_ERR_CUDA, "lgx_ring_kernels spectrum: %s", cudaGetErrorString(e));
  } else if (j->k_half) {
    const int N = j->size;
    float2* kh = reinterpret_cast<float2*>(j->k_half);
    const int planes = j->nb_dims == 2 ? j->n : j->n * N;  // 3D: every z plane first
    e = launch_spectrum(N, planes, j->kernel_out, spec_ws, kh, st);
    if (e == cudaSuccess && j->nb_dims == 3) {
      const long lines = (long)j->n * N * (N / 2 + 1);
      const unsigned blocks = (unsigned)((lines + 31) / 32);
      if (N == 32) zline_fft_kernel<32><<<blocks, 128, 0, st>>>(lines, kh);
      else zline_fft_kernel<64><<<blocks, 128, 0, st>>>(lines, kh);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return kfail(LGX_ERR_CUDA, "lgx_ring_kernels spectrum: %s", cudaGetErrorString(e));
  }
  return LGX_OK;
}

}  // extern "C"
