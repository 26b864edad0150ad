// General N-D engine: any 2D or 3D torus whose sides factor into 2, 3, 5
// and 7 (odd, non-square and non-power-of-two sides included, e.g. 48^3),
// any number of channels and kernels -- the forward Euler step and its
// adjoint.  leniax's get_potential_fft transforms every world axis
// (core.py:74-87); here each axis is one pass of mixed-radix line FFTs over
// complex planes in HBM:
//
//   forward step : x pass (real state in), y pass, z pass   -> state spectra S
//                  S[c_in(k)] x prepared spectrum[k]           -> products P
//                  z, y, x inverse passes (real part out)      -> potentials u_k
//                  growth, weighted field, state update and the statistics
//                  moments per block (core.py:163-319, statistics.py:36-126)
//                  per-world reduction of the moments, carried torus shift
//   adjoint step : clip / state-function gradient, dL/df, dL/dg, growth
//                  derivative -> a_k = dL/du_k; forward passes of a_k and of
//                  the state; kernel gradient A_k conj(S) accumulated; the
//                  correlation sum_k A_k conj(K_k) per input channel through
//                  the inverse passes added to lambda; growth-parameter and
//                  weight gradients reduced per (world, kernel)
//
// A pass stages a tile of lines in shared memory (consecutive lines of the
// same group so that global loads and stores are coalesced), runs the
// Stockham transform of fft_mixed.cuh and writes the tile back in place.
// Spectra are full complex (no Hermitian packing), so odd sides need no
// special case.  This engine serves the worlds the specialised engines do not
// (resident: 2D 32..128 C = K = 1; streamed: square 2D; one world per CTA:
// 3D 32^3 / 64^3 C = K = 1) and every differentiated model beyond C = K = 1.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "engine.h"
#include "fft_mixed.cuh"

namespace lgx {
namespace {

constexpr int kNT = 256;          // threads per block
constexpr int kMaxPts = 4096;     // complex points of one pass tile (two buffers in shared memory)
constexpr int kRawMax = RAW_CM + kMaxChannels;

struct NdTab {  // kernel table of a model, passed by value
  int C, K, max_k, mean, state_fn, dt_mode, nd;
  int D, H, W;
  long cells;
  int cin[kMaxKernels];
  int slot[kMaxKernels];
  int gf[kMaxKernels];
};

NdTab make_tab(const Model& m, int dt_mode) {
  NdTab t;
  t.C = m.C;
  t.K = m.K;
  t.max_k = m.max_k;
  t.mean = m.mean;
  t.state_fn = m.state_fn;
  t.dt_mode = dt_mode;
  t.nd = m.nb_dims;
  t.D = m.D;
  t.H = m.H;
  t.W = m.W;
  t.cells = m.cells;
  for (int k = 0; k < kMaxKernels; ++k) {
    t.cin[k] = k < m.K ? m.cin[k] : 0;
    t.slot[k] = k < m.K ? m.slot[k] : 0;
    t.gf[k] = k < m.K ? m.gf[k] : 0;
  }
  return t;
}

// ------------------------------------------------------------------ passes
// Lines of a pass: line (g, i) starts at g * gstride + i and has L points
// `stride` apart; g < G, i < I.  I == 1: a tile is nl consecutive groups
// (rows of the x pass, contiguous); I > 1: nl consecutive i of one group.
struct Pass {
  float2* data;          // complex planes (in and out, in place)
  const float* src_real;  // IN_REAL: real input of the same geometry
  float* dst_real;        // OUT_REAL: Re(result) * scale (stored, or added when accumulate)
  long G, I, gstride, stride;
  int L, nl;
  int in_real, out_real, accumulate;
  float scale;
};

template <bool INV>
__global__ void __launch_bounds__(kNT) nd_pass_kernel(Pass a, GPlan p) {
  extern __shared__ __align__(16) float2 ndsm[];
  const int L = a.L, nl = a.nl;
  float2* tw = ndsm;
  float2* A = tw + L;
  float2* B = A + (size_t)nl * L;
  long g0, i0;
  int lines;
  if (a.I == 1) {
    g0 = (long)blockIdx.x * nl;
    i0 = 0;
    lines = (int)min((long)nl, a.G - g0);
  } else {
    const long tiles = (a.I + nl - 1) / nl;
    g0 = blockIdx.x / tiles;
    i0 = (blockIdx.x % tiles) * nl;
    lines = (int)min((long)nl, a.I - i0);
  }
  fill_twiddles(tw, L);
  const int pts = nl * L;
  // kLoadBatch independent global loads in flight per thread before their
  // shared-memory stores (one load per iteration would serialise on latency)
  constexpr int kLoadBatch = 8;
  for (int base = threadIdx.x; base < pts; base += kLoadBatch * blockDim.x) {
    float2 v[kLoadBatch];
    int dst[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = base + u * blockDim.x;
      int l, j;
      if (a.I == 1) {
        l = idx / L;
        j = idx - l * L;
      } else {
        j = idx / nl;
        l = idx - j * nl;
      }
      dst[u] = idx < pts ? l * L + j : -1;
      v[u] = make_float2(0.f, 0.f);
      if (idx < pts && l < lines) {
        const long off = (a.I == 1 ? (g0 + l) * a.gstride : g0 * a.gstride + i0 + l) + (long)j * a.stride;
        v[u] = a.in_real ? make_float2(__ldg(a.src_real + off), 0.f) : a.data[off];
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u)
      if (dst[u] >= 0) A[dst[u]] = v[u];
  }
  __syncthreads();
  const float2* res = fft_line<INV>(A, B, p, tw, nl);
  for (int idx = threadIdx.x; idx < pts; idx += blockDim.x) {
    int l, j;
    if (a.I == 1) {
      l = idx / L;
      j = idx - l * L;
    } else {
      j = idx / nl;
      l = idx - j * nl;
    }
    if (l >= lines) continue;
    const long off = (a.I == 1 ? (g0 + l) * a.gstride : g0 * a.gstride + i0 + l) + (long)j * a.stride;
    const float2 v = res[l * L + j];
    if (a.out_real) {
      const float r = v.x * a.scale;
      a.dst_real[off] = a.accumulate ? a.dst_real[off] + r : r;
    } else {
      a.data[off] = v;
    }
  }
}

// Opt the pass kernels into their shared-memory tile (set on the current
// device; cheap, so it is set before every pass).
cudaError_t allow_pass_smem() {
  const int bytes = (int)((2 * kMaxPts + kGMaxN) * sizeof(float2));
  cudaError_t e = cudaFuncSetAttribute(nd_pass_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(nd_pass_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

// One axis pass over `planes` planes of D x H x W points.  axis 0 = x
// (contiguous), 1 = y, 2 = z.
cudaError_t run_pass(bool inv, int axis, const NdTab& t, long planes, float2* data, const float* src_real,
                     float* dst_real, bool accumulate, float scale, cudaStream_t st) {
  Pass a;
  a.data = data;
  a.src_real = src_real;
  a.dst_real = dst_real;
  a.in_real = src_real != nullptr;
  a.out_real = dst_real != nullptr;
  a.accumulate = accumulate ? 1 : 0;
  a.scale = scale;
  const long HW = (long)t.H * t.W;
  if (axis == 0) {
    a.L = t.W;
    a.G = planes * t.D * t.H;
    a.I = 1;
    a.gstride = t.W;
    a.stride = 1;
  } else if (axis == 1) {
    a.L = t.H;
    a.G = planes * t.D;
    a.I = t.W;
    a.gstride = HW;
    a.stride = t.W;
  } else {
    a.L = t.D;
    a.G = planes;
    a.I = HW;
    a.gstride = HW * t.D;
    a.stride = HW;
  }
  const GPlan p = make_plan(a.L);
  if (p.stages == 0) return cudaErrorInvalidValue;
  const int cap = std::max(1, kMaxPts / a.L);
  a.nl = (int)std::min<long>(cap, a.I == 1 ? a.G : a.I);
  const long tiles = a.I == 1 ? (a.G + a.nl - 1) / a.nl : a.G * ((a.I + a.nl - 1) / a.nl);
  const size_t smem = (size_t)(a.L + 2 * a.nl * a.L) * sizeof(float2);
  cudaError_t e = allow_pass_smem();
  if (e != cudaSuccess) return e;
  if (tiles >= (1L << 31)) return cudaErrorInvalidConfiguration;
  if (inv) nd_pass_kernel<true><<<(unsigned)tiles, kNT, smem, st>>>(a, p);
  else nd_pass_kernel<false><<<(unsigned)tiles, kNT, smem, st>>>(a, p);
  return cudaGetLastError();
}

// Full forward transform of real planes (src) into complex planes (dst).
cudaError_t forward_real(const NdTab& t, long planes, const float* src, float2* dst, cudaStream_t st) {
  cudaError_t e = run_pass(false, 0, t, planes, dst, src, nullptr, false, 1.f, st);
  if (e == cudaSuccess) e = run_pass(false, 1, t, planes, dst, nullptr, nullptr, false, 1.f, st);
  if (e == cudaSuccess && t.D > 1) e = run_pass(false, 2, t, planes, dst, nullptr, nullptr, false, 1.f, st);
  return e;
}

// Unnormalised inverse transform of complex planes; the real part times
// `scale` is stored into (or added to) dst.
cudaError_t inverse_real(const NdTab& t, long planes, float2* data, float* dst, bool accumulate, float scale,
                         cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (t.D > 1) e = run_pass(true, 2, t, planes, data, nullptr, nullptr, false, 1.f, st);
  if (e == cudaSuccess) e = run_pass(true, 1, t, planes, data, nullptr, nullptr, false, 1.f, st);
  if (e == cudaSuccess) e = run_pass(true, 0, t, planes, data, nullptr, dst, accumulate, scale, st);
  return e;
}

// ------------------------------------------------------------------ spectra
// Prepared spectra: the Hermitian half [planes, D, H, W/2+1] extended to the
// full spectrum [planes, D, H, W] and scaled by 1/cells (the inverse passes
// are unnormalised).
__global__ void nd_prepare_kernel(long planes, int D, int H, int W, float scale, const float2* __restrict__ kh,
                                  float2* __restrict__ kf) {
  const int HWH = W / 2 + 1;
  const long cells = (long)D * H * W, total = planes * cells;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long pl = i / cells;
    long r = i - pl * cells;
    const int x = (int)(r % W);
    r /= W;
    const int y = (int)(r % H), z = (int)(r / H);
    float2 v;
    if (x < HWH) {
      v = kh[((pl * D + z) * H + y) * HWH + x];
    } else {  // K[z, y, x] = conj(K[-z, -y, W - x])
      const int zz = z == 0 ? 0 : D - z, yy = y == 0 ? 0 : H - y;
      const float2 c = kh[((pl * D + zz) * H + yy) * HWH + (W - x)];
      v = make_float2(c.x, -c.y);
    }
    kf[i] = make_float2(v.x * scale, v.y * scale);
  }
}

// Hermitian half of full spectra: [planes, D, H, W] -> [planes, D, H, W/2+1].
__global__ void nd_half_kernel(long planes, int D, int H, int W, const float2* __restrict__ full,
                               float2* __restrict__ half) {
  const int HWH = W / 2 + 1;
  const long rows = planes * D * H, total = rows * HWH;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long row = i / HWH;
    const int x = (int)(i - row * HWH);
    half[i] = full[row * W + x];
  }
}

inline int grid_for(long total) { return (int)std::max(1L, std::min<long>((total + kNT - 1) / kNT, 1L << 16)); }

// P[w, k] = S[w, c_in(k)] * prepared[sol(w), c_in(k), slot(k)]
__global__ void nd_multiply_kernel(NdTab t, int n_worlds, int n_init, const float2* __restrict__ S,
                                   const float2* __restrict__ kf, long kf_sol_stride, float2* __restrict__ P) {
  const long total = (long)n_worlds * t.K * t.cells;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long cell = i % t.cells;
    const long wk = i / t.cells;
    const int k = (int)(wk % t.K), w = (int)(wk / t.K);
    const int sol = w / n_init, c = t.cin[k];
    const float2 s = S[((long)w * t.C + c) * t.cells + cell];
    const float2 kk = __ldg(kf + sol * kf_sol_stride + ((long)c * t.max_k + t.slot[k]) * t.cells + cell);
    P[i] = cmul(s, kk);
  }
}

// ------------------------------------------------------------------ forward epilogue
struct EpiArgs {
  int n_worlds, n_init, bpw;
  const float* state;   // [nw, C, cells]
  float* state_out;     // [nw, C, cells]
  const float* pot;     // [nw, K, cells]
  const float* gf;      // [Ns, K, 2] (sol stride gf_sol_stride)
  long gf_sol_stride;
  const float* w;       // [Ns, C, K]
  long w_sol_stride;
  const float* dt;
  float* field_out;     // [nw, C, cells] or null
  const int* shift;     // [nw, 3]
  float* partial;       // [nw, bpw, RAWS]
};

// per-cell centred coordinate on one axis (statistics.py:64-81 on the world
// rolled by the carried shift): ((i - shift) mod n) - n // 2
__device__ __forceinline__ float centred(int i, int sh, int n) { return (float)(pmod(i - sh, n) - n / 2); }

__global__ void __launch_bounds__(kNT) nd_epilogue_kernel(NdTab t, EpiArgs a) {
  constexpr int NWARP = kNT / 32;
  __shared__ float red[NWARP][kRawMax];
  const int w = blockIdx.x / a.bpw, b = blockIdx.x % a.bpw;
  const int sol = w / a.n_init, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int C = t.C, K = t.K;
  const float* gf = a.gf + sol * a.gf_sol_stride;
  const float* wt = a.w + sol * a.w_sol_stride;
  float dt;
  if (t.dt_mode == 0) dt = __ldg(a.dt);
  else if (t.dt_mode == 1) dt = __ldg(a.dt + w);
  else dt = 1.f / __ldg(a.dt + sol);
  const int nd = t.nd;
  // axis order of the moments: 2D (y, x), 3D (z, y, x)
  const int s0 = a.shift[3 * w], s1 = a.shift[3 * w + 1], s2 = a.shift[3 * w + 2];
  const long chunk = (t.cells + a.bpw - 1) / a.bpw;
  const long c0 = (long)b * chunk, c1 = min(t.cells, c0 + chunk);
  float m00 = 0.f, g00 = 0.f, cpot = 0.f, cmass = 0.f, cgrow = 0.f;
  float mx0 = 0.f, mx1 = 0.f, mx2 = 0.f, gx0 = 0.f, gx1 = 0.f, gx2 = 0.f, q0 = 0.f, q1 = 0.f, q2 = 0.f;
  float cm[kMaxChannels];
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) cm[c] = 0.f;
  bool border = false;
  for (long cell = c0 + threadIdx.x; cell < c1; cell += blockDim.x) {
    const int x = (int)(cell % t.W);
    const long r = cell / t.W;
    const int y = (int)(r % t.H), z = (int)(r / t.H);
    float ca, cb, cc;  // centred coordinates along the moment axes
    if (nd == 2) {
      ca = centred(y, s0, t.H);
      cb = centred(x, s1, t.W);
      cc = 0.f;
    } else {
      ca = centred(z, s0, t.D);
      cb = centred(y, s1, t.H);
      cc = centred(x, s2, t.W);
    }
    const bool edge = x == 0 || x == t.W - 1 || y == 0 || y == t.H - 1 || (nd == 3 && (z == 0 || z == t.D - 1));
    for (int k = 0; k < K; ++k) cpot += __ldg(a.pot + ((long)w * K + k) * t.cells + cell) > kEps ? 1.f : 0.f;
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      float f = 0.f, wsum = 0.f;
      for (int k = 0; k < K; ++k) {
        const float wk = __ldg(wt + c * K + k);
        wsum += wk;
        if (wk == 0.f) continue;
        const float u = __ldg(a.pot + ((long)w * K + k) * t.cells + cell);
        f = fmaf(wk, growth_fn(t.gf[k], u, __ldg(gf + 2 * k), __ldg(gf + 2 * k + 1)), f);
      }
      if (t.mean) f = f / wsum;
      const long off = ((long)w * C + c) * t.cells + cell;
      const float sv = __ldg(a.state + off);
      a.state_out[off] = state_fn(t.state_fn, sv, f, dt);
      if (a.field_out) a.field_out[off] = f;
      const float fp = fmaxf(f, 0.f);
      m00 += sv;
      g00 += fp;
      cm[c] += sv;
      mx0 = fmaf(ca, sv, mx0);
      mx1 = fmaf(cb, sv, mx1);
      mx2 = fmaf(cc, sv, mx2);
      gx0 = fmaf(ca, fp, gx0);
      gx1 = fmaf(cb, fp, gx1);
      gx2 = fmaf(cc, fp, gx2);
      q0 = fmaf(ca * ca, sv, q0);
      q1 = fmaf(cb * cb, sv, q1);
      q2 = fmaf(cc * cc, sv, q2);
      const bool live = sv > kEps;
      cmass += live ? 1.f : 0.f;
      cgrow += fp > kEps ? 1.f : 0.f;
      border |= live && edge;
    }
  }
  float v[14] = {m00, g00, cpot, cmass, cgrow, mx0, mx1, mx2, gx0, gx1, gx2, q0, q1, q2};
#pragma unroll
  for (int i = 0; i < 14; ++i) v[i] = warp_sum(v[i]);
  const bool anyb = __any_sync(0xffffffffu, border);
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) {
    if (c >= C) break;
    cm[c] = warp_sum(cm[c]);
  }
  if (lane == 0) {
    float* rd = red[wid];
    rd[RAW_M00] = v[0];
    rd[RAW_G00] = v[1];
    rd[RAW_CNT_POT] = v[2];
    rd[RAW_CNT_MASS] = v[3];
    rd[RAW_CNT_GROW] = v[4];
    for (int i = 0; i < 3; ++i) {
      rd[RAW_MX + i] = v[5 + i];
      rd[RAW_GX + i] = v[8 + i];
      rd[RAW_MX2 + i] = v[11 + i];
    }
    rd[RAW_BORDER] = anyb ? 1.f : 0.f;
    for (int i = 0; i < 3; ++i) rd[RAW_SHIFT + i] = 0.f;
    for (int c = 0; c < C; ++c) rd[RAW_CM + c] = cm[c];
  }
  __syncthreads();
  const int RAWS = raw_stride(C);
  if (threadIdx.x < RAWS) {
    float s = 0.f;
    for (int i = 0; i < NWARP; ++i) s += red[i][threadIdx.x];
    if (threadIdx.x == RAW_BORDER) s = s > 0.f ? 1.f : 0.f;
    a.partial[((long)w * a.bpw + b) * RAWS + threadIdx.x] = s;
  }
}

// Per world: block moments -> the step's raw record (with the shift that
// centred it), then the carried shift advances by the integer part of the
// centred-frame centroid (statistics.py:117-124).
__global__ void nd_reduce_kernel(NdTab t, int n_worlds, int n_init, int bpw, const float* __restrict__ partial,
                                 float* __restrict__ raw, long raw_sol_stride, long raw_init_stride,
                                 int* __restrict__ shift) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= n_worlds) return;
  const int RAWS = raw_stride(t.C);
  const int sol = w / n_init, init = w - sol * n_init;
  float* rw = raw ? raw + sol * raw_sol_stride + init * raw_init_stride : nullptr;
  const int sh[3] = {shift[3 * w], shift[3 * w + 1], shift[3 * w + 2]};
  float m00 = 0.f, mx[3] = {0.f, 0.f, 0.f};
  for (int s = lane; s < RAWS; s += 32) {
    float v = 0.f;
    for (int b = 0; b < bpw; ++b) v += partial[((long)w * bpw + b) * RAWS + s];
    if (s == RAW_BORDER) v = v > 0.f ? 1.f : 0.f;
    if (s >= RAW_SHIFT && s < RAW_SHIFT + 3) v = (float)sh[s - RAW_SHIFT];
    if (rw) rw[s] = v;
  }
  __syncwarp();
  if (lane == 0) {
    for (int b = 0; b < bpw; ++b) {
      const float* pp = partial + ((long)w * bpw + b) * RAWS;
      m00 += pp[RAW_M00];
      for (int i = 0; i < 3; ++i) mx[i] += pp[RAW_MX + i];
    }
    const int n[3] = {t.nd == 2 ? t.H : t.D, t.nd == 2 ? t.W : t.H, t.W};
    for (int i = 0; i < t.nd; ++i) shift[3 * w + i] = pmod(sh[i] + (int)(mx[i] / (m00 + kEps)), n[i]);
  }
}

// ------------------------------------------------------------------ adjoint
struct AdjArgs {
  int n_worlds, n_init, clip_mask;
  const float* s;      // [nw, C, cells] state entering the step
  const float* s_next;  // [nw, C, cells] state after the step, or null
  const float* u;      // [nw, K, cells] potentials of the step
  const float* lam;    // [nw, C, cells] dL/d(state after the step)
  float* lam_out;      // [nw, C, cells] direct part of dL/d(state before the step)
  float* a;            // [nw, K, cells] dL/du_k
  float* bf;           // [nw, C, cells] dL/df_c
  float* ff;           // [nw, C, cells] f_c
  const float* gf;     // [Ns, K, 2]
  const float* w;      // [Ns, C, K]
  const float* T;      // [Ns]
};

// growth(u) and its derivative in u (growth_functions.py); every family but
// identity is a function of (u - m) / s, so d/dm = -d/du and
// d/ds = -d/du (u - m) / s.
__device__ __forceinline__ float growth_du(int id, float u, float m, float s, float* g) {
  if (id == LGX_GF_GAUSSIAN || id == LGX_GF_GAUSSIAN_TARGET) {
    const float d = (u - m) / s;
    const float e = expf(-(d * d) / 2.f);
    const float amp = id == LGX_GF_GAUSSIAN ? 2.f : 1.f;
    *g = id == LGX_GF_GAUSSIAN ? 2.f * e - 1.f : e;
    return -amp * e * d / s;
  }
  if (id == LGX_GF_POLY_QUAD4) {
    const float d = u - m, c = 9.f * s * s;
    const float q = 1.f - d * d / c;
    if (q > 0.f) {
      const float q3 = q * q * q;
      *g = 2.f * q3 * q - 1.f;
      return 8.f * q3 * (-2.f * d / c);
    }
    *g = -1.f;
    return 0.f;
  }
  *g = growth_fn(id, u, m, s);
  if (id == LGX_GF_IDENTITY) return 1.f;
  if (id == LGX_GF_TRIANGLE) {  // growth_functions.py:234-243: slopes 2/s and -2/s
    if (u >= m - s && u < m) return 2.f / s;
    if (u >= m && u <= m + s) return -2.f / s;
  }
  return 0.f;  // step, staircase: piecewise constant
}

__global__ void __launch_bounds__(kNT) nd_adj_point_kernel(NdTab t, AdjArgs a) {
  const long total = (long)a.n_worlds * t.cells;
  const int C = t.C, K = t.K;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int w = (int)(i / t.cells);
    const long cell = i - (long)w * t.cells;
    const int sol = w / a.n_init;
    const float dt = 1.f / __ldg(a.T + sol);
    const float* gf = a.gf + (long)sol * 2 * K;
    const float* wt = a.w + (long)sol * C * K;
    float f[kMaxChannels], bb[kMaxChannels], ws[kMaxChannels];
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      f[c] = 0.f;
      ws[c] = 0.f;
      bb[c] = 0.f;
    }
    for (int k = 0; k < K; ++k) {
      const float u = __ldg(a.u + ((long)w * K + k) * t.cells + cell);
      const float g = growth_fn(t.gf[k], u, __ldg(gf + 2 * k), __ldg(gf + 2 * k + 1));
#pragma unroll
      for (int c = 0; c < kMaxChannels; ++c) {
        if (c >= C) break;
        const float wk = __ldg(wt + c * K + k);
        ws[c] += wk;
        if (wk != 0.f) f[c] = fmaf(wk, g, f[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      if (t.mean) f[c] = f[c] / ws[c];
      const long off = ((long)w * C + c) * t.cells + cell;
      const float lam = __ldg(a.lam + off);
      const float sv = __ldg(a.s + off);
      float dsds, dsdf;  // d state' / d state and d state' / d field (core.py:245-319)
      if (t.state_fn == LGX_STATE_V1) {
        // mask: the forward's clip was inactive where its output lies strictly inside (0, 1)
        const float n = a.s_next ? __ldg(a.s_next + off) : fmaf(dt, f[c], sv);
        const float cg = a.clip_mask ? ((n > 0.f && n < 1.f) ? 1.f : 0.f) : 1.f;  // mask or straight-through
        dsds = cg;
        dsdf = dt * cg;
      } else if (t.state_fn == LGX_STATE_V2) {
        dsds = 1.f - dt;
        dsdf = dt;
      } else {
        dsds = 1.f;
        dsdf = dt;
      }
      a.lam_out[off] = lam * dsds;
      bb[c] = lam * dsdf;
      a.bf[off] = bb[c];
      a.ff[off] = f[c];
    }
    for (int k = 0; k < K; ++k) {
      const float u = __ldg(a.u + ((long)w * K + k) * t.cells + cell);
      float g;
      const float gu = growth_du(t.gf[k], u, __ldg(gf + 2 * k), __ldg(gf + 2 * k + 1), &g);
      float dg = 0.f;  // dL/dg_k = sum_c dL/df_c * w_ck (/ sum_j w_cj in mean mode)
#pragma unroll
      for (int c = 0; c < kMaxChannels; ++c) {
        if (c >= C) break;
        const float wk = __ldg(wt + c * K + k);
        dg = fmaf(bb[c], t.mean ? wk / ws[c] : wk, dg);
      }
      a.a[((long)w * K + k) * t.cells + cell] = dg * gu;
    }
  }
}

// Per (world, kernel): dL/dm_k = -sum a_k, dL/ds_k = -sum a_k (u_k - m) / s,
// dL/dw_ck = sum dL/df_c * (g_k - f_c) / sum_j w_cj (mean) or dL/df_c * g_k
// (sum), accumulated into pacc[w] ([2K] growth parameters, then [C, K]).
__global__ void __launch_bounds__(kNT) nd_adj_param_kernel(NdTab t, int n_init, const float* __restrict__ u,
                                                           const float* __restrict__ a, const float* __restrict__ bf,
                                                           const float* __restrict__ ff, const float* __restrict__ gfp,
                                                           const float* __restrict__ wts, float* __restrict__ pacc) {
  const int C = t.C, K = t.K;
  const int w = blockIdx.x / K, k = blockIdx.x % K;
  const int sol = w / n_init;
  const float m = __ldg(gfp + ((long)sol * K + k) * 2), s = __ldg(gfp + ((long)sol * K + k) * 2 + 1);
  const int id = t.gf[k];
  float wsum[kMaxChannels];
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) {
    wsum[c] = 0.f;
    if (c < C)
      for (int j = 0; j < K; ++j) wsum[c] += __ldg(wts + ((long)sol * C + c) * K + j);
  }
  float dm = 0.f, ds = 0.f, dw[kMaxChannels];
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) dw[c] = 0.f;
  for (long cell = threadIdx.x; cell < t.cells; cell += blockDim.x) {
    const float uu = __ldg(u + ((long)w * K + k) * t.cells + cell);
    const float ak = __ldg(a + ((long)w * K + k) * t.cells + cell);
    if (id != LGX_GF_IDENTITY) {
      dm -= ak;
      ds -= ak * (uu - m) / s;
    }
    const float g = growth_fn(id, uu, m, s);
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      const long off = ((long)w * C + c) * t.cells + cell;
      const float b = __ldg(bf + off);
      dw[c] = fmaf(b, t.mean ? (g - __ldg(ff + off)) / wsum[c] : g, dw[c]);
    }
  }
  __shared__ float red[kNT / 32][2 + kMaxChannels];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  dm = warp_sum(dm);
  ds = warp_sum(ds);
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) dw[c] = warp_sum(dw[c]);
  if (lane == 0) {
    red[wid][0] = dm;
    red[wid][1] = ds;
    for (int c = 0; c < kMaxChannels; ++c) red[wid][2 + c] = dw[c];
  }
  __syncthreads();
  if (threadIdx.x < 2 + C) {
    float v = 0.f;
    for (int i = 0; i < kNT / 32; ++i) v += red[i][threadIdx.x];
    float* pw = pacc + (long)w * (2 * K + C * K);
    if (threadIdx.x < 2) pw[2 * k + threadIdx.x] += v;
    else pw[2 * K + (threadIdx.x - 2) * K + k] += v;
  }
}

// Spectral part of the reverse step: gk[w, k] += A_k conj(S_cin(k)) (kernel
// gradient), Q[w, c] = sum_{k: c_in(k) = c} A_k conj(prepared K_k).
__global__ void nd_adj_spectral_kernel(NdTab t, int n_worlds, int n_init, const float2* __restrict__ A,
                                       const float2* __restrict__ S, const float2* __restrict__ kf,
                                       long kf_sol_stride, float2* __restrict__ gk, float2* __restrict__ Q) {
  const long total = (long)n_worlds * t.cells;
  const int C = t.C, K = t.K;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int w = (int)(i / t.cells);
    const long cell = i - (long)w * t.cells;
    const int sol = w / n_init;
    float2 q[kMaxChannels];
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) q[c] = make_float2(0.f, 0.f);
    for (int k = 0; k < K; ++k) {
      const int c = t.cin[k];
      const float2 ak = A[((long)w * K + k) * t.cells + cell];
      const float2 sc = S[((long)w * C + c) * t.cells + cell];
      float2* g = gk + ((long)w * K + k) * t.cells + cell;
      *g = cadd(*g, cmulc(ak, sc));
      const float2 kk = __ldg(kf + sol * kf_sol_stride + ((long)c * t.max_k + t.slot[k]) * t.cells + cell);
      const float2 pr = cmulc(ak, kk);
#pragma unroll
      for (int cc = 0; cc < kMaxChannels; ++cc)
        if (cc == c) q[cc] = cadd(q[cc], pr);
    }
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      Q[((long)w * C + c) * t.cells + cell] = q[c];
    }
  }
}

// per solution: grad_gf[s] += sum over its inits of pacc[..., :2K],
// grad_w[s] += sum of pacc[..., 2K:]
__global__ void nd_param_reduce_kernel(int n_sols, int n_init, int K, int C, const float* __restrict__ pacc,
                                       float* __restrict__ grad_gf, float* __restrict__ grad_w) {
  const int per = 2 * K + C * K;
  const long total = (long)n_sols * per;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int sol = (int)(i / per), j = (int)(i % per);
    float v = 0.f;
    for (int n = 0; n < n_init; ++n) v += pacc[((long)sol * n_init + n) * per + j];
    if (j < 2 * K) grad_gf[(long)sol * 2 * K + j] += v;
    else grad_w[(long)sol * C * K + (j - 2 * K)] += v;
  }
}

// gsum[s, k] = sum over the inits of solution s of gk[w, k]
__global__ void nd_sum_inits_kernel(long per_sol, int n_sols, int n_init, const float2* __restrict__ gk,
                                    float2* __restrict__ gsum) {
  const long total = (long)n_sols * per_sol;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int sol = (int)(i / per_sol);
    const long j = i - (long)sol * per_sol;
    float2 v = make_float2(0.f, 0.f);
    for (int n = 0; n < n_init; ++n) v = cadd(v, gk[((long)sol * n_init + n) * per_sol + j]);
    gsum[i] = v;
  }
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// ---------------------------------------------------------------------- API
bool nd_side_ok(int n) { return n >= 2 && n <= kGMaxN && make_plan(n).stages > 0; }

bool nd_supported(const Model& m) {
  if (m.nb_dims != 2 && m.nb_dims != 3) return false;
  if (m.C > kMaxChannels || m.K > kMaxKernels) return false;
  for (int i = 0; i < m.nb_dims; ++i)
    if (!nd_side_ok(m.world[i])) return false;
  return true;
}

int nd_blocks_per_world(const Model& m) {
  return (int)std::max(1L, std::min<long>(256, (m.cells + (long)kNT * 16 - 1) / ((long)kNT * 16)));
}

size_t nd_step_workspace_bytes(const Model& m, int n_worlds) {
  const size_t nw = (size_t)n_worlds, cells = (size_t)m.cells;
  return al256(nw * m.C * cells * sizeof(float2)) + al256(nw * m.K * cells * sizeof(float2)) +
         al256(nw * m.K * cells * sizeof(float)) + al256(nw * nd_blocks_per_world(m) * raw_stride(m.C) * sizeof(float));
}

size_t nd_prepared_bytes(const Model& m, int n_sols) {
  return al256((size_t)n_sols * m.C * m.max_k * m.cells * sizeof(float2));
}

cudaError_t launch_nd_prepare(const Model& m, int n_sols, const float2* k_half, float2* kf, cudaStream_t st) {
  const long planes = (long)n_sols * m.C * m.max_k;
  nd_prepare_kernel<<<grid_for(planes * m.cells), kNT, 0, st>>>(planes, m.D, m.H, m.W, 1.f / (float)m.cells, k_half,
                                                                kf);
  return cudaGetLastError();
}

cudaError_t launch_nd_step(const NdStep& s, cudaStream_t st) {
  const Model& m = *s.m;
  const NdTab t = make_tab(m, s.dt_mode);
  const size_t nw = (size_t)s.n_worlds, cells = (size_t)m.cells;
  const int bpw = nd_blocks_per_world(m);
  char* p = static_cast<char*>(s.ws);
  float2* S = reinterpret_cast<float2*>(p);
  p += al256(nw * m.C * cells * sizeof(float2));
  float2* P = reinterpret_cast<float2*>(p);
  p += al256(nw * m.K * cells * sizeof(float2));
  float* U = reinterpret_cast<float*>(p);
  p += al256(nw * m.K * cells * sizeof(float));
  float* partial = reinterpret_cast<float*>(p);
  float* pot = s.pot_out ? s.pot_out : U;
  cudaError_t e = forward_real(t, (long)nw * m.C, s.state, S, st);
  if (e != cudaSuccess) return e;
  nd_multiply_kernel<<<grid_for((long)nw * m.K * cells), kNT, 0, st>>>(t, s.n_worlds, s.n_init, S, s.kf,
                                                                        s.kf_sol_stride, P);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = inverse_real(t, (long)nw * m.K, P, pot, false, 1.f, st)) != cudaSuccess) return e;
  EpiArgs a;
  a.n_worlds = s.n_worlds;
  a.n_init = s.n_init;
  a.bpw = bpw;
  a.state = s.state;
  a.state_out = s.state_out;
  a.pot = pot;
  a.gf = s.gf;
  a.gf_sol_stride = s.gf_sol_stride;
  a.w = s.w;
  a.w_sol_stride = s.w_sol_stride;
  a.dt = s.dt;
  a.field_out = s.field_out;
  a.shift = s.shift;
  a.partial = partial;
  nd_epilogue_kernel<<<(unsigned)(nw * bpw), kNT, 0, st>>>(t, a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int wpb = 4;
  nd_reduce_kernel<<<(unsigned)((nw + wpb - 1) / wpb), 32 * wpb, 0, st>>>(
      t, s.n_worlds, s.n_init, bpw, partial, s.raw, s.raw_sol_stride, s.raw_world_stride, s.shift);
  return cudaGetLastError();
}

size_t nd_adjoint_workspace_bytes(const Model& m, int n_sols, int n_init) {
  const size_t nw = (size_t)n_sols * n_init, cells = (size_t)m.cells;
  return nd_prepared_bytes(m, n_sols) + al256(nw * m.K * cells * sizeof(float2)) +  // kf, A
         2 * al256(nw * m.C * cells * sizeof(float2)) +                              // S, Q
         al256(nw * m.K * cells * sizeof(float)) +                                   // a
         3 * al256(nw * m.C * cells * sizeof(float)) +                               // bf, ff, lambda ping-pong
         al256(nw * (2 * m.K + m.C * m.K) * sizeof(float));                          // parameter partials
}

size_t nd_kernel_grad_acc_bytes(const Model& m, int n_sols, int n_init) {
  return (size_t)n_sols * n_init * m.K * m.cells * sizeof(float2);
}

cudaError_t launch_nd_adjoint(const Model& m, const NdAdjoint& j, void* ws, cudaStream_t st) {
  const NdTab t = make_tab(m, 2);
  const int nw = j.n_sols * j.n_init;
  const size_t cells = (size_t)m.cells;
  char* p = static_cast<char*>(ws);
  float2* kf = reinterpret_cast<float2*>(p);
  p += nd_prepared_bytes(m, j.n_sols);
  float2* A = reinterpret_cast<float2*>(p);
  p += al256((size_t)nw * m.K * cells * sizeof(float2));
  float2* S = reinterpret_cast<float2*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float2));
  float2* Q = reinterpret_cast<float2*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float2));
  float* ar = reinterpret_cast<float*>(p);
  p += al256((size_t)nw * m.K * cells * sizeof(float));
  float* bf = reinterpret_cast<float*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float));
  float* ff = reinterpret_cast<float*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float));
  float* lam_tmp = reinterpret_cast<float*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float));
  float* pacc = reinterpret_cast<float*>(p);
  const long kf_sol = (long)m.C * m.max_k * m.cells;
  cudaError_t e = launch_nd_prepare(m, j.n_sols, j.k_half, kf, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(pacc, 0, (size_t)nw * (2 * m.K + m.C * m.K) * sizeof(float), st);
  if (e != cudaSuccess) return e;
  const size_t plane_c = (size_t)m.C * cells, plane_k = (size_t)m.K * cells;
  const float* lam_in = j.lambda_in;
  for (int step = j.steps - 1; step >= 0; --step) {
    float* lam_out = (step % 2 == 0) ? j.lambda_out : lam_tmp;  // step 0 lands in lambda_out
    AdjArgs a;
    a.n_worlds = nw;
    a.n_init = j.n_init;
    a.clip_mask = j.clip_mask;
    a.s = j.traj_cells + (size_t)step * nw * plane_c;
    a.s_next = step + 1 < j.steps ? a.s + (size_t)nw * plane_c : j.cells_after;
    a.u = j.traj_potential + (size_t)step * nw * plane_k;
    a.lam = lam_in;
    a.lam_out = lam_out;
    a.a = ar;
    a.bf = bf;
    a.ff = ff;
    a.gf = j.gf_params;
    a.w = j.weights;
    a.T = j.T;
    nd_adj_point_kernel<<<grid_for((long)nw * cells), kNT, 0, st>>>(t, a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    nd_adj_param_kernel<<<(unsigned)(nw * m.K), kNT, 0, st>>>(t, j.n_init, a.u, ar, bf, ff, j.gf_params, j.weights,
                                                                pacc);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = forward_real(t, (long)nw * m.K, ar, A, st)) != cudaSuccess) return e;
    if ((e = forward_real(t, (long)nw * m.C, a.s, S, st)) != cudaSuccess) return e;
    nd_adj_spectral_kernel<<<grid_for((long)nw * cells), kNT, 0, st>>>(t, nw, j.n_init, A, S, kf, kf_sol, j.gk, Q);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = inverse_real(t, (long)nw * m.C, Q, lam_out, true, 1.f, st)) != cudaSuccess) return e;
    lam_in = lam_out;
  }
  nd_param_reduce_kernel<<<grid_for((long)j.n_sols * (2 * m.K + m.C * m.K)), kNT, 0, st>>>(
      j.n_sols, j.n_init, m.K, m.C, pacc, j.grad_gf, j.grad_weights);
  return cudaGetLastError();
}

size_t nd_kernel_grad_workspace_bytes(const Model& m, int n_sols) {
  return al256((size_t)n_sols * m.K * m.cells * sizeof(float2));
}

cudaError_t launch_nd_kernel_grad(const Model& m, int n_sols, int n_init, const float2* gk, float* out, void* ws,
                                  cudaStream_t st) {
  const NdTab t = make_tab(m, 2);
  float2* gsum = static_cast<float2*>(ws);
  const long per = (long)m.K * m.cells;
  nd_sum_inits_kernel<<<grid_for((long)n_sols * per), kNT, 0, st>>>(per, n_sols, n_init, gk, gsum);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // dL/dk = Re(IFFT(sum_t A_t conj(S_t))) = unnormalised inverse / cells
  return inverse_real(t, (long)n_sols * m.K, gsum, out, false, 1.f / (float)m.cells, st);
}

size_t nd_spectrum_workspace_bytes(int nb_dims, const int* world, int planes) {
  long cells = 1;
  for (int i = 0; i < nb_dims; ++i) cells *= world[i];
  return al256((size_t)planes * cells * sizeof(float2));
}

cudaError_t launch_nd_spectrum(int nb_dims, const int* world, int planes, const float* k_real, float2* k_half,
                               void* ws, cudaStream_t st) {
  Model m;
  m.nb_dims = nb_dims;
  m.D = nb_dims == 3 ? world[0] : 1;
  m.H = world[nb_dims - 2];
  m.W = world[nb_dims - 1];
  m.cells = (long)m.D * m.H * m.W;
  m.C = m.K = m.max_k = 1;
  m.mean = 1;
  m.state_fn = 0;
  m.cin[0] = m.slot[0] = m.gf[0] = 0;
  const NdTab t = make_tab(m, 0);
  float2* full = static_cast<float2*>(ws);
  cudaError_t e = forward_real(t, planes, k_real, full, st);
  if (e != cudaSuccess) return e;
  const long total = (long)planes * m.D * m.H * (m.W / 2 + 1);
  nd_half_kernel<<<grid_for(total), kNT, 0, st>>>(planes, m.D, m.H, m.W, full, k_half);
  return cudaGetLastError();
}

}  // namespace lgx
