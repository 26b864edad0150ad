// Streamed Lenia step for any channel/kernel topology (2D, square power-of-two
// worlds): the spectra of a step travel through HBM/L2 between four kernels.
//
//   row_fwd  : per (world, channel, packed row) N-point FFT of rows (2r, 2r+1)
//              packed as one complex row -> spec[n][c][r][k]
//   col_conv : per (world, channel, column pair) unpack + N-point FFT, then for
//              every kernel reading that channel: x prepared spectrum, inverse
//              FFT -> prod[n][k] (packed rows layout)
//   row_inv  : per (world, packed-row block) inverse row FFTs of all kernels ->
//              potential, growth, weighted field (core.py:163-242), state
//              update (core.py:245-319), per-block raw statistics moments
//   reduce   : per world: block moments -> raw moments of the step, carried
//              torus shift update (statistics.py:117-119)
//
// This is leniax core.update with get_potential_fft (core.py:52-102), the
// true-kernel selection (tc_indices, core.py:97-98) being the (c_in, slot)
// table of the plan.
#include <algorithm>

#include "common.cuh"
#include "engine.h"
#include "fft.cuh"

namespace lgx {

namespace {

constexpr int kThreads = 256;     // row_fwd blocks
constexpr int kColThreads = 128;  // col_conv blocks (register-heavy: several blocks per SM)

struct KTab {  // per-plan kernel table, passed by value
  int C, K, max_k, mean, state_fn, dt_mode;
  int cin[kMaxKernels];
  int slot[kMaxKernels];
  int gf[kMaxKernels];
};

template <int N>
struct SCfg;
template <>
struct SCfg<32> { static constexpr int G = 4; };
template <>
struct SCfg<64> { static constexpr int G = 4; };
template <>
struct SCfg<128> { static constexpr int G = 8; };
template <>
struct SCfg<256> { static constexpr int G = 8; };

template <int N>
__device__ __forceinline__ float2* init_tw(float2* sm) {
  using GE = Geo<N, SCfg<N>::G>;
  init_twiddles<GE>(sm, sm + N, sm + 2 * N, threadIdx.x, blockDim.x);
  return sm + 3 * N;
}

// ------------------------------------------------------------------ row_fwd
template <int N>
__global__ void __launch_bounds__(kThreads) row_fwd_kernel(int n_worlds, int C, const float* __restrict__ state,
                                                           float2* __restrict__ spec) {
  constexpr int G = SCfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q, GPB = kThreads / G;  // groups per block
  constexpr int BPP = (N / 2 + GPB - 1) / GPB;             // blocks per plane
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = init_tw<N>(sm);
  __syncthreads();
  const int plane = blockIdx.x / BPP;  // n*C + c
  if (plane >= n_worlds * C) return;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int r = (blockIdx.x % BPP) * GPB + grp;
  if (r >= N / 2) return;  // whole groups exit together (never used with N/2 % GPB != 0 and partial warps)
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const float* src = state + (size_t)plane * N * N;
  float2 v[P];
#pragma unroll
  for (int n2 = 0; n2 < P; ++n2)
    v[n2] = make_float2(__ldg(src + (2 * r) * N + t + G * n2), __ldg(src + (2 * r + 1) * N + t + G * n2));
  float2 u[Q][G];
  fft_standard<GE, false, false>(v, u, scr + grp * GE::SCR, sm, t, gmask);
  float2* dst = spec + ((size_t)plane * (N / 2) + r) * N;
#pragma unroll
  for (int q = 0; q < Q; ++q)
#pragma unroll
    for (int k1 = 0; k1 < G; ++k1) dst[t + G * q + P * k1] = u[q][k1];
}

// ----------------------------------------------------------------- col_conv
template <int N>
__global__ void __launch_bounds__(kColThreads) col_conv_kernel(int n_worlds, int n_init, KTab tab,
                                                               const float2* __restrict__ spec,
                                                               const float2* __restrict__ kp, long kp_sol_stride,
                                                               float2* __restrict__ prod) {
  constexpr int G = SCfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q, GPB = kColThreads / G;
  constexpr int BPP = (N / 2 + GPB - 1) / GPB;
  constexpr int KPITCH = N / 2 + 2;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = init_tw<N>(sm);
  __syncthreads();
  const int plane = blockIdx.x / BPP;  // n*C + c
  if (plane >= n_worlds * tab.C) return;
  const int n = plane / tab.C, ch = plane % tab.C;
  const int sol = n / n_init;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int c = (blockIdx.x % BPP) * GPB + grp;
  if (c >= N / 2) return;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  float2* cs = scr + grp * GE::SCR;
  const float2* sp = spec + (size_t)plane * (N / 2) * N;

  float2 v[Q][G];
#pragma unroll
  for (int jp = 0; jp < Q / 2; ++jp) {
    const int m = t + G * jp;
#pragma unroll
    for (int n2 = 0; n2 < G; ++n2) {
      const int r = m + (P / 2) * n2;
      if (c != 0) {
        float2 z1 = sp[r * N + c], z2 = sp[r * N + N - c];
        v[2 * jp][n2] = make_float2(z1.x + z2.x, z1.y - z2.y);
        v[2 * jp + 1][n2] = make_float2(z1.y + z2.y, z2.x - z1.x);
      } else {
        float2 z1 = sp[r * N], z2 = sp[r * N + N / 2];
        v[2 * jp][n2] = make_float2(z1.x, z2.x);
        v[2 * jp + 1][n2] = make_float2(z1.y, z2.y);
      }
    }
  }
  float2 w0[P];
  fft_mirrored<GE, false, false>(v, w0, cs, sm + N, t, gmask);
  // the packed DC / Nyquist column (c == 0, one group per plane) keeps its
  // spectrum in the block's mirror buffer: Q[ky] needs A[-ky] for every kernel
  float2* mirror = scr + GPB * GE::SCR;
  if (c == 0) {
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) mirror[t + G * k1] = w0[k1];
    __syncwarp(gmask);
  }
  for (int k = 0; k < tab.K; ++k) {
    if (tab.cin[k] != ch) continue;
    const float2* kk = kp + sol * kp_sol_stride + ((size_t)(ch * tab.max_k + tab.slot[k]) * N) * KPITCH;
    float2 w[P];
    if (c != 0) {
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) w[k1] = cmul(w0[k1], __ldg(kk + (t + G * k1) * KPITCH + c));
    } else {
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) {
        const int ky = t + G * k1;
        const float2 A = __ldg(kk + ky * KPITCH), B = __ldg(kk + ky * KPITCH + N / 2);
        w[k1] = cadd(cmul(w0[k1], A), cmul(conjf2(mirror[(N - ky) & (N - 1)]), B));
      }
    }
    float2 u[Q][G];
    fft_standard<GE, true, true>(w, u, cs, sm, t, gmask);
    float2* pd = prod + ((size_t)n * tab.K + k) * (N / 2) * N;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int m = t + G * (q >> 1);
#pragma unroll
      for (int k1 = 0; k1 < G; ++k1) {
        const int r = m + (P / 2) * k1;
        const int col = (c != 0) ? ((q & 1) ? N - c : c) : ((q & 1) ? N / 2 : 0);
        pd[r * N + col] = u[q][k1];
      }
    }
  }
}

// ------------------------------------------------------------------ row_inv
// Block = GPB groups = GPB packed rows of one world.  Output channels are
// processed one after the other; the weighted field of the current channel is
// accumulated in registers (the row pair of a group: 2*P values per thread)
// over the kernels that feed it.  A kernel feeding several channels is
// inverse-transformed once per channel; its potential is counted (and
// written) once, at the first channel it feeds; kernels that feed no channel
// are transformed at the end for the potential count alone.
template <int N>
struct RowInvCfg {
  static constexpr int G = SCfg<N>::G;
  static constexpr int T = ((N / 2) * G < 128) ? (N / 2) * G : 128;  // threads per block
  static constexpr int GPB = T / G;
  static constexpr int BPW = (N / 2) / GPB;  // blocks per world
};

template <int N, int GF>
__global__ void __launch_bounds__(RowInvCfg<N>::T) row_inv_kernel(
    int n_worlds, int n_init, KTab tab, const float2* __restrict__ prod, const float* __restrict__ gfp,
    long gf_sol_stride, const float* __restrict__ wts, long w_sol_stride, const float* __restrict__ dtp,
    const float* __restrict__ state, float* __restrict__ state_out, float* __restrict__ field_out,
    float* __restrict__ pot_out, const int* __restrict__ shift, float* __restrict__ partial) {
  using RC = RowInvCfg<N>;
  constexpr int G = RC::G, GPB = RC::GPB, BPW = RC::BPW;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q;
  constexpr int RAWS_MAX = RAW_CM + kMaxChannels;
  constexpr int NWARPS = RC::T / 32;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = init_tw<N>(sm);                                   // GPB * SCR
  float* red = reinterpret_cast<float*>(scr + GPB * GE::SCR);  // [warps][RAWS_MAX]
  __syncthreads();
  const int n = blockIdx.x / BPW;
  if (n >= n_worlds) return;
  const int sol = n / n_init;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r = (blockIdx.x % BPW) * GPB + grp;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int C = tab.C, K = tab.K;
  float2* rs = scr + grp * GE::SCR;
  const float* gf = gfp + sol * gf_sol_stride;
  const float* wt = wts + sol * w_sol_stride;

  // inverse row transform of kernel k's product spectrum -> potentials of
  // rows (2r, 2r+1) at x = t + G*k1; counts them, writes them if requested
  auto potential = [&](int k, bool count, float2 (&w)[P], float& cpot) {
    const float2* pr = prod + (((size_t)n * K + k) * (N / 2) + r) * N;
    float2 v[Q][G];
    unpack_row_pair<GE>(pr, v, t);
    fft_mirrored<GE, true, true>(v, w, rs, sm + 2 * N, t, gmask);
    if (count) {
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) cpot += (w[k1].x > kEps ? 1.f : 0.f) + (w[k1].y > kEps ? 1.f : 0.f);
      if (pot_out) {
        float* po = pot_out + ((size_t)n * K + k) * N * N;
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          po[(2 * r) * N + t + G * k1] = w[k1].x;
          po[(2 * r + 1) * N + t + G * k1] = w[k1].y;
        }
      }
    }
  };

  float dt;
  if (tab.dt_mode == 0) dt = __ldg(dtp);
  else if (tab.dt_mode == 1) dt = __ldg(dtp + n);
  else dt = 1.f / __ldg(dtp + sol);
  const int sy = shift[3 * n], sx = shift[3 * n + 1];
  float cpot = 0.f, m00 = 0.f, g00 = 0.f, cmass = 0.f, cgrow = 0.f, mxy = 0.f, mxx = 0.f, gxy = 0.f, gxx = 0.f,
        m2y = 0.f, m2x = 0.f;
  bool border = false;
  const float cya = (float)(((2 * r - sy) & (N - 1)) - N / 2);
  const float cyb = (float)(((2 * r + 1 - sy) & (N - 1)) - N / 2);

  for (int co = 0; co < C; ++co) {
    float2 acc[P];
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) acc[k1] = make_float2(0.f, 0.f);
    float wsum = 0.f;
    for (int k = 0; k < K; ++k) {
      const float wk = __ldg(wt + co * K + k);
      wsum += wk;
      if (wk == 0.f) continue;  // uniform over the block
      bool first = true;
      for (int c2 = 0; c2 < co; ++c2) first = first && (__ldg(wt + c2 * K + k) == 0.f);
      float2 w[P];
      potential(k, first, w, cpot);
      GrowthP g;
      g.m = __ldg(gf + 2 * k);
      g.s = __ldg(gf + 2 * k + 1);
      g.id = tab.gf[k];
      g.a = GF == GF_FAST_GAUSSIAN ? 0.84932180028801904272f / g.s
                                   : (GF == GF_FAST_POLY4 ? 1.f / (9.f * (g.s * g.s)) : 0.f);
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) {
        acc[k1].x = fmaf(wk, growth_cell<GF>(g, w[k1].x), acc[k1].x);
        acc[k1].y = fmaf(wk, growth_cell<GF>(g, w[k1].y), acc[k1].y);
      }
    }
    // field (weighted_sum / weighted_mean, core.py:202-242), state update, moments
    const size_t base = ((size_t)n * C + co) * N * N;
    const float* sa_row = state + base + (size_t)(2 * r) * N;
    float* da_row = state_out + base + (size_t)(2 * r) * N;
    float* fa_row = field_out ? field_out + base + (size_t)(2 * r) * N : nullptr;
    float Sa = 0.f, Sb = 0.f, Ga = 0.f, Gb = 0.f;
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      const int x = t + G * k1;
      float fa = acc[k1].x, fb = acc[k1].y;
      if (tab.mean) {
        fa = fa / wsum;
        fb = fb / wsum;
      }
      const float sa = __ldg(sa_row + x), sb = __ldg(sa_row + N + x);
      da_row[x] = state_fn(tab.state_fn, sa, fa, dt);
      da_row[N + x] = state_fn(tab.state_fn, sb, fb, dt);
      if (fa_row) {
        fa_row[x] = fa;
        fa_row[N + x] = fb;
      }
      const float fpa = fmaxf(fa, 0.f), fpb = fmaxf(fb, 0.f);
      const float cx = (float)(((x - sx) & (N - 1)) - N / 2);
      Sa += sa;
      Sb += sb;
      Ga += fpa;
      Gb += fpb;
      const float ss = sa + sb, gg = fpa + fpb;
      mxx = fmaf(ss, cx, mxx);
      gxx = fmaf(gg, cx, gxx);
      m2x = fmaf(ss * cx, cx, m2x);
      const bool la = sa > kEps, lb = sb > kEps;
      cmass += (la ? 1.f : 0.f) + (lb ? 1.f : 0.f);
      cgrow += (fpa > kEps ? 1.f : 0.f) + (fpb > kEps ? 1.f : 0.f);
      border |= ((x == 0 || x == N - 1) && (la || lb)) || (r == 0 && la) || (r == N / 2 - 1 && lb);
    }
    m00 += Sa + Sb;
    g00 += Ga + Gb;
    mxy += cya * Sa + cyb * Sb;
    gxy += cya * Ga + cyb * Gb;
    m2y += cya * cya * Sa + cyb * cyb * Sb;
    const float cms = warp_sum(Sa + Sb);
    if (lane == 0) red[wid * RAWS_MAX + RAW_CM + co] = cms;
  }
  // kernels that feed no channel still count in potential_volume
  for (int k = 0; k < K; ++k) {
    bool unused = true;
    for (int c2 = 0; c2 < C; ++c2) unused = unused && (__ldg(wt + c2 * K + k) == 0.f);
    if (!unused) continue;
    float2 w[P];
    potential(k, true, w, cpot);
  }
  // block reduction: warp shuffles then shared memory
  float acc[11] = {m00, g00, cpot, cmass, cgrow, mxy, mxx, gxy, gxx, m2y, m2x};
#pragma unroll
  for (int i = 0; i < 11; ++i) acc[i] = warp_sum(acc[i]);
  const bool anyb = __any_sync(0xffffffffu, border);
  if (lane == 0) {
    float* rd = red + wid * RAWS_MAX;
    rd[RAW_M00] = acc[0];
    rd[RAW_G00] = acc[1];
    rd[RAW_CNT_POT] = acc[2];
    rd[RAW_CNT_MASS] = acc[3];
    rd[RAW_CNT_GROW] = acc[4];
    rd[RAW_MX + 0] = acc[5];
    rd[RAW_MX + 1] = acc[6];
    rd[RAW_MX + 2] = 0.f;
    rd[RAW_GX + 0] = acc[7];
    rd[RAW_GX + 1] = acc[8];
    rd[RAW_GX + 2] = 0.f;
    rd[RAW_MX2 + 0] = acc[9];
    rd[RAW_MX2 + 1] = acc[10];
    rd[RAW_MX2 + 2] = 0.f;
    rd[RAW_BORDER] = anyb ? 1.f : 0.f;
    rd[RAW_SHIFT + 0] = rd[RAW_SHIFT + 1] = rd[RAW_SHIFT + 2] = 0.f;
  }
  __syncthreads();
  const int RAWS = raw_stride(C);
  if (threadIdx.x < RAWS) {
    float s = 0.f;
    for (int w = 0; w < NWARPS; ++w) s += red[w * RAWS_MAX + threadIdx.x];
    if (threadIdx.x == RAW_BORDER) s = s > 0.f ? 1.f : 0.f;
    partial[((size_t)n * BPW + (blockIdx.x % BPW)) * RAWS + threadIdx.x] = s;
  }
}

// ----------------------------------------------------------------- reduce
// One warp per world: sum the block partials, write the step's raw moments,
// update the carried torus shift with trunc(centroid) (statistics.py:117-119).
__global__ void reduce_kernel(int n_worlds, int n_init, int bpw, int C, int H, int W, const float* __restrict__ partial,
                              float* __restrict__ raw, long raw_sol_stride, long raw_init_stride, int* __restrict__ shift) {
  const int n = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (n >= n_worlds) return;
  const int RAWS = raw_stride(C);
  const int sol = n / n_init, init = n - sol * n_init;
  float* rw = raw ? raw + sol * raw_sol_stride + init * raw_init_stride : nullptr;
  float m00 = 0.f, mxy = 0.f, mxx = 0.f;
  const int sh0 = shift[3 * n], sh1 = shift[3 * n + 1];
  for (int s = lane; s < RAWS; s += 32) {
    float v = 0.f;
    for (int b = 0; b < bpw; ++b) v += partial[((size_t)n * bpw + b) * RAWS + s];
    if (s == RAW_BORDER) v = v > 0.f ? 1.f : 0.f;
    if (s == RAW_SHIFT) v = (float)sh0;
    if (s == RAW_SHIFT + 1) v = (float)sh1;
    if (s == RAW_SHIFT + 2) v = 0.f;
    if (rw) rw[s] = v;
    if (s == RAW_M00) m00 = v;
    if (s == RAW_MX) mxy = v;
    if (s == RAW_MX + 1) mxx = v;
  }
  __syncwarp();
  m00 = __shfl_sync(0xffffffffu, m00, RAW_M00);
  mxy = __shfl_sync(0xffffffffu, mxy, RAW_MX);
  mxx = __shfl_sync(0xffffffffu, mxx, RAW_MX + 1);
  if (lane == 0) {
    const float cy = mxy / (m00 + kEps), cx = mxx / (m00 + kEps);
    shift[3 * n] = pmod(sh0 + (int)cy, H);
    shift[3 * n + 1] = pmod(sh1 + (int)cx, W);
  }
}

template <int N>
__global__ void prepare_streamed_kernel(long n_planes, const float2* __restrict__ kh, float2* __restrict__ kp) {
  constexpr int KP = N / 2 + 2, HW = N / 2 + 1;
  const float scale = 1.f / (2.f * (float)N * (float)N);
  const long total = n_planes * N * KP;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % KP);
    const long row = i / KP;
    const float2* src = kh + row * HW;
    float2 o = make_float2(0.f, 0.f);
    if (c == 0) {
      float2 k0 = src[0], kn = src[N / 2];
      o = make_float2((k0.x + kn.x) * scale, (k0.y + kn.y) * scale);
    } else if (c == N / 2) {
      float2 k0 = src[0], kn = src[N / 2];
      o = make_float2((k0.x - kn.x) * scale, (k0.y - kn.y) * scale);
    } else if (c < N / 2) {
      float2 k = src[c];
      o = make_float2(k.x * scale, k.y * scale);
    }
    kp[i] = o;
  }
}

template <int N>
size_t row_inv_smem() {
  using RC = RowInvCfg<N>;
  using GE = Geo<N, RC::G>;
  return (size_t)3 * N * sizeof(float2) + (size_t)RC::GPB * GE::SCR * sizeof(float2) +
         (size_t)(RC::T / 32) * (RAW_CM + kMaxChannels) * sizeof(float);
}

template <int N, int GF>
cudaError_t launch_row_inv(const StreamedStep& s, const KTab& tab, cudaStream_t st) {
  using RC = RowInvCfg<N>;
  const size_t sm_inv = row_inv_smem<N>();
  cudaError_t e = cudaFuncSetAttribute(row_inv_kernel<N, GF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_inv);
  if (e != cudaSuccess) return e;
  row_inv_kernel<N, GF><<<(unsigned)((long)s.n_worlds * RC::BPW), RC::T, sm_inv, st>>>(
      s.n_worlds, s.n_init, tab, s.prod, s.gf, s.gf_sol_stride, s.w, s.w_sol_stride, s.dt, s.state, s.state_out,
      s.field_out, s.pot_out, s.shift, s.partial);
  return cudaGetLastError();
}

template <int N>
cudaError_t step_n(const StreamedStep& s, cudaStream_t st) {
  const Model& m = *s.m;
  constexpr int G = SCfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int GPB = kThreads / G;
  constexpr int BPP = (N / 2 + GPB - 1) / GPB;
  KTab tab;
  tab.C = m.C;
  tab.K = m.K;
  tab.max_k = m.max_k;
  tab.mean = m.mean;
  tab.state_fn = m.state_fn;
  tab.dt_mode = s.dt_mode;
  for (int k = 0; k < m.K; ++k) {
    tab.cin[k] = m.cin[k];
    tab.slot[k] = m.slot[k];
    tab.gf[k] = m.gf[k];
  }
  const size_t sm_fwd = (size_t)3 * N * sizeof(float2) + (size_t)GPB * GE::SCR * sizeof(float2);
  constexpr int CGPB = kColThreads / G;
  constexpr int CBPP = (N / 2 + CGPB - 1) / CGPB;
  const size_t sm_col = (size_t)3 * N * sizeof(float2) + (size_t)CGPB * GE::SCR * sizeof(float2) +
                        (size_t)N * sizeof(float2);  // + DC / Nyquist mirror
  cudaError_t e;
  e = cudaFuncSetAttribute(row_fwd_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_fwd);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(col_conv_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_col);
  if (e != cudaSuccess) return e;
  const long planes = (long)s.n_worlds * m.C;
  row_fwd_kernel<N><<<(unsigned)(planes * BPP), kThreads, sm_fwd, st>>>(s.n_worlds, m.C, s.state, s.spec);
  col_conv_kernel<N><<<(unsigned)(planes * CBPP), kColThreads, sm_col, st>>>(s.n_worlds, s.n_init, tab, s.spec, s.kp,
                                                                           s.kp_sol_stride, s.prod);
  using RC = RowInvCfg<N>;
  bool all_gauss = true, all_poly = true;
  for (int k = 0; k < m.K; ++k) {
    all_gauss = all_gauss && m.gf[k] == LGX_GF_GAUSSIAN;
    all_poly = all_poly && m.gf[k] == LGX_GF_POLY_QUAD4;
  }
  if (all_gauss) e = launch_row_inv<N, GF_FAST_GAUSSIAN>(s, tab, st);
  else if (all_poly) e = launch_row_inv<N, GF_FAST_POLY4>(s, tab, st);
  else e = launch_row_inv<N, GF_GENERIC>(s, tab, st);
  if (e != cudaSuccess) return e;
  const int wpb = 8;
  reduce_kernel<<<(s.n_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(s.n_worlds, s.n_init, RC::BPW, m.C, N, N,
                                                                  s.partial, s.raw, s.raw_sol_stride,
                                                                  s.raw_world_stride, s.shift);
  return cudaGetLastError();
}

}  // namespace

bool streamed_supported(const Model& m) {
  if (m.nb_dims != 2 || m.H != m.W) return false;
  if (m.C > kMaxChannels || m.K > kMaxKernels) return false;
  if (!(m.H == 32 || m.H == 64 || m.H == 128 || m.H == 256)) return false;
  return true;
}

int streamed_blocks_per_world(const Model& m) {
  switch (m.H) {
    case 32: return RowInvCfg<32>::BPW;
    case 64: return RowInvCfg<64>::BPW;
    case 128: return RowInvCfg<128>::BPW;
    case 256: return RowInvCfg<256>::BPW;
  }
  return 1;
}

size_t streamed_workspace_bytes(const Model& m, int n_worlds, int n_sols) {
  const size_t plane = (size_t)m.H * m.W * sizeof(float);  // packed spectrum plane == state plane bytes
  size_t b = 0;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  b += al(plane * n_worlds * m.C);                                          // spec
  b += al(plane * n_worlds * m.K);                                          // prod
  b += al((size_t)n_sols * m.C * m.max_k * m.H * (m.W / 2 + 2) * sizeof(float2));  // kp
  b += al((size_t)n_worlds * streamed_blocks_per_world(m) * raw_stride(m.C) * sizeof(float));  // partial
  b += al((size_t)n_worlds * 3 * sizeof(int));                              // shift
  return b;
}

cudaError_t launch_streamed_step(const StreamedStep& s, cudaStream_t st) {
  switch (s.m->H) {
    case 32: return step_n<32>(s, st);
    case 64: return step_n<64>(s, st);
    case 128: return step_n<128>(s, st);
    case 256: return step_n<256>(s, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_prepare_streamed_spectrum(const Model& m, int n_sols, const float2* k_half, float2* kp,
                                             cudaStream_t st) {
  const long planes = (long)n_sols * m.C * m.max_k;
  const long total = planes * m.H * (m.W / 2 + 2);
  const int threads = 256;
  const int blocks = (int)std::min<long>((total + threads - 1) / threads, 8192);
  switch (m.H) {
    case 32: prepare_streamed_kernel<32><<<blocks, threads, 0, st>>>(planes, k_half, kp); break;
    case 64: prepare_streamed_kernel<64><<<blocks, threads, 0, st>>>(planes, k_half, kp); break;
    case 128: prepare_streamed_kernel<128><<<blocks, threads, 0, st>>>(planes, k_half, kp); break;
    case 256: prepare_streamed_kernel<256><<<blocks, threads, 0, st>>>(planes, k_half, kp); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace lgx
