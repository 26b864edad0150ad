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

constexpr int kThreads = 256;

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
__global__ void __launch_bounds__(kThreads) col_conv_kernel(int n_worlds, int n_init, KTab tab,
                                                            const float2* __restrict__ spec,
                                                            const float2* __restrict__ kp, long kp_sol_stride,
                                                            float2* __restrict__ prod) {
  constexpr int G = SCfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q, GPB = kThreads / G;
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
  float2 mir[P];
  if (c == 0) {
    const int src_lane = (lane & ~(G - 1)) | ((G - t) & (G - 1));
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      float2 val = (t != 0) ? w0[P - 1 - k1] : w0[(P - k1) & (P - 1)];
      mir[k1].x = __shfl_sync(gmask, val.x, src_lane);
      mir[k1].y = __shfl_sync(gmask, val.y, src_lane);
    }
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
        float2 A = __ldg(kk + ky * KPITCH), B = __ldg(kk + ky * KPITCH + N / 2);
        w[k1] = cadd(cmul(w0[k1], A), cmul(conjf2(mir[k1]), B));
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
// Block = GPB groups = GPB packed rows of one world.  Field accumulators for
// the block's 2*GPB rows live in shared memory ([C][2*GPB][N] floats).
template <int N>
struct RowInvCfg {
  static constexpr int G = SCfg<N>::G;
  static constexpr int T = ((N / 2) * G < 128) ? (N / 2) * G : 128;  // threads per block
  static constexpr int GPB = T / G;
  static constexpr int BPW = (N / 2) / GPB;  // blocks per world
};

template <int N>
__global__ void __launch_bounds__(128) row_inv_kernel(int n_worlds, int n_init, KTab tab, const float2* __restrict__ prod,
                                                      const float* __restrict__ gfp, long gf_sol_stride,
                                                      const float* __restrict__ wts, long w_sol_stride,
                                                      const float* __restrict__ dtp, const float* __restrict__ state,
                                                      float* __restrict__ state_out, float* __restrict__ field_out,
                                                      float* __restrict__ pot_out, const int* __restrict__ shift,
                                                      float* __restrict__ partial) {
  using RC = RowInvCfg<N>;
  constexpr int G = RC::G, GPB = RC::GPB, BPW = RC::BPW;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q;
  constexpr int RAWS_MAX = RAW_CM + kMaxChannels;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = init_tw<N>(sm);  // GPB * SCR
  float* facc = reinterpret_cast<float*>(scr + GPB * GE::SCR);  // [C][2*GPB][N]
  float* red = facc + tab.C * 2 * GPB * N;                      // [warps][RAWS_MAX]
  const int n = blockIdx.x / BPW;
  if (n >= n_worlds) return;
  const int sol = n / n_init;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r = (blockIdx.x % BPW) * GPB + grp;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int C = tab.C;
  for (int i = threadIdx.x; i < C * 2 * GPB * N; i += blockDim.x) facc[i] = 0.f;
  __syncthreads();
  float2* rs = scr + grp * GE::SCR;
  const float* gf = gfp + sol * gf_sol_stride;
  const float* wt = wts + sol * w_sol_stride;
  float cpot = 0.f;

  for (int k = 0; k < tab.K; ++k) {
    const float2* pr = prod + (((size_t)n * tab.K + k) * (N / 2) + r) * N;
    float2 v[Q][G];
#pragma unroll
    for (int jp = 0; jp < Q / 2; ++jp) {
      const int m = t + G * jp;
      if (m != 0) {
#pragma unroll
        for (int n2 = 0; n2 < G; ++n2) {
          const int kx = m + P * n2, kk = N - kx;
          float2 zk, zkk;
          if (n2 < G / 2) {
            float2 s1 = pr[kx], s2 = pr[kk];
            zk = make_float2(s1.x - s2.y, s1.y + s2.x);
            zkk = make_float2(s1.x + s2.y, s2.x - s1.y);
          } else {
            float2 s1 = pr[kk], s2 = pr[kx];
            zkk = make_float2(s1.x - s2.y, s1.y + s2.x);
            zk = make_float2(s1.x + s2.y, s2.x - s1.y);
          }
          v[2 * jp][n2] = zk;
          v[2 * jp + 1][G - 1 - n2] = zkk;
        }
      } else {
        float2 s0 = pr[0], sn = pr[N / 2];
        v[2 * jp][0] = make_float2(s0.x, sn.x);
        v[2 * jp][G / 2] = make_float2(s0.y, sn.y);
#pragma unroll
        for (int n2 = 1; n2 < G / 2; ++n2) {
          const int kx = P * n2, kk = N - kx;
          float2 s1 = pr[kx], s2 = pr[kk];
          v[2 * jp][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
          v[2 * jp][G - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
        }
#pragma unroll
        for (int n2 = 0; n2 < G / 2; ++n2) {
          const int kx = P / 2 + P * n2, kk = N - kx;
          float2 s1 = pr[kx], s2 = pr[kk];
          v[2 * jp + 1][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
          v[2 * jp + 1][G - 1 - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
        }
      }
    }
    float2 w[P];
    fft_mirrored<GE, true, true>(v, w, rs, sm + 2 * N, t, gmask);
    const float gm = __ldg(gf + 2 * k), gs = __ldg(gf + 2 * k + 1);
    const int gid = tab.gf[k];
    if (pot_out) {
      float* po = pot_out + ((size_t)n * tab.K + k) * N * N;
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) {
        po[(2 * r) * N + t + G * k1] = w[k1].x;
        po[(2 * r + 1) * N + t + G * k1] = w[k1].y;
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      float2 g = make_float2(growth_fn(gid, w[k1].x, gm, gs), growth_fn(gid, w[k1].y, gm, gs));
      cpot += (w[k1].x > kEps ? 1.f : 0.f) + (w[k1].y > kEps ? 1.f : 0.f);
      w[k1] = g;
    }
    for (int co = 0; co < C; ++co) {
      const float wk = __ldg(wt + co * tab.K + k);
      if (wk == 0.f) continue;
      float* fa = facc + (co * 2 * GPB + 2 * grp) * N;
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) {
        const int x = t + G * k1;
        fa[x] = fmaf(wk, w[k1].x, fa[x]);
        fa[N + x] = fmaf(wk, w[k1].y, fa[N + x]);
      }
    }
  }

  // field, state update, moments
  float dt;
  if (tab.dt_mode == 0) dt = __ldg(dtp);
  else if (tab.dt_mode == 1) dt = __ldg(dtp + n);
  else dt = 1.f / __ldg(dtp + sol);
  const int sy = shift[3 * n], sx = shift[3 * n + 1];
  float m00 = 0.f, g00 = 0.f, cmass = 0.f, cgrow = 0.f, mxy = 0.f, mxx = 0.f, gxy = 0.f, gxx = 0.f, m2y = 0.f,
        m2x = 0.f;
  bool border = false;
  float cm_part[kMaxChannels];
#pragma unroll
  for (int i = 0; i < kMaxChannels; ++i) cm_part[i] = 0.f;
  for (int co = 0; co < C; ++co) {
    float wsum = 0.f;
    for (int k = 0; k < tab.K; ++k) wsum += __ldg(wt + co * tab.K + k);
    const float* fa = facc + (co * 2 * GPB + 2 * grp) * N;
    const size_t base = ((size_t)n * C + co) * N * N;
    float cms = 0.f;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int y = 2 * r + e;
      const float cy = (float)(((y - sy) & (N - 1)) - N / 2);
#pragma unroll 4
      for (int k1 = 0; k1 < P; ++k1) {
        const int x = t + G * k1;
        float f = fa[e * N + x];
        if (tab.mean) f = f / wsum;
        const float s = __ldg(state + base + y * N + x);
        state_out[base + y * N + x] = state_fn(tab.state_fn, s, f, dt);
        if (field_out) field_out[base + y * N + x] = f;
        const float fp = fmaxf(f, 0.f);
        const float cx = (float)(((x - sx) & (N - 1)) - N / 2);
        m00 += s;
        cms += s;
        g00 += fp;
        cmass += s > kEps ? 1.f : 0.f;
        cgrow += fp > kEps ? 1.f : 0.f;
        mxy = fmaf(s, cy, mxy);
        mxx = fmaf(s, cx, mxx);
        gxy = fmaf(fp, cy, gxy);
        gxx = fmaf(fp, cx, gxx);
        m2y = fmaf(s * cy, cy, m2y);
        m2x = fmaf(s * cx, cx, m2x);
        if ((x == 0 || x == N - 1 || y == 0 || y == N - 1) && s > kEps) border = true;
      }
    }
    if (co < kMaxChannels) cm_part[co] = cms;
  }
  // block reduction: warp shuffles then shared memory
  float acc[12] = {m00, g00, cpot, cmass, cgrow, mxy, mxx, gxy, gxx, m2y, m2x, 0.f};
  const int nwarps = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < 11; ++i) acc[i] = warp_sum(acc[i]);
  const bool anyb = __any_sync(0xffffffffu, border);
  for (int co = 0; co < C; ++co) cm_part[co] = warp_sum(cm_part[co]);
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
    for (int co = 0; co < C; ++co) rd[RAW_CM + co] = cm_part[co];
  }
  __syncthreads();
  const int RAWS = raw_stride(C);
  if (threadIdx.x < RAWS) {
    float s = 0.f;
    for (int w = 0; w < nwarps; ++w) s += red[w * RAWS_MAX + threadIdx.x];
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
size_t row_inv_smem(int C) {
  using RC = RowInvCfg<N>;
  using GE = Geo<N, RC::G>;
  return (size_t)3 * N * sizeof(float2) + (size_t)RC::GPB * GE::SCR * sizeof(float2) +
         (size_t)C * 2 * RC::GPB * N * sizeof(float) + (size_t)(RC::T / 32) * (RAW_CM + kMaxChannels) * sizeof(float);
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
  cudaError_t e;
  e = cudaFuncSetAttribute(row_fwd_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_fwd);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(col_conv_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_fwd);
  if (e != cudaSuccess) return e;
  const long planes = (long)s.n_worlds * m.C;
  row_fwd_kernel<N><<<(unsigned)(planes * BPP), kThreads, sm_fwd, st>>>(s.n_worlds, m.C, s.state, s.spec);
  col_conv_kernel<N><<<(unsigned)(planes * BPP), kThreads, sm_fwd, st>>>(s.n_worlds, s.n_init, tab, s.spec, s.kp,
                                                                           s.kp_sol_stride, s.prod);
  using RC = RowInvCfg<N>;
  const size_t sm_inv = row_inv_smem<N>(m.C);
  e = cudaFuncSetAttribute(row_inv_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_inv);
  if (e != cudaSuccess) return e;
  row_inv_kernel<N><<<(unsigned)((long)s.n_worlds * RC::BPW), RC::T, sm_inv, st>>>(
      s.n_worlds, s.n_init, tab, s.prod, s.gf, s.gf_sol_stride, s.w, s.w_sol_stride, s.dt, s.state, s.state_out,
      s.field_out, s.pot_out, s.shift, s.partial);
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
  // row_inv keeps C field planes of its rows in shared memory
  size_t smem = 0;
  switch (m.H) {
    case 32: smem = row_inv_smem<32>(m.C); break;
    case 64: smem = row_inv_smem<64>(m.C); break;
    case 128: smem = row_inv_smem<128>(m.C); break;
    case 256: smem = row_inv_smem<256>(m.C); break;
  }
  return smem <= 227 * 1024;
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
