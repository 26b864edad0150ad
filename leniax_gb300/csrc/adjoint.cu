// Adjoint (reverse-mode) Lenia step for 2D single-channel single-kernel
// worlds, and the real-kernel -> half-spectrum transform.
//
// Forward map of one step (core.py:13-49 with get_state v1/v2/simple):
//   u = K (*) s           circular convolution (get_potential_fft)
//   f = wf * G(u; m, s)   growth, weighted with one kernel
//   s' = clip(s + dt f)   (v1) | s (1 - dt) + dt f (v2) | s + dt f (simple)
// Given lambda' = dL/ds', one adjoint step computes
//   mu     = lambda' * clip'(s + dt f)          clip' = 1 (straight-through,
//                                               as leniax's get_state v1,
//                                               core.py:267-270) or 1[0<n<1]
//   a      = dL/du = dt * mu * wf * G'(u)
//   lambda = mu * (1 - dt if v2 else 1) + K (*)^T a     (correlation: the
//            spectrum of a times conj(K^))
//   dL/dm, dL/ds, dL/dw  += sums of dt * mu * df/dparam
//   dL/dK  += a (*)^T s  (accumulated as spectrum(a) * conj(spectrum(s)))
// Kernels of one adjoint step: adj_rows (pointwise adjoint + row FFTs of the
// a and s planes) -> col_adj -> row_inv_add; the parameter partials are
// reduced once per segment.  The same packed real-FFT
// passes as the streamed engine are used (rows paired as one complex row,
// columns 0 and N/2 packed together).
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "engine.h"
#include "fft.cuh"

namespace lgx {

namespace {

template <int N>
struct ACfg;
template <>
struct ACfg<32> { static constexpr int G = 4; };
template <>
struct ACfg<64> { static constexpr int G = 4; };
template <>
struct ACfg<128> { static constexpr int G = 8; };
template <>
struct ACfg<256> { static constexpr int G = 8; };

constexpr int kT = 256;  // threads per block of the FFT pass kernels

template <int N>
__device__ __forceinline__ float2* twiddles(float2* sm) {
  using GE = Geo<N, ACfg<N>::G>;
  init_twiddles<GE>(sm, sm + N, sm + 2 * N, threadIdx.x, blockDim.x);
  return sm + 3 * N;
}

struct AdjParams {
  int n_worlds, n_init, gf_id, state_fn, mean, clip_mask;
  const float* gf;  // [Ns, 2]
  const float* w;   // [Ns]
  const float* T;   // [Ns]
};

// growth value and its derivatives d/du, d/dm, d/ds (growth_functions.py)
__device__ __forceinline__ void growth_and_grads(int id, float u, float m, float s, float& g, float& gu, float& gm,
                                                 float& gs) {
  if (id == LGX_GF_GAUSSIAN || id == LGX_GF_GAUSSIAN_TARGET) {
    const float d = (u - m) / s;
    const float e = expf(-(d * d) / 2.f);
    const float amp = id == LGX_GF_GAUSSIAN ? 2.f : 1.f;
    g = id == LGX_GF_GAUSSIAN ? 2.f * e - 1.f : e;
    gu = -amp * e * d / s;
    gm = -gu;
    gs = amp * e * d * d / s;
  } else if (id == LGX_GF_POLY_QUAD4) {
    const float d = u - m, c = 9.f * s * s;
    const float q = 1.f - d * d / c;
    if (q > 0.f) {
      const float q3 = q * q * q;
      g = 2.f * q3 * q - 1.f;
      gu = 8.f * q3 * (-2.f * d / c);
      gm = -gu;
      gs = 8.f * q3 * (2.f * d * d / (c * s));
    } else {
      g = -1.f;
      gu = gm = gs = 0.f;
    }
  } else {  // identity and the piecewise-constant families: d/du = 1 or 0
    g = growth_fn(id, u, m, s);
    gu = id == LGX_GF_IDENTITY ? 1.f : 0.f;
    gm = gs = 0.f;
  }
}

// per solution: grad_gf[s] += (dm, ds), grad_w[s] += dw over its inits and blocks
__global__ void adj_param_reduce_kernel(int n_sols, int n_init, int blocks, const float* __restrict__ partial,
                                        float* __restrict__ grad_gf, float* __restrict__ grad_w) {
  const int sol = blockIdx.x;
  float v[3] = {0.f, 0.f, 0.f};
  for (int i = threadIdx.x; i < n_init * blocks; i += blockDim.x) {
    const int init = i / blocks, b = i % blocks;
    const float* pp = partial + ((size_t)(sol * n_init + init) * blocks + b) * 3;
    v[0] += pp[0];
    v[1] += pp[1];
    v[2] += pp[2];
  }
  __shared__ float red[3][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < 3; ++k) {
    const float s = warp_sum(v[k]);
    if (lane == 0) red[k][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
    if (threadIdx.x < 2) grad_gf[2 * sol + threadIdx.x] += s;
    else grad_w[sol] += s;
  }
}

// ------------------------------------------------------------ row_fwd (planes)
template <int N>
__global__ void __launch_bounds__(kT) adj_row_fwd_kernel(int planes, const float* __restrict__ x,
                                                         float2* __restrict__ spec) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = twiddles<N>(sm);
  __syncthreads();
  const int plane = blockIdx.x / BPP;
  if (plane >= planes) return;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int r = (blockIdx.x % BPP) * GPB + grp;
  if (r >= N / 2) return;  // whole warps (see launch shapes)
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const float* src = x + (size_t)plane * N * N;
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

// ------------------------------------------------------------- adj_rows
// Pointwise adjoint fused with the row FFTs: per (world, packed row pair) the
// direct term lambda_next, a = dL/du and the row spectra of a (plane 2n) and
// s (plane 2n+1); per-block partial sums of dL/dm, dL/ds, dL/dw accumulate
// over the segment's steps in pacc (one slot per block, reduced once per
// segment).
template <int N>
__global__ void __launch_bounds__(kT) adj_rows_kernel(AdjParams p, const float* __restrict__ lam_in,
                                                      const float* __restrict__ s_t, const float* __restrict__ u_t,
                                                      const float* __restrict__ s_next, float* __restrict__ lam_next,
                                                      float2* __restrict__ spec, float* __restrict__ pacc) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = twiddles<N>(sm);
  __shared__ float red[3][kT / 32];
  __syncthreads();
  const int n = blockIdx.x / BPP;
  if (n >= p.n_worlds) return;  // whole blocks
  const int sol = n / p.n_init;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r = (blockIdx.x % BPP) * GPB + grp;
  const bool active = r < N / 2;  // idle groups (small N) still reach the block barrier
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  float am = 0.f, as = 0.f, aw = 0.f;
  if (active) {
    const float m = __ldg(p.gf + 2 * sol), sg = __ldg(p.gf + 2 * sol + 1);
    const float wk = __ldg(p.w + sol), dt = 1.f / __ldg(p.T + sol);
    const float wf = p.mean ? wk / wk : wk;
    const size_t base = (size_t)n * N * N + (size_t)(2 * r) * N;
    float2 va[P], vs[P];
#pragma unroll
    for (int n2 = 0; n2 < P; ++n2) {
      float ae[2], se[2];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const size_t off = base + (size_t)e * N + t + G * n2;
        const float lam = lam_in[off], sv = __ldg(s_t + off), u = __ldg(u_t + off);
        float g, gu, gm, gs;
        growth_and_grads(p.gf_id, u, m, sg, g, gu, gm, gs);
        float mu = lam;
        if (p.state_fn == LGX_STATE_V1 && p.clip_mask) {
          // the forward's clip was inactive where its output lies strictly inside (0, 1)
          const float nn = s_next ? __ldg(s_next + off) : sv + dt * (g * wf);
          mu = (nn > 0.f && nn < 1.f) ? lam : 0.f;
        }
        lam_next[off] = p.state_fn == LGX_STATE_V2 ? mu * (1.f - dt) : mu;
        const float dfl = dt * mu;  // dL/df
        ae[e] = dfl * wf * gu;      // a = dL/du
        se[e] = sv;
        am += dfl * wf * gm;
        as += dfl * wf * gs;
        aw += p.mean ? 0.f : dfl * g;  // weighted_sum: f = w g; weighted_mean with one kernel: f = g
      }
      va[n2] = make_float2(ae[0], ae[1]);
      vs[n2] = make_float2(se[0], se[1]);
    }
    float2 u[Q][G];
    float2* rs = scr + grp * GE::SCR;
    fft_standard<GE, false, false>(va, u, rs, sm, t, gmask);
    float2* da = spec + ((size_t)(2 * n) * (N / 2) + r) * N;
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int k1 = 0; k1 < G; ++k1) da[t + G * q + P * k1] = u[q][k1];
    fft_standard<GE, false, false>(vs, u, rs, sm, t, gmask);
    float2* ds = spec + ((size_t)(2 * n + 1) * (N / 2) + r) * N;
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int k1 = 0; k1 < G; ++k1) ds[t + G * q + P * k1] = u[q][k1];
  }
  am = warp_sum(am);
  as = warp_sum(as);
  aw = warp_sum(aw);
  if (lane == 0) {
    red[0][wid] = am;
    red[1][wid] = as;
    red[2][wid] = aw;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    float v = 0.f;
    for (int w = 0; w < kT / 32; ++w) v += red[threadIdx.x][w];
    pacc[((size_t)n * BPP + blockIdx.x % BPP) * 3 + threadIdx.x] += v;
  }
}

// Load column pair c of a packed-row spectrum plane and run the forward column
// FFT: w[k1] = column spectrum at ky = t + G*k1 (x2 for c > 0; packed
// DC + i Nyquist for c == 0).
template <int N>
__device__ __forceinline__ void column_forward(const float2* sp, int c, int t, unsigned gmask, float2* cs,
                                               const float2* tw_colf, float2 (&w)[Geo<N, ACfg<N>::G>::P]) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q;
  float2 v[Q][G];
#pragma unroll
  for (int jp = 0; jp < Q / 2; ++jp) {
    const int m = t + G * jp;
#pragma unroll
    for (int n2 = 0; n2 < G; ++n2) {
      const int r = m + (P / 2) * n2;
      if (c != 0) {
        const float2 z1 = sp[r * N + c], z2 = sp[r * N + N - c];
        v[2 * jp][n2] = caddc(z1, z2);
        const float2 d = csubc(z1, z2);
        v[2 * jp + 1][n2] = make_float2(d.y, -d.x);
      } else {
        const float2 z1 = sp[r * N], z2 = sp[r * N + N / 2];
        v[2 * jp][n2] = make_float2(z1.x, z2.x);
        v[2 * jp + 1][n2] = make_float2(z1.y, z2.y);
      }
    }
  }
  fft_mirrored<GE, false, false>(v, w, cs, tw_colf, t, gmask);
}

// Inverse column FFT of w (ky = t + G*k1) and store into packed rows of pd.
template <int N>
__device__ __forceinline__ void column_inverse_store(float2 (&w)[Geo<N, ACfg<N>::G>::P], int c, int t,
                                                     unsigned gmask, float2* cs, const float2* tw_std, float2* pd) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q;
  float2 u[Q][G];
  fft_standard<GE, true, true>(w, u, cs, tw_std, t, gmask);
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

// ------------------------------------------------------------------ col_adj
// Per (world, column pair): spectra of a and s, kernel-gradient accumulation,
// correlation with conj(K^) and inverse column FFT into prod.
// gk layout: [world][c][ky] complex; c == 0 holds the packed (DC + i Nyquist)
// products, the other columns 4 x spectrum(a) x conj(spectrum(s)).
template <int N>
__global__ void __launch_bounds__(kT) col_adj_kernel(int n_worlds, int n_init, const float2* __restrict__ spec,
                                                     const float2* __restrict__ kp, long kp_sol_stride,
                                                     float2* __restrict__ gk, float2* __restrict__ prod) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = twiddles<N>(sm);
  __syncthreads();
  const int n = blockIdx.x / BPP;
  if (n >= n_worlds) return;
  const int sol = n / n_init;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int c = (blockIdx.x % BPP) * GPB + grp;
  if (c >= N / 2) return;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  float2* cs = scr + grp * GE::SCR;
  float2 wa[P], ws[P];
  column_forward<N>(spec + (size_t)(2 * n) * (N / 2) * N, c, t, gmask, cs, sm + N, wa);
  column_forward<N>(spec + (size_t)(2 * n + 1) * (N / 2) * N, c, t, gmask, cs, sm + N, ws);
  const float2* kk = kp + sol * kp_sol_stride;
  float2* g = gk + ((size_t)n * (N / 2) + c) * N;
  if (c != 0) {
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      const int ky = t + G * k1;
      g[ky] = cadd(g[ky], cmulc(wa[k1], ws[k1]));
      wa[k1] = cmulc(wa[k1], __ldg(kk + (size_t)c * N + ky));
    }
  } else {
    // unpack DC / Nyquist columns of a and s through the scratch mirror
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) cs[t + G * k1] = wa[k1];
    __syncwarp(gmask);
    float2 ma[P];
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) ma[k1] = cs[(N - (t + G * k1)) & (N - 1)];
    __syncwarp(gmask);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) cs[t + G * k1] = ws[k1];
    __syncwarp(gmask);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      const int ky = t + G * k1;
      const float2 msv = cs[(N - ky) & (N - 1)];
      // X0 = (C + conj(C-))/2, XN = (C - conj(C-))/(2i)
      const float2 a0 = make_float2(0.5f * (wa[k1].x + ma[k1].x), 0.5f * (wa[k1].y - ma[k1].y));
      const float2 aN = make_float2(0.5f * (wa[k1].y + ma[k1].y), 0.5f * (ma[k1].x - wa[k1].x));
      const float2 s0 = make_float2(0.5f * (ws[k1].x + msv.x), 0.5f * (ws[k1].y - msv.y));
      const float2 sN = make_float2(0.5f * (ws[k1].y + msv.y), 0.5f * (msv.x - ws[k1].x));
      const float2 g0 = cmulc(a0, s0), gN = cmulc(aN, sN);
      g[ky] = cadd(g[ky], make_float2(g0.x - gN.y, g0.y + gN.x));  // g0 + i gN
      // correlation: Q = C conj(A) + conj(C-) conj(B)
      const float2 A = __ldg(kk + ky), B = __ldg(kk + (N / 2) * N + ky);
      wa[k1] = cadd(cmulc(wa[k1], A), cmulc(conjf2(ma[k1]), B));
    }
    __syncwarp(gmask);
  }
  column_inverse_store<N>(wa, c, t, gmask, cs, sm, prod + (size_t)n * (N / 2) * N);
}

// Packed rows -> real rows (inverse row FFT).  out[...] = (accumulate ? out : 0) + scale * result
template <int N>
__device__ __forceinline__ void row_inverse(const float2* pr, int r, int t, unsigned gmask, float2* rs,
                                            const float2* tw_rowi, float2 (&w)[Geo<N, ACfg<N>::G>::P]) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q;
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
          const float2 s1 = pr[kx], s2 = pr[kk];
          zk = make_float2(s1.x - s2.y, s1.y + s2.x);
          zkk = make_float2(s1.x + s2.y, s2.x - s1.y);
        } else {
          const float2 s1 = pr[kk], s2 = pr[kx];
          zkk = make_float2(s1.x - s2.y, s1.y + s2.x);
          zk = make_float2(s1.x + s2.y, s2.x - s1.y);
        }
        v[2 * jp][n2] = zk;
        v[2 * jp + 1][G - 1 - n2] = zkk;
      }
    } else {
      const float2 s0 = pr[0], sn = pr[N / 2];
      v[2 * jp][0] = make_float2(s0.x, sn.x);
      v[2 * jp][G / 2] = make_float2(s0.y, sn.y);
#pragma unroll
      for (int n2 = 1; n2 < G / 2; ++n2) {
        const int kx = P * n2, kk = N - kx;
        const float2 s1 = pr[kx], s2 = pr[kk];
        v[2 * jp][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
        v[2 * jp][G - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
      }
#pragma unroll
      for (int n2 = 0; n2 < G / 2; ++n2) {
        const int kx = P / 2 + P * n2, kk = N - kx;
        const float2 s1 = pr[kx], s2 = pr[kk];
        v[2 * jp + 1][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
        v[2 * jp + 1][G - 1 - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
      }
    }
  }
  fft_mirrored<GE, true, true>(v, w, rs, tw_rowi, t, gmask);
}

template <int N>
__global__ void __launch_bounds__(kT) row_inv_add_kernel(int planes, const float2* __restrict__ prod,
                                                         float* __restrict__ out, float scale, int accumulate) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = twiddles<N>(sm);
  __syncthreads();
  const int plane = blockIdx.x / BPP;
  if (plane >= planes) return;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int r = (blockIdx.x % BPP) * GPB + grp;
  if (r >= N / 2) return;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  float2 w[P];
  row_inverse<N>(prod + ((size_t)plane * (N / 2) + r) * N, r, t, gmask, scr + grp * GE::SCR, sm + 2 * N, w);
  float* o = out + (size_t)plane * N * N;
#pragma unroll
  for (int k1 = 0; k1 < P; ++k1) {
    const int x = t + G * k1;
    const float va = scale * w[k1].x, vb = scale * w[k1].y;
    o[(2 * r) * N + x] = accumulate ? o[(2 * r) * N + x] + va : va;
    o[(2 * r + 1) * N + x] = accumulate ? o[(2 * r + 1) * N + x] + vb : vb;
  }
}

// Kernel-gradient finish: sum a solution's per-world column-domain
// accumulators, scale to a true inverse DFT, inverse column FFT into packed rows.
template <int N>
__global__ void __launch_bounds__(kT) gk_finish_col_kernel(int n_sols, int n_init, const float2* __restrict__ gk,
                                                           float2* __restrict__ prod) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = twiddles<N>(sm);
  __syncthreads();
  const int sol = blockIdx.x / BPP;
  if (sol >= n_sols) return;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int c = (blockIdx.x % BPP) * GPB + grp;
  if (c >= N / 2) return;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  // regular columns hold 4 x true products, the packed column true products;
  // the unnormalised inverse passes need true / (N*N)
  const float scale = (c != 0 ? 0.25f : 1.f) / ((float)N * (float)N);
  float2 w[P];
#pragma unroll
  for (int k1 = 0; k1 < P; ++k1) w[k1] = make_float2(0.f, 0.f);
  for (int i = 0; i < n_init; ++i) {
    const float2* g = gk + ((size_t)(sol * n_init + i) * (N / 2) + c) * N;
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) w[k1] = cadd(w[k1], g[t + G * k1]);
  }
#pragma unroll
  for (int k1 = 0; k1 < P; ++k1) w[k1] = make_float2(w[k1].x * scale, w[k1].y * scale);
  column_inverse_store<N>(w, c, t, gmask, scr + grp * GE::SCR, sm, prod + (size_t)sol * (N / 2) * N);
}

// Real kernel planes -> leniax half spectrum [planes][N][N/2+1] (unscaled fftn).
template <int N>
__global__ void __launch_bounds__(kT) spectrum_col_kernel(int planes, const float2* __restrict__ spec,
                                                          float2* __restrict__ out) {
  constexpr int G = ACfg<N>::G;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB, HW = N / 2 + 1;
  extern __shared__ __align__(16) float2 sm[];
  float2* scr = twiddles<N>(sm);
  __syncthreads();
  const int plane = blockIdx.x / BPP;
  if (plane >= planes) return;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int c = (blockIdx.x % BPP) * GPB + grp;
  if (c >= N / 2) return;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  float2* cs = scr + grp * GE::SCR;
  float2 w[P];
  column_forward<N>(spec + (size_t)plane * (N / 2) * N, c, t, gmask, cs, sm + N, w);
  float2* o = out + (size_t)plane * N * HW;
  if (c != 0) {
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) o[(t + G * k1) * HW + c] = make_float2(0.5f * w[k1].x, 0.5f * w[k1].y);
  } else {
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) cs[t + G * k1] = w[k1];
    __syncwarp(gmask);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      const int ky = t + G * k1;
      const float2 mm = cs[(N - ky) & (N - 1)];
      o[ky * HW] = make_float2(0.5f * (w[k1].x + mm.x), 0.5f * (w[k1].y - mm.y));
      o[ky * HW + N / 2] = make_float2(0.5f * (w[k1].y + mm.y), 0.5f * (mm.x - w[k1].x));
    }
  }
}

template <int N>
size_t pass_smem() {
  using GE = Geo<N, ACfg<N>::G>;
  return (size_t)3 * N * sizeof(float2) + (size_t)(kT / ACfg<N>::G) * GE::SCR * sizeof(float2);
}

template <class K>
cudaError_t allow_smem(K kern, size_t bytes) {
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int N>
cudaError_t adjoint_n(const AdjointSegment& j, cudaStream_t st) {
  constexpr int G = ACfg<N>::G, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  const size_t smem = pass_smem<N>();
  cudaError_t e;
  if ((e = allow_smem(col_adj_kernel<N>, smem)) != cudaSuccess) return e;
  if ((e = allow_smem(row_inv_add_kernel<N>, smem)) != cudaSuccess) return e;
  const int nw = j.n_sols * j.n_init;
  const int cells = N * N;
  AdjParams p;
  p.n_worlds = nw;
  p.n_init = j.n_init;
  p.gf_id = j.gf_id;
  p.state_fn = j.state_fn;
  p.mean = j.mean;
  p.clip_mask = j.clip_mask;
  p.gf = j.gf_params;
  p.w = j.weights;
  p.T = j.T;
  if ((e = allow_smem(adj_rows_kernel<N>, smem)) != cudaSuccess) return e;
  const long kp_sol = (long)N * (N / 2 + 2);
  // per-block parameter partials accumulate over the segment, reduced once
  if ((e = cudaMemsetAsync(j.partial, 0, (size_t)nw * BPP * 3 * sizeof(float), st)) != cudaSuccess) return e;
  // lambda ping-pong: step t reads lam_cur, writes lam_next
  const float* lam_cur = j.lambda_in;
  for (int s = j.steps - 1; s >= 0; --s) {
    float* lam_next = (s == 0) ? j.lambda_out : ((s & 1) ? j.lam_a : j.lam_b);
    const float* st_s = j.traj_cells + (size_t)s * nw * cells;
    const float* st_u = j.traj_potential + (size_t)s * nw * cells;
    const float* st_n = s + 1 < j.steps ? st_s + (size_t)nw * cells : j.cells_after;
    adj_rows_kernel<N><<<(unsigned)(nw * BPP), kT, smem, st>>>(p, lam_cur, st_s, st_u, st_n, lam_next, j.spec,
                                                               j.partial);
    col_adj_kernel<N><<<(unsigned)(nw * BPP), kT, smem, st>>>(nw, j.n_init, j.spec, j.kp, kp_sol, j.gk, j.prod);
    row_inv_add_kernel<N><<<(unsigned)(nw * BPP), kT, smem, st>>>(nw, j.prod, lam_next, 1.f, 1);
    lam_cur = lam_next;
  }
  adj_param_reduce_kernel<<<j.n_sols, 256, 0, st>>>(j.n_sols, j.n_init, BPP, j.partial, j.grad_gf, j.grad_w);
  return cudaGetLastError();
}

template <int N>
cudaError_t gk_finish_n(int n_sols, int n_init, const float2* gk, float2* prod, float* out, cudaStream_t st) {
  constexpr int G = ACfg<N>::G, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  const size_t smem = pass_smem<N>();
  cudaError_t e;
  if ((e = allow_smem(gk_finish_col_kernel<N>, smem)) != cudaSuccess) return e;
  if ((e = allow_smem(row_inv_add_kernel<N>, smem)) != cudaSuccess) return e;
  gk_finish_col_kernel<N><<<(unsigned)(n_sols * BPP), kT, smem, st>>>(n_sols, n_init, gk, prod);
  row_inv_add_kernel<N><<<(unsigned)(n_sols * BPP), kT, smem, st>>>(n_sols, prod, out, 1.f, 0);
  return cudaGetLastError();
}

template <int N>
cudaError_t spectrum_n(int planes, const float* k_real, float2* spec, float2* out, cudaStream_t st) {
  constexpr int G = ACfg<N>::G, GPB = kT / G, BPP = (N / 2 + GPB - 1) / GPB;
  const size_t smem = pass_smem<N>();
  cudaError_t e;
  if ((e = allow_smem(adj_row_fwd_kernel<N>, smem)) != cudaSuccess) return e;
  if ((e = allow_smem(spectrum_col_kernel<N>, smem)) != cudaSuccess) return e;
  adj_row_fwd_kernel<N><<<(unsigned)(planes * BPP), kT, smem, st>>>(planes, k_real, spec);
  spectrum_col_kernel<N><<<(unsigned)(planes * BPP), kT, smem, st>>>(planes, spec, out);
  return cudaGetLastError();
}

}  // namespace

bool adjoint_supported(const Model& m) {
  return m.nb_dims == 2 && m.C == 1 && m.K == 1 && m.H == m.W &&
         (m.H == 32 || m.H == 64 || m.H == 128 || m.H == 256);
}

bool spectrum_supported(int H, int W) { return H == W && (H == 32 || H == 64 || H == 128 || H == 256); }

cudaError_t launch_param_reduce(int n_sols, int n_init, int blocks, const float* partial, float* grad_gf,
                                float* grad_w, cudaStream_t st) {
  adj_param_reduce_kernel<<<n_sols, 256, 0, st>>>(n_sols, n_init, blocks, partial, grad_gf, grad_w);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_segment(int N, const AdjointSegment& j, cudaStream_t st) {
  switch (N) {
    case 32: return adjoint_n<32>(j, st);
    case 64: return adjoint_n<64>(j, st);
    case 128: return adjoint_n<128>(j, st);
    case 256: return adjoint_n<256>(j, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_gk_finish(int N, int n_sols, int n_init, const float2* gk, float2* prod, float* out,
                             cudaStream_t st) {
  switch (N) {
    case 32: return gk_finish_n<32>(n_sols, n_init, gk, prod, out, st);
    case 64: return gk_finish_n<64>(n_sols, n_init, gk, prod, out, st);
    case 128: return gk_finish_n<128>(n_sols, n_init, gk, prod, out, st);
    case 256: return gk_finish_n<256>(n_sols, n_init, gk, prod, out, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_spectrum(int N, int planes, const float* k_real, float2* spec, float2* out, cudaStream_t st) {
  switch (N) {
    case 32: return spectrum_n<32>(planes, k_real, spec, out, st);
    case 64: return spectrum_n<64>(planes, k_real, spec, out, st);
    case 128: return spectrum_n<128>(planes, k_real, spec, out, st);
    case 256: return spectrum_n<256>(planes, k_real, spec, out, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace lgx
