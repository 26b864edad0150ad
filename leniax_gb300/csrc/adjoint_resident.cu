// Resident adjoint: the reverse steps of one checkpoint segment for C = K = 1
// worlds of 32^2, 64^2 or 128^2 in one persistent launch, each world's adjoint
// lambda kept in the registers of an (N/2)*G-thread slice for the whole
// segment (the resident engine's slices and shared-memory layout).
//
// Per reverse step t (core.py:13-49 differentiated; the same maths as the
// multi-kernel adjoint in adjoint.cu):
//   pointwise : mu = lambda * clip'(s + dt f), a = dt mu wf G'(u),
//               lambda <- mu (v1, simple) | mu (1 - dt) (v2); dL/dm, dL/ds,
//               dL/dw partial sums (s, u from the segment's recomputed states
//               and potentials)
//   rows      : FFT of the packed rows of a and of s into two shared buffers
//   columns   : per column pair, column FFTs of both; the kernel-gradient
//               spectrum 4 A conj(S) accumulated in the world's column-domain
//               accumulator (global, one owner thread per element); the
//               correlation A conj(K^) and its inverse column FFT
//   rows      : inverse row FFT -> K (*)^T a, added to lambda
// Two slice barriers per step.
#include <algorithm>

#include "resident.cuh"
#include "tma.cuh"

namespace lgx {

namespace {

template <int N, int G>
struct ACF {
  using GE = Geo<N, G>;
  static constexpr int P = GE::P, Q = GE::Q;
  static constexpr int NT = (N / 2) * G;  // threads per world
  static constexpr int WPC = 512 / NT;    // worlds per CTA
  static constexpr int NW = NT / 32;      // warps per world
  static constexpr int PITCH = N + G;
  static constexpr int KP = N / 2 + 2;
  static constexpr int BUF = (N / 2) * PITCH;
  static constexpr int CSCR = (N / 2) * GE::SCR;
  static constexpr int SLICE = 2 * BUF + CSCR;  // float2: a rows, s rows, column scratch
  static constexpr int PART = NW * 4;            // floats: per-warp parameter partials
  static constexpr size_t SMEM =
      (size_t)3 * N * sizeof(float2) + (size_t)WPC * ((size_t)SLICE * sizeof(float2) + PART * sizeof(float));
  static_assert(G != 8 || P == 16, "swizzled layout assumes N = 128 for G = 8");
};

// growth value and its derivatives d/du, d/dm, d/ds (growth_functions.py);
// GF selects a compile-time family (GF_FAST_GAUSSIAN: gaussian, GF_FAST_POLY4:
// poly_quad4, GF_GENERIC: any id) so the unrolled per-cell code stays small
template <int GF>
__device__ __forceinline__ void growth_grads(int id, float u, float m, float s, float& g, float& gu, float& gm,
                                             float& gs) {
  if constexpr (GF == GF_FAST_GAUSSIAN) id = LGX_GF_GAUSSIAN;
  if constexpr (GF == GF_FAST_POLY4) id = LGX_GF_POLY_QUAD4;
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

// ---- shared-memory passes of the resident layout (packed rows, column pairs,
// low-bit XOR swizzle for G == 8); the same addressing as resident_item.
template <int N, int G>
__device__ __forceinline__ void rows_store(float2* rowbuf, int s_row, int t, float2 (&u)[Geo<N, G>::Q][G]) {
  constexpr int P = Geo<N, G>::P, Q = Geo<N, G>::Q;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    float2* base = rowbuf + (G == 8 ? ((t + G * q) ^ s_row) : (t + G * q));
#pragma unroll
    for (int k1 = 0; k1 < G; ++k1) base[P * k1] = u[q][k1];
  }
}

template <int N, int G>
__device__ __forceinline__ void cols_load(const float2* buf, int c, int t, float2 (&v)[Geo<N, G>::Q][G]) {
  constexpr int P = Geo<N, G>::P, Q = Geo<N, G>::Q, PITCH = N + G;
  const int c1 = c != 0 ? c : 0, c2 = c != 0 ? N - c : N / 2;
#pragma unroll
  for (int jp = 0; jp < Q / 2; ++jp) {
    const int m = t + G * jp;
    int a1e, a2e, a1o, a2o;
    if constexpr (G == 8) {
      a1e = m * PITCH + (c1 ^ (m & 6));
      a2e = m * PITCH + (c2 ^ (m & 6));
      a1o = m * PITCH + (c1 ^ ((m & 6) | 8));
      a2o = m * PITCH + (c2 ^ ((m & 6) | 8));
    } else {
      a1e = a1o = m * PITCH + c1;
      a2e = a2o = m * PITCH + c2;
    }
#pragma unroll
    for (int n2 = 0; n2 < G; ++n2) {
      const int off = (P / 2) * n2 * PITCH;
      const float2 z1 = buf[((n2 & 1) ? a1o : a1e) + off];
      const float2 z2 = buf[((n2 & 1) ? a2o : a2e) + off];
      if (c != 0) {
        v[2 * jp][n2] = caddc(z1, z2);
        const float2 d = csubc(z1, z2);
        v[2 * jp + 1][n2] = make_float2(d.y, -d.x);
      } else {
        v[2 * jp][n2] = make_float2(z1.x, z2.x);
        v[2 * jp + 1][n2] = make_float2(z1.y, z2.y);
      }
    }
  }
}

template <int N, int G>
__device__ __forceinline__ void cols_store(float2* buf, int c, int t, float2 (&u)[Geo<N, G>::Q][G]) {
  constexpr int P = Geo<N, G>::P, Q = Geo<N, G>::Q, PITCH = N + G;
  const int c1 = c != 0 ? c : 0, c2 = c != 0 ? N - c : N / 2;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int m = t + G * (q >> 1);
    const int col = (q & 1) ? c2 : c1;
    int ae, ao;
    if constexpr (G == 8) {
      ae = m * PITCH + (col ^ (m & 6));
      ao = m * PITCH + (col ^ ((m & 6) | 8));
    } else {
      ae = ao = m * PITCH + col;
    }
#pragma unroll
    for (int k1 = 0; k1 < G; ++k1) buf[((k1 & 1) ? ao : ae) + (P / 2) * k1 * PITCH] = u[q][k1];
  }
}

template <int N, int G>
__device__ __forceinline__ void rows_load(const float2* rowbuf, int s_row, int t, float2 (&v)[Geo<N, G>::Q][G]) {
  constexpr int P = Geo<N, G>::P, Q = Geo<N, G>::Q;
#pragma unroll
  for (int jp = 0; jp < Q / 2; ++jp) {
    const int m = t + G * jp;
    if (m != 0) {
      int lo1, lo2;
      if constexpr (G == 8) {
        lo1 = m ^ s_row;
        lo2 = (16 - m) ^ s_row;
      } else {
        lo1 = m;
        lo2 = P - m;
      }
#pragma unroll
      for (int n2 = 0; n2 < G; ++n2) {
        const float2* p1 = rowbuf + lo1 + P * n2;
        const float2* p2 = rowbuf + lo2 + (N - P - P * n2);
        float2 zk, zkk;
        if (n2 < G / 2) {
          const float2 s1 = *p1, s2 = *p2;
          zk = make_float2(s1.x - s2.y, s1.y + s2.x);
          zkk = make_float2(s1.x + s2.y, s2.x - s1.y);
        } else {
          const float2 s1 = *p2, s2 = *p1;
          zkk = make_float2(s1.x - s2.y, s1.y + s2.x);
          zk = make_float2(s1.x + s2.y, s2.x - s1.y);
        }
        v[2 * jp][n2] = zk;
        v[2 * jp + 1][G - 1 - n2] = zkk;
      }
    } else {
      auto sl = [&](int k) -> float2 {
        return G == 8 ? rowbuf[(k & ~15) + ((k & 15) ^ s_row)] : rowbuf[k];
      };
      const float2 s0 = sl(0), sn = sl(N / 2);
      v[2 * jp][0] = make_float2(s0.x, sn.x);
      v[2 * jp][G / 2] = make_float2(s0.y, sn.y);
#pragma unroll
      for (int n2 = 1; n2 < G / 2; ++n2) {
        const int k = P * n2, kk = N - k;
        const float2 s1 = sl(k), s2 = sl(kk);
        v[2 * jp][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
        v[2 * jp][G - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
      }
#pragma unroll
      for (int n2 = 0; n2 < G / 2; ++n2) {
        const int k = P / 2 + P * n2, kk = N - k;
        const float2 s1 = sl(k), s2 = sl(kk);
        v[2 * jp + 1][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
        v[2 * jp + 1][G - 1 - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
      }
    }
  }
}

template <int N, int G, int GF>
__global__ void __launch_bounds__(512, 1) adjoint_resident_kernel(AdjResArgs a) {
  using CF = ACF<N, G>;
  using GE = typename CF::GE;
  constexpr int P = CF::P, Q = CF::Q, NT = CF::NT, WPC = CF::WPC, NW = CF::NW, PITCH = CF::PITCH, KP = CF::KP;
  extern __shared__ __align__(16) float2 sm[];
  init_twiddles<GE>(sm, sm + N, sm + 2 * N, threadIdx.x, blockDim.x);
  __syncthreads();
  const float2 *tw_std = sm, *tw_colf = sm + N, *tw_rowi = sm + 2 * N;
  const int sub = threadIdx.x / NT, tid = threadIdx.x - sub * NT;
  float2* bufa = sm + 3 * N + sub * CF::SLICE;
  float2* bufs = bufa + CF::BUF;
  float2* cscr = bufs + CF::BUF;
  float* part = reinterpret_cast<float*>(sm + 3 * N + WPC * CF::SLICE) + sub * CF::PART;
  const int grp = tid / G, t = tid % G, lane = threadIdx.x & 31, wid = tid >> 5;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int bar_id = 1 + sub;
  const int s_row = swz<G>(grp);
  float2* const rowa = bufa + grp * PITCH;
  float2* const rows = bufs + grp * PITCH;
  float2* const cs = cscr + grp * GE::SCR;
  const int c = grp;  // column pair (c, N-c) of the column pass; c == 0 carries (0, N/2)
  const int n_items = (a.n_worlds + WPC - 1) / WPC;

  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int world = item * WPC + sub;
    if (world >= a.n_worlds) continue;  // idle slice: only its own named barrier is involved
    const int sol = world / a.n_init;
    const float m = __ldg(a.gf + 2 * sol), sg = __ldg(a.gf + 2 * sol + 1);
    const float wk = __ldg(a.w + sol), dt = 1.f / __ldg(a.T + sol);
    const float wf = a.mean ? wk / wk : wk;
    const size_t plane = (size_t)N * N;
    const float* lin = a.lambda_in + world * plane + (size_t)(2 * grp) * N;
    float2 lam[P];
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) lam[k1] = make_float2(lin[t + G * k1], lin[N + t + G * k1]);
    float am = 0.f, as = 0.f, aw = 0.f;
    const float2* kk = a.kp + (size_t)sol * N * KP;
    float2* gk = a.gk + ((size_t)world * (N / 2) + c) * N;
    for (int st = a.steps - 1; st >= 0; --st) {
      // L2 prefetch of the previous step's trajectory planes (cells, potential), 16 KB pieces
      constexpr int kPieces = (int)((size_t)N * N * sizeof(float) / 16384);
      if constexpr (kPieces > 0) {
        if (st > 0 && tid < 2 * kPieces) {
          const float* base =
              (tid < kPieces ? a.traj_cells : a.traj_pot) + ((size_t)(st - 1) * a.n_worlds + world) * plane;
          prefetch_l2(base + (size_t)(tid % kPieces) * 4096, 16384);
        }
      }
      // ---------------------------------------------------------- pointwise + row FFTs of a and s
      {
        const size_t off = ((size_t)st * a.n_worlds + world) * plane + (size_t)(2 * grp) * N;
        const float* sp = a.traj_cells + off;
        const float* up = a.traj_pot + off;
        // state after this step: the next trajectory entry, or the segment's result
        const float* snp = st + 1 < a.steps ? sp + (size_t)a.n_worlds * plane
                                            : (a.cells_after ? a.cells_after + world * plane + (size_t)(2 * grp) * N
                                                             : nullptr);
        float2 za[P], zs[P];
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          const int x = t + G * k1;
          float ae[2], se[2], le[2];
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const float sv = __ldg(sp + e * N + x), u = __ldg(up + e * N + x);
            const float lamv = e == 0 ? lam[k1].x : lam[k1].y;
            float g, gu, gm, gs;
            growth_grads<GF>(a.gf_id, u, m, sg, g, gu, gm, gs);
            float mu = lamv;
            if (a.state_fn == LGX_STATE_V1 && a.clip_mask) {
              // the forward's clip was inactive where its output lies strictly inside (0, 1)
              const float nn = snp ? __ldg(snp + e * N + x) : sv + dt * (g * wf);
              mu = (nn > 0.f && nn < 1.f) ? lamv : 0.f;
            }
            le[e] = a.state_fn == LGX_STATE_V2 ? mu * (1.f - dt) : mu;
            const float dfl = dt * mu;
            ae[e] = dfl * wf * gu;
            se[e] = sv;
            am += dfl * wf * gm;
            as += dfl * wf * gs;
            aw += a.mean ? 0.f : dfl * g;
          }
          lam[k1] = make_float2(le[0], le[1]);
          za[k1] = make_float2(ae[0], ae[1]);
          zs[k1] = make_float2(se[0], se[1]);
        }
        float2 u[Q][G];
        fft_standard<GE, false, false>(za, u, rowa, tw_std, t, gmask);
        rows_store<N, G>(rowa, s_row, t, u);
        fft_standard<GE, false, false>(zs, u, rows, tw_std, t, gmask);
        rows_store<N, G>(rows, s_row, t, u);
      }
      named_bar(bar_id, NT);
      // ---------------------------------------------------------- column pass
      {
        float2 v[Q][G];
        float2 ws[P], wa[P];
        cols_load<N, G>(bufs, c, t, v);
        fft_mirrored<GE, false, false>(v, ws, cs, tw_colf, t, gmask);  // ky = t + G*k1
        cols_load<N, G>(bufa, c, t, v);
        fft_mirrored<GE, false, false>(v, wa, cs, tw_colf, t, gmask);
        if (c != 0) {
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) {
            const int ky = t + G * k1;
            gk[ky] = cadd(gk[ky], cmulc(wa[k1], ws[k1]));  // 4 A conj(S)
            wa[k1] = cmulc(wa[k1], __ldg(kk + ky * KP + c));
          }
        } else {
          // DC / Nyquist columns of a and s unpacked through their ky mirrors
          float2 ma[P];
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) cs[t + G * k1] = wa[k1];
          __syncwarp(gmask);
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
            const float2 a0 = make_float2(0.5f * (wa[k1].x + ma[k1].x), 0.5f * (wa[k1].y - ma[k1].y));
            const float2 aN = make_float2(0.5f * (wa[k1].y + ma[k1].y), 0.5f * (ma[k1].x - wa[k1].x));
            const float2 s0 = make_float2(0.5f * (ws[k1].x + msv.x), 0.5f * (ws[k1].y - msv.y));
            const float2 sN = make_float2(0.5f * (ws[k1].y + msv.y), 0.5f * (msv.x - ws[k1].x));
            const float2 g0 = cmulc(a0, s0), gN = cmulc(aN, sN);
            gk[ky] = cadd(gk[ky], make_float2(g0.x - gN.y, g0.y + gN.x));  // g0 + i gN
            const float2 A = __ldg(kk + ky * KP), B = __ldg(kk + ky * KP + N / 2);
            wa[k1] = cadd(cmulc(wa[k1], A), cmulc(conjf2(ma[k1]), B));  // C conj(A) + conj(C-) conj(B)
          }
          __syncwarp(gmask);
        }
        float2 u[Q][G];
        fft_standard<GE, true, true>(wa, u, cs, tw_std, t, gmask);
        cols_store<N, G>(bufa, c, t, u);
      }
      named_bar(bar_id, NT);
      // ---------------------------------------------------------- row inverse: lambda += K (*)^T a
      {
        float2 v[Q][G];
        rows_load<N, G>(rowa, s_row, t, v);
        __syncwarp(gmask);
        float2 w[P];
        fft_mirrored<GE, true, true>(v, w, rowa, tw_rowi, t, gmask);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) lam[k1] = make_float2(lam[k1].x + w[k1].x, lam[k1].y + w[k1].y);
      }
      // no barrier: the next row pass of this group writes only its own rows
    }
    float* lout = a.lambda_out + world * plane + (size_t)(2 * grp) * N;
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      lout[t + G * k1] = lam[k1].x;
      lout[N + t + G * k1] = lam[k1].y;
    }
    am = warp_sum(am);
    as = warp_sum(as);
    aw = warp_sum(aw);
    if (lane == 0) {
      part[wid * 4 + 0] = am;
      part[wid * 4 + 1] = as;
      part[wid * 4 + 2] = aw;
    }
    named_bar(bar_id, NT);
    if (tid < 3) {
      float v = 0.f;
      for (int w = 0; w < NW; ++w) v += part[w * 4 + tid];
      a.pacc[(size_t)world * 3 + tid] += v;
    }
    named_bar(bar_id, NT);  // part and the buffers are free for the slice's next world
  }
}

template <int N, int G, int GF>
cudaError_t launch_gf(const AdjResArgs& a, cudaStream_t st) {
  using CF = ACF<N, G>;
  cudaError_t e = cudaFuncSetAttribute(adjoint_resident_kernel<N, G, GF>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF::SMEM);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int items = (a.n_worlds + CF::WPC - 1) / CF::WPC;
  const int grid = std::max(1, std::min(items, sms > 0 ? sms : 1));
  adjoint_resident_kernel<N, G, GF><<<grid, 512, CF::SMEM, st>>>(a);
  return cudaGetLastError();
}

template <int N, int G>
cudaError_t launch_n(const AdjResArgs& a, cudaStream_t st) {
  if (a.gf_id == LGX_GF_GAUSSIAN) return launch_gf<N, G, GF_FAST_GAUSSIAN>(a, st);
  if (a.gf_id == LGX_GF_POLY_QUAD4) return launch_gf<N, G, GF_FAST_POLY4>(a, st);
  return launch_gf<N, G, GF_GENERIC>(a, st);
}

}  // namespace

bool adjoint_resident_supported(const Model& m) { return resident_supported(m); }

cudaError_t launch_adjoint_resident(int N, const AdjResArgs& a, cudaStream_t st) {
  switch (N) {
    case 32: return launch_n<32, 4>(a, st);
    case 64: return launch_n<64, 4>(a, st);
    case 128: return launch_n<128, 8>(a, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace lgx
