// Resident-engine building blocks shared by the resident kernel and the
// uneven-batch kernel: slice geometry, growth specialisations and the per-item
// world processor.  See resident.cu for the algorithm.
#pragma once
#include "common.cuh"
#include "engine.h"
#include "fft.cuh"

namespace lgx {

template <int N, int G>
struct RCfg {
  using GE = Geo<N, G>;
  static constexpr int P = GE::P, Q = GE::Q;
  static constexpr int NT = (N / 2) * G;  // threads per world
  static constexpr int WPC = 512 / NT;    // worlds per CTA
  static constexpr int NW = NT / 32;      // warps per world
  static constexpr int PITCH = N + G;     // spectrum buffer row pitch (float2)
  static constexpr int KP = N / 2 + 2;    // prepared spectrum pitch (float2)
  static constexpr int BUF = (N / 2) * PITCH;
  static constexpr int CSCR = (N / 2) * GE::SCR;
  static constexpr int KPS = N * KP;
  static constexpr int PART = NW * 16 + 16;  // floats: per-warp partials + carried shift
  static constexpr size_t SMEM =
      (size_t)3 * N * sizeof(float2) + (size_t)WPC * ((size_t)(BUF + CSCR + KPS) * sizeof(float2) + PART * 4);
  static_assert(NT % 32 == 0 && 512 % NT == 0, "slice size");
  // The XOR swizzle of the spectrum buffer (G == 8) is applied to the low four
  // bits of the column index; the address helpers below rely on P == 16 then.
  static_assert(G != 8 || P == 16, "swizzled layout assumes N = 128 for G = 8");
};

// Low-bit swizzle of the spectrum buffer (bank-conflict-free row and column
// access for 64-bit elements; G = 4 layouts need none).
template <int G>
__device__ __forceinline__ int swz(int r) {
  return G == 8 ? (((r >> 1) & 7) << 1) : 0;
}

// One work item of the resident engine: WPC consecutive worlds, one per
// (N/2)*G-thread slice of the 512-thread CTA.  `tw` holds the three N-entry
// twiddle tables, `work` the slices' shared buffers (RCfg::SMEM - 3N float2).
// `loaded_sol` caches which solution's prepared spectrum each slice holds.
template <int N, int G, int GF, bool STATS = true>
__device__ __forceinline__ void resident_item(const ResidentArgs& a, int item, const float2* tw, float2* work,
                                              int& loaded_sol) {
  using CF = RCfg<N, G>;
  using GE = typename CF::GE;
  constexpr int P = CF::P, Q = CF::Q, NT = CF::NT, WPC = CF::WPC, NW = CF::NW;
  constexpr int PITCH = CF::PITCH, KP = CF::KP;
  constexpr int RAWS = raw_stride(1);

  const float2* tw_std = tw;
  const float2* tw_colf = tw_std + N;
  const float2* tw_rowi = tw_colf + N;
  const int sub = threadIdx.x / NT;
  const int tid = threadIdx.x - sub * NT;
  float2* buf = work + sub * (CF::BUF + CF::CSCR + CF::KPS);
  float2* cscr = buf + CF::BUF;
  float2* kp = cscr + CF::CSCR;
  float* part = reinterpret_cast<float*>(work + WPC * (CF::BUF + CF::CSCR + CF::KPS)) + sub * CF::PART;
  int* shv = reinterpret_cast<int*>(part + NW * 16);

  const int grp = tid / G, t = tid % G;
  const int lane = threadIdx.x & 31, wid = tid >> 5;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int bar_id = 1 + sub;

  // ---- per-thread address bases (see RCfg: the swizzle touches the low 4 bits)
  const int s_row = swz<G>(grp);  // row passes: this thread's packed row is grp
  float2* const rowbuf = buf + grp * PITCH;
  float2* const cs = cscr + grp * GE::SCR;  // column pass: this thread's column pair is grp

  {
    const int world = item * WPC + sub;
    if (world >= a.n_worlds) return;  // idle slice: uses only its own named barrier
    const int sol = world / a.n_init, init = world - sol * a.n_init;
    if (sol != loaded_sol) {
      const float4* src = reinterpret_cast<const float4*>(a.kp + (size_t)sol * CF::KPS);
      float4* dst = reinterpret_cast<float4*>(kp);
      for (int i = tid; i < CF::KPS / 2; i += NT) dst[i] = __ldg(src + i);
      loaded_sol = sol;
    }
    GrowthP gp;
    gp.m = __ldg(a.gf + 2 * sol);
    gp.s = __ldg(a.gf + 2 * sol + 1);
    gp.id = a.gf_id;
    if (GF == GF_FAST_GAUSSIAN) gp.a = 0.84932180028801904272f / gp.s;  // sqrt(log2(e)/2) / s
    else if (GF == GF_FAST_POLY4) gp.a = 1.f / (9.f * (gp.s * gp.s));
    else gp.a = 0.f;
    const float wk = __ldg(a.w + sol);
    // weighted_mean with one kernel: (w*g)/w (core.py:240); weighted_sum: w*g
    const float wf = a.mean ? wk / wk : wk;
    const float dt = 1.f / __ldg(a.T + sol);
    const int sfid = a.state_fn;

    const float* c0 = a.cells0 + (size_t)world * N * N;
    float2 z[P];
#pragma unroll
    for (int n2 = 0; n2 < P; ++n2)
      z[n2] = make_float2(__ldg(c0 + (2 * grp) * N + t + G * n2), __ldg(c0 + (2 * grp + 1) * N + t + G * n2));
    if (tid == 0) {
      shv[0] = a.shift_in ? __ldg(a.shift_in + 2 * world) : 0;
      shv[1] = a.shift_in ? __ldg(a.shift_in + 2 * world + 1) : 0;
    }
    named_bar(bar_id, NT);

    // reduce step `st`'s per-warp moments, record them, advance the shift
    auto finalize = [&](int st) {
      const int sy = shv[0], sx = shv[1];  // shift that centred step st
      float v = 0.f;
      if (lane < 12) {
        for (int w = 0; w < NW; ++w) v += part[w * 16 + lane];
      }
      const float m00 = __shfl_sync(0xffffffffu, v, 0);
      const float mxy = __shfl_sync(0xffffffffu, v, 5);
      const float mxx = __shfl_sync(0xffffffffu, v, 6);
      float* rw = a.raw + (((size_t)sol * a.steps + st) * a.n_init + init) * RAWS;
      // lanes 0..11 -> M00, G00, CNT_POT, CNT_MASS, CNT_GROW, MX0, MX1, GX0, GX1, MX2_0, MX2_1, BORDER
      if (lane < 12) {
        const int slot = lane < 7 ? lane : (lane < 9 ? lane + 1 : (lane < 11 ? lane + 2 : RAW_BORDER));
        rw[slot] = (lane == 11) ? (v > 0.f ? 1.f : 0.f) : v;
      } else if (lane == 12) {
        rw[RAW_CM] = m00;
      } else if (lane < 16) {
        rw[RAW_MX + 2 + 3 * (lane - 13)] = 0.f;  // third-axis slots of MX, GX, MX2
      } else if (lane < 19) {
        rw[RAW_SHIFT + lane - 16] = (lane == 16) ? (float)sy : (lane == 17 ? (float)sx : 0.f);
      }
      __syncwarp();
      if (lane == 0) {
        const float cy = mxy / (m00 + kEps), cx = mxx / (m00 + kEps);
        shv[0] = pmod(sy + (int)cy, N);
        shv[1] = pmod(sx + (int)cx, N);
      }
    };

    for (int step = 0; step < a.steps; ++step) {
      // ------------------------------------------------------- row forward
      {
        float2 v[P];
        float2 u[Q][G];
#pragma unroll
        for (int i = 0; i < P; ++i) v[i] = z[i];
        fft_standard<GE, false, false>(v, u, rowbuf, tw_std, t, gmask);
        // X[k] for k = t + G*q + P*k1: the low four bits carry the swizzle
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          if constexpr (G == 8) {
            float2* base = rowbuf + ((t + G * q) ^ s_row);
#pragma unroll
            for (int k1 = 0; k1 < G; ++k1) base[P * k1] = u[q][k1];
          } else {
            float2* base = rowbuf + t + G * q;
#pragma unroll
            for (int k1 = 0; k1 < G; ++k1) base[P * k1] = u[q][k1];
          }
        }
      }
      named_bar(bar_id, NT);
      if (STATS && step > 0 && wid == NW - 1) finalize(step - 1);
      // ------------------------------------------------------- column pass
      {
        const int c = grp;  // column pair (c, N-c); c == 0 carries (0, N/2)
        const int c1 = c != 0 ? c : 0, c2 = c != 0 ? N - c : N / 2;
        float2 v[Q][G];
#pragma unroll
        for (int jp = 0; jp < Q / 2; ++jp) {
          const int m = t + G * jp;
          // rows r = m + (P/2)*n2; for G == 8 (m < 8): swz(r) = (m & 6) | 8*(n2 & 1)
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
              v[2 * jp][n2] = caddc(z1, z2);  // 2*X[2r][c]
              const float2 d = csubc(z1, z2);  // 2i*X[2r+1][c]
              v[2 * jp + 1][n2] = make_float2(d.y, -d.x);
            } else {
              v[2 * jp][n2] = make_float2(z1.x, z2.x);  // X[2r][0] + i X[2r][N/2]
              v[2 * jp + 1][n2] = make_float2(z1.y, z2.y);
            }
          }
        }
        float2 w[P];
        fft_mirrored<GE, false, false>(v, w, cs, tw_colf, t, gmask);  // w[k1] = spectrum at ky = t + G*k1
        if (c != 0) {
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) w[k1] = cmul(w[k1], kp[(t + G * k1) * KP + c]);
        } else {
          // packed DC/Nyquist column: Q[ky] = C[ky]*A[ky] + conj(C[-ky])*B[ky];
          // the mirror C[-ky] is read back through the group's scratch
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) cs[t + G * k1] = w[k1];
          __syncwarp(gmask);
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) {
            const int ky = t + G * k1;
            const float2 mir = cs[(N - ky) & (N - 1)];
            const float2 A = kp[ky * KP], B = kp[ky * KP + N / 2];
            w[k1] = cadd(cmul(w[k1], A), cmul(conjf2(mir), B));
          }
          __syncwarp(gmask);
        }
        float2 u[Q][G];
        fft_standard<GE, true, true>(w, u, cs, tw_std, t, gmask);
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
      named_bar(bar_id, NT);
      // ---------------------------------------- row inverse, growth, update
      {
        const int r = grp;
        float2 v[Q][G];
#pragma unroll
        for (int jp = 0; jp < Q / 2; ++jp) {
          const int m = t + G * jp;
          if (m != 0) {
            // k = m + P*n2 and N - k; low-bit swizzle split as in the row pass
            int lo1, lo2;
            if constexpr (G == 8) {
              lo1 = m ^ s_row;         // (m + 16 n2) ^ s = (m ^ s) + 16 n2
              lo2 = (16 - m) ^ s_row;  // N - m - 16 n2 = (16 - m) + (N - 16 - 16 n2)
            } else {
              lo1 = m;
              lo2 = P - m;
            }
#pragma unroll
            for (int n2 = 0; n2 < G; ++n2) {
              const float2* p1 = rowbuf + lo1 + P * n2;            // slot(r, k)
              const float2* p2 = rowbuf + lo2 + (N - P - P * n2);  // slot(r, N - k)
              float2 zk, zkk;
              if (n2 < G / 2) {  // k < N/2: slot(r,k) = P[2r][k], slot(r,N-k) = P[2r+1][k]
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
            auto sl = [&](int k) -> float2 { return rowbuf[(k & ~15) + ((k & 15) ^ s_row)]; };
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
        __syncwarp(gmask);
        float2 w[P];
        fft_mirrored<GE, true, true>(v, w, rowbuf, tw_rowi, t, gmask);  // w[k1]: x = t + G*k1

        const int sy = shv[0], sx = shv[1];
        const float cya = (float)(((2 * r - sy) & (N - 1)) - N / 2);
        const float cyb = (float)(((2 * r + 1 - sy) & (N - 1)) - N / 2);
        const int xb = t - sx;
        float2 S2 = make_float2(0.f, 0.f), G2 = make_float2(0.f, 0.f);  // (row 2r, row 2r+1) sums
        float mxx = 0.f, mx2x = 0.f, gxx = 0.f;
        float cpot = 0.f, cmass = 0.f, cgrow = 0.f;
        bool liveA = false, liveB = false, liveX = false;
        const size_t tbase = ((size_t)step * a.n_worlds + world) * (size_t)(N * N);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          const int x = t + G * k1;
          const float pa = w[k1].x, pb = w[k1].y;
          const float2 s2 = z[k1];
          const float sa = s2.x, sb = s2.y;
          const float2 f2 = weighted_growth2<GF>(gp, w[k1], wf);
          const float fa = f2.x, fb = f2.y;
          if (sfid == LGX_STATE_V1) {
            z[k1] = make_float2(__saturatef(fmaf(dt, fa, sa)), __saturatef(fmaf(dt, fb, sb)));
          } else {
            z[k1] = make_float2(state_fn(sfid, sa, fa, dt), state_fn(sfid, sb, fb, dt));
          }
          if constexpr (STATS) {
            // statistics moments of the pre-update cells (statistics.py:64-100)
            const float fpa = fmaxf(fa, 0.f), fpb = fmaxf(fb, 0.f);
            const float cx = (float)(((xb + G * k1) & (N - 1)) - N / 2);
            S2 = __fadd2_rn(S2, s2);
            G2 = __fadd2_rn(G2, make_float2(fpa, fpb));
            const float ss = sa + sb, gg = fpa + fpb;
            mxx = fmaf(ss, cx, mxx);
            mx2x = fmaf(ss * cx, cx, mx2x);
            gxx = fmaf(gg, cx, gxx);
            cpot += (pa > kEps ? 1.f : 0.f) + (pb > kEps ? 1.f : 0.f);
            const bool la = sa > kEps, lb = sb > kEps;
            cmass += (la ? 1.f : 0.f) + (lb ? 1.f : 0.f);
            cgrow += (fpa > kEps ? 1.f : 0.f) + (fpb > kEps ? 1.f : 0.f);
            liveA |= la;
            liveB |= lb;
            if (k1 == 0 || k1 == P - 1) liveX |= (x == 0 || x == N - 1) && (la || lb);
          }
          if (a.traj_cells) {
            float* tc = a.traj_cells + tbase;
            tc[(2 * r) * N + x] = sa;
            tc[(2 * r + 1) * N + x] = sb;
          }
          if (a.traj_field) {
            float* tf = a.traj_field + tbase;
            tf[(2 * r) * N + x] = fa;
            tf[(2 * r + 1) * N + x] = fb;
          }
          if (a.traj_pot) {
            float* tp = a.traj_pot + tbase;
            tp[(2 * r) * N + x] = pa;
            tp[(2 * r + 1) * N + x] = pb;
          }
        }
        if constexpr (STATS) {
        // live cell on the outer layer of the un-centred torus (box stop set)
        const bool border = liveX || (r == 0 && liveA) || (r == N / 2 - 1 && liveB);
        const float Sa = S2.x, Sb = S2.y, Ga = G2.x, Gb = G2.y;
        float acc[16];
        acc[0] = Sa + Sb;
        acc[1] = Ga + Gb;
        acc[2] = cpot;
        acc[3] = cmass;
        acc[4] = cgrow;
        acc[5] = cya * Sa + cyb * Sb;
        acc[6] = mxx;
        acc[7] = cya * Ga + cyb * Gb;
        acc[8] = gxx;
        acc[9] = cya * cya * Sa + cyb * cyb * Sb;
        acc[10] = mx2x;
        acc[11] = border ? 1.f : 0.f;  // a count of border lanes; the finaliser tests > 0
#pragma unroll
        for (int i = 12; i < 16; ++i) acc[i] = 0.f;
        const float tot = warp_sum16(acc);  // lane L: total of value L >> 1
        if ((lane & 1) == 0 && lane < 24) part[wid * 16 + (lane >> 1)] = tot;
        }
      }
      // no barrier here: the next row pass of this group touches only its own
      // packed row, and the next step's first barrier orders these partials
    }
    named_bar(bar_id, NT);
    if (STATS && a.steps > 0 && wid == NW - 1) {
      finalize(a.steps - 1);
      if (a.shift_out && lane == 0) {  // the lane that advanced the shift
        a.shift_out[2 * world] = shv[0];
        a.shift_out[2 * world + 1] = shv[1];
      }
    }
    if (a.final_cells) {
      float* fc = a.final_cells + (size_t)world * N * N;
#pragma unroll
      for (int n2 = 0; n2 < P; ++n2) {
        fc[(2 * grp) * N + t + G * n2] = z[n2].x;
        fc[(2 * grp + 1) * N + t + G * n2] = z[n2].y;
      }
    }
    named_bar(bar_id, NT);
  }
}

// Shared-memory bytes one resident item needs after the twiddle tables.
template <int N, int G>
constexpr size_t resident_work_bytes() {
  using CF = RCfg<N, G>;
  return (size_t)CF::WPC * ((size_t)(CF::BUF + CF::CSCR + CF::KPS) * sizeof(float2) + CF::PART * 4);
}

}  // namespace lgx
