// Resident batched Lenia engine: each world (C = 1, K = 1, N x N torus,
// N in {32, 64, 128}) lives in the registers of an (N/2)*G-thread slice of a
// 512-thread CTA for all of its steps.  Per Euler step and world:
//
//   row pass     : rows (2r, 2r+1) packed as one complex row, N-point FFT,
//                  written to the shared spectrum buffer (packed layout)
//   column pass  : column pairs (c, N-c) unpacked to the half spectrum column
//                  c, N-point FFT, x prepared spectrum, inverse FFT, written
//                  back in place; columns 0 and N/2 travel packed together
//   row inverse  : rows re-packed as (row 2r) + i (row 2r+1), inverse FFT ->
//                  potential, growth, weighted field, Euler update in registers,
//                  raw statistics moments reduced with warp shuffles
//
// This is leniax core.update (core.py:13-49) with get_potential_fft
// (core.py:52-102), get_field (core.py:163-199) and get_state (core.py:245-319)
// iterated as in runner._scan_fn (runner.py:295-334); the statistics moments
// follow statistics.py:36-126 on the world rolled by the carried shift.
#include "common.cuh"
#include "engine.h"
#include "fft.cuh"

namespace lgx {

namespace {

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
};

template <int G>
__device__ __forceinline__ int swz(int r) {
  return G == 8 ? (((r >> 1) & 7) << 1) : 0;
}

template <int N, int G>
__global__ void __launch_bounds__(512, 1) resident_kernel(ResidentArgs a) {
  using CF = RCfg<N, G>;
  using GE = typename CF::GE;
  constexpr int P = CF::P, Q = CF::Q, NT = CF::NT, WPC = CF::WPC, NW = CF::NW;
  constexpr int PITCH = CF::PITCH, KP = CF::KP;
  constexpr int RAWS = raw_stride(1);

  extern __shared__ __align__(16) float2 sm[];
  float2* tw_std = sm;
  float2* tw_colf = tw_std + N;
  float2* tw_rowi = tw_colf + N;
  const int sub = threadIdx.x / NT;
  const int tid = threadIdx.x - sub * NT;
  float2* buf = tw_rowi + N + sub * (CF::BUF + CF::CSCR + CF::KPS);
  float2* cscr = buf + CF::BUF;
  float2* kp = cscr + CF::CSCR;
  float* part = reinterpret_cast<float*>(tw_rowi + N + WPC * (CF::BUF + CF::CSCR + CF::KPS)) + sub * CF::PART;
  int* shv = reinterpret_cast<int*>(part + NW * 16);

  const int grp = tid / G, t = tid % G;
  const int lane = threadIdx.x & 31, wid = tid >> 5;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int bar_id = 1 + sub;

  init_twiddles<GE>(tw_std, tw_colf, tw_rowi, threadIdx.x, blockDim.x);
  __syncthreads();

  auto slot = [&](int r, int k) { return r * PITCH + (k ^ swz<G>(r)); };

  int loaded_sol = -1;
  const int n_items = (a.n_worlds + WPC - 1) / WPC;
  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int world = item * WPC + sub;
    if (world >= a.n_worlds) continue;  // idle slice: uses only its own named barrier
    const int sol = world / a.n_init, init = world - sol * a.n_init;
    if (sol != loaded_sol) {
      const float4* src = reinterpret_cast<const float4*>(a.kp + (size_t)sol * CF::KPS);
      float4* dst = reinterpret_cast<float4*>(kp);
      for (int i = tid; i < CF::KPS / 2; i += NT) dst[i] = __ldg(src + i);
      loaded_sol = sol;
    }
    const float gm = __ldg(a.gf + 2 * sol), gs = __ldg(a.gf + 2 * sol + 1);
    const float wk = __ldg(a.w + sol);
    const float fscale = a.mean ? 1.f / wk : 1.f;  // weighted_mean divides by sum_k w (core.py:240)
    const float dt = 1.f / __ldg(a.T + sol);
    const int gfid = a.gf_id, sfid = a.state_fn;

    const float* c0 = a.cells0 + (size_t)world * N * N;
    float2 z[P];
#pragma unroll
    for (int n2 = 0; n2 < P; ++n2)
      z[n2] = make_float2(__ldg(c0 + (2 * grp) * N + t + G * n2), __ldg(c0 + (2 * grp + 1) * N + t + G * n2));
    if (tid == 0) {
      shv[0] = 0;
      shv[1] = 0;
    }
    named_bar(bar_id, NT);

    for (int step = 0; step < a.steps; ++step) {
      // ------------------------------------------------------- row forward
      {
        float2 v[P];
        float2 u[Q][G];
#pragma unroll
        for (int i = 0; i < P; ++i) v[i] = z[i];
        float2* rs = buf + grp * PITCH;
        fft_standard<GE, false, false>(v, u, rs, tw_std, t, gmask);
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
          for (int k1 = 0; k1 < G; ++k1) buf[slot(grp, t + G * q + P * k1)] = u[q][k1];
      }
      named_bar(bar_id, NT);
      // ------------------------------------------------------- column pass
      {
        const int c = grp;  // column pair (c, N-c); c == 0 carries (0, N/2)
        float2 v[Q][G];
#pragma unroll
        for (int jp = 0; jp < Q / 2; ++jp) {
          const int m = t + G * jp;
#pragma unroll
          for (int n2 = 0; n2 < G; ++n2) {
            const int r = m + (P / 2) * n2;
            float2 z1, z2;
            if (c != 0) {
              z1 = buf[slot(r, c)];
              z2 = buf[slot(r, N - c)];
              v[2 * jp][n2] = make_float2(z1.x + z2.x, z1.y - z2.y);      // 2*X[2r][c]
              v[2 * jp + 1][n2] = make_float2(z1.y + z2.y, z2.x - z1.x);  // 2*X[2r+1][c]
            } else {
              z1 = buf[slot(r, 0)];
              z2 = buf[slot(r, N / 2)];
              v[2 * jp][n2] = make_float2(z1.x, z2.x);  // X[2r][0] + i X[2r][N/2]
              v[2 * jp + 1][n2] = make_float2(z1.y, z2.y);
            }
          }
        }
        float2 w[P];
        float2* cs = cscr + c * GE::SCR;
        fft_mirrored<GE, false, false>(v, w, cs, tw_colf, t, gmask);  // w[k1] = spectrum at ky = t + G*k1
        if (c != 0) {
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) w[k1] = cmul(w[k1], kp[(t + G * k1) * KP + c]);
        } else {
          // packed DC/Nyquist column: Q = C*A + conj(C[-ky])*B, mirror lane (G-t)%G
          float2 mir[P];
          const int src_lane = (lane & ~(G - 1)) | ((G - t) & (G - 1));
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) {
            float2 val = (t != 0) ? w[P - 1 - k1] : w[(P - k1) & (P - 1)];
            mir[k1].x = __shfl_sync(gmask, val.x, src_lane);
            mir[k1].y = __shfl_sync(gmask, val.y, src_lane);
          }
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) {
            const int ky = t + G * k1;
            float2 A = kp[ky * KP], B = kp[ky * KP + N / 2];
            float2 r1 = cmul(w[k1], A);
            float2 r2 = cmul(conjf2(mir[k1]), B);
            w[k1] = cadd(r1, r2);
          }
        }
        float2 u[Q][G];
        fft_standard<GE, true, true>(w, u, cs, tw_std, t, gmask);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int m = t + G * (q >> 1);
#pragma unroll
          for (int k1 = 0; k1 < G; ++k1) {
            const int r = m + (P / 2) * k1;
            const int col = (c != 0) ? ((q & 1) ? N - c : c) : ((q & 1) ? N / 2 : 0);
            buf[slot(r, col)] = u[q][k1];
          }
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
#pragma unroll
            for (int n2 = 0; n2 < G; ++n2) {
              const int k = m + P * n2, kk = N - k;
              float2 zk, zkk;
              if (n2 < G / 2) {
                float2 s1 = buf[slot(r, k)], s2 = buf[slot(r, kk)];
                zk = make_float2(s1.x - s2.y, s1.y + s2.x);
                zkk = make_float2(s1.x + s2.y, s2.x - s1.y);
              } else {
                float2 s1 = buf[slot(r, kk)], s2 = buf[slot(r, k)];
                zkk = make_float2(s1.x - s2.y, s1.y + s2.x);
                zk = make_float2(s1.x + s2.y, s2.x - s1.y);
              }
              v[2 * jp][n2] = zk;
              v[2 * jp + 1][G - 1 - n2] = zkk;
            }
          } else {
            float2 s0 = buf[slot(r, 0)], sn = buf[slot(r, N / 2)];
            v[2 * jp][0] = make_float2(s0.x, sn.x);
            v[2 * jp][G / 2] = make_float2(s0.y, sn.y);
#pragma unroll
            for (int n2 = 1; n2 < G / 2; ++n2) {
              const int k = P * n2, kk = N - k;
              float2 s1 = buf[slot(r, k)], s2 = buf[slot(r, kk)];
              v[2 * jp][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
              v[2 * jp][G - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
            }
#pragma unroll
            for (int n2 = 0; n2 < G / 2; ++n2) {
              const int k = P / 2 + P * n2, kk = N - k;
              float2 s1 = buf[slot(r, k)], s2 = buf[slot(r, kk)];
              v[2 * jp + 1][n2] = make_float2(s1.x - s2.y, s1.y + s2.x);
              v[2 * jp + 1][G - 1 - n2] = make_float2(s1.x + s2.y, s2.x - s1.y);
            }
          }
        }
        __syncwarp(gmask);
        float2 w[P];
        fft_mirrored<GE, true, true>(v, w, buf + r * PITCH, tw_rowi, t, gmask);  // w[k1]: x = t + G*k1

        const int sy = shv[0], sx = shv[1];
        const float cya = (float)(((2 * r - sy) & (N - 1)) - N / 2);
        const float cyb = (float)(((2 * r + 1 - sy) & (N - 1)) - N / 2);
        float Sa = 0.f, Sb = 0.f, Ga = 0.f, Gb = 0.f, mxx = 0.f, mx2x = 0.f, gxx = 0.f;
        float cpot = 0.f, cmass = 0.f, cgrow = 0.f;
        bool border = false;
        const size_t tbase = ((size_t)step * a.n_worlds + world) * (size_t)(N * N);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          const int x = t + G * k1;
          const float pa = w[k1].x, pb = w[k1].y;
          const float sa = z[k1].x, sb = z[k1].y;
          const float fa = (wk * growth_fn(gfid, pa, gm, gs)) * fscale;
          const float fb = (wk * growth_fn(gfid, pb, gm, gs)) * fscale;
          z[k1] = make_float2(state_fn(sfid, sa, fa, dt), state_fn(sfid, sb, fb, dt));
          // statistics moments of the pre-update cells (statistics.py:64-100)
          const float fpa = fmaxf(fa, 0.f), fpb = fmaxf(fb, 0.f);
          const float cx = (float)(((x - sx) & (N - 1)) - N / 2);
          Sa += sa;
          Sb += sb;
          Ga += fpa;
          Gb += fpb;
          const float ss = sa + sb, gg = fpa + fpb;
          mxx = fmaf(ss, cx, mxx);
          mx2x = fmaf(ss * cx, cx, mx2x);
          gxx = fmaf(gg, cx, gxx);
          cpot += (pa > kEps ? 1.f : 0.f) + (pb > kEps ? 1.f : 0.f);
          cmass += (sa > kEps ? 1.f : 0.f) + (sb > kEps ? 1.f : 0.f);
          cgrow += (fpa > kEps ? 1.f : 0.f) + (fpb > kEps ? 1.f : 0.f);
          // live cell on the outer layer of the un-centred torus (box stop set)
          const bool la = sa > kEps, lb = sb > kEps;
          if (x == 0 || x == N - 1) border |= la || lb;
          if (r == 0) border |= la;
          if (r == N / 2 - 1) border |= lb;
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
        float acc[12];
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
        acc[11] = border ? 1.f : 0.f;
#pragma unroll
        for (int i = 0; i < 11; ++i) acc[i] = warp_sum(acc[i]);
        acc[11] = __any_sync(0xffffffffu, border) ? 1.f : 0.f;
        if (lane == 0) {
#pragma unroll
          for (int i = 0; i < 12; ++i) part[wid * 16 + i] = acc[i];
        }
      }
      named_bar(bar_id, NT);
      // --------------------------------------------- per-step finalisation
      if (wid == 0) {
        const int sy = shv[0], sx = shv[1];  // shift that centred this step
        float v = 0.f;
        if (lane < 12) {
          for (int w = 0; w < NW; ++w) v += part[w * 16 + lane];
        }
        const float m00 = __shfl_sync(0xffffffffu, v, 0);
        const float mxy = __shfl_sync(0xffffffffu, v, 5);
        const float mxx = __shfl_sync(0xffffffffu, v, 6);
        float* rw = a.raw + (((size_t)sol * a.steps + step) * a.n_init + init) * RAWS;
        // lane -> raw slot
        if (lane < 12) {
          const int slotmap[12] = {RAW_M00,    RAW_G00,    RAW_CNT_POT, RAW_CNT_MASS, RAW_CNT_GROW, RAW_MX + 0,
                                   RAW_MX + 1, RAW_GX + 0, RAW_GX + 1,  RAW_MX2 + 0,  RAW_MX2 + 1,  RAW_BORDER};
          rw[slotmap[lane]] = (lane == 11) ? (v > 0.f ? 1.f : 0.f) : v;
        } else if (lane == 12) {
          rw[RAW_CM] = m00;
        } else if (lane < 16) {
          const int zero_slots[3] = {RAW_MX + 2, RAW_GX + 2, RAW_MX2 + 2};
          rw[zero_slots[lane - 13]] = 0.f;
        } else if (lane < 19) {
          rw[RAW_SHIFT + lane - 16] = (lane == 16) ? (float)sy : (lane == 17 ? (float)sx : 0.f);
        }
        __syncwarp();
        if (lane == 0) {
          const float cy = mxy / (m00 + kEps), cx = mxx / (m00 + kEps);
          shv[0] = pmod(sy + (int)cy, N);
          shv[1] = pmod(sx + (int)cx, N);
        }
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

template <int N, int G>
__global__ void prepare_resident_kernel(int n_sols, const float2* __restrict__ kh, float2* __restrict__ kp) {
  constexpr int KP = N / 2 + 2, HW = N / 2 + 1;
  const float scale = 1.f / (2.f * (float)N * (float)N);
  const long total = (long)n_sols * N * KP;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % KP);
    const long row = i / KP;  // s*N + ky
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

template <int N, int G>
cudaError_t launch_one(const ResidentArgs& a, int grid, cudaStream_t st) {
  using CF = RCfg<N, G>;
  cudaError_t e = cudaFuncSetAttribute(resident_kernel<N, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)CF::SMEM);
  if (e != cudaSuccess) return e;
  resident_kernel<N, G><<<grid, 512, CF::SMEM, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

bool resident_supported(const Model& m) {
  return m.nb_dims == 2 && m.C == 1 && m.K == 1 && m.H == m.W && (m.H == 32 || m.H == 64 || m.H == 128);
}

size_t resident_smem_bytes(int N) {
  switch (N) {
    case 32: return RCfg<32, 4>::SMEM;
    case 64: return RCfg<64, 4>::SMEM;
    case 128: return RCfg<128, 8>::SMEM;
  }
  return 0;
}

int resident_max_grid(int N) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  (void)N;
  return sms > 0 ? sms : 1;
}

cudaError_t launch_resident(int N, const ResidentArgs& a, int grid, cudaStream_t st) {
  switch (N) {
    case 32: return launch_one<32, 4>(a, grid, st);
    case 64: return launch_one<64, 4>(a, grid, st);
    case 128: return launch_one<128, 8>(a, grid, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_prepare_resident_spectrum(int N, int n_sols, const float2* k_half, float2* kp, cudaStream_t st) {
  const int threads = 256;
  const long total = (long)n_sols * N * (N / 2 + 2);
  const int blocks = (int)((total + threads - 1) / threads > 4096 ? 4096 : (total + threads - 1) / threads);
  switch (N) {
    case 32: prepare_resident_kernel<32, 4><<<blocks, threads, 0, st>>>(n_sols, k_half, kp); break;
    case 64: prepare_resident_kernel<64, 4><<<blocks, threads, 0, st>>>(n_sols, k_half, kp); break;
    case 128: prepare_resident_kernel<128, 8><<<blocks, threads, 0, st>>>(n_sols, k_half, kp); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace lgx
