// Uneven batch engine: worlds of different sizes and dimensions, radii and
// growth parameters in one persistent launch fed by a device work queue.
//
// A 512-thread CTA per SM loops: it dequeues an item with an atomic counter
// and processes it with the code for its class:
//   * resident classes (2D 32^2, 64^2, 128^2): resident_item() -- 8, 4 or 1
//     worlds per CTA, states in registers, spectra in shared memory;
//   * big 2D (256^2): one world per CTA, packed-row spectrum in a per-CTA
//     global (L2-resident) scratch, the resident engine's FFT passes;
//   * big 3D (32^3, 64^3): one world per CTA, half spectrum [D][H][W/2+1] in
//     the per-CTA scratch; x, y and z passes, the spectrum multiply fused into
//     the z pass.  Lines of the y and z passes are transformed by groups of G
//     lanes (G = 4 or 2, chosen per batch by the autotuner).
// The host orders the queue (largest first by default) so long worlds start
// early.
//
// This replaces leniax's vmap over identically-shaped worlds
// (runner.py:167-168, experiments/readme.md:26-35) for heterogeneous batches;
// every world follows core.update (core.py:13-49) and compute_stats
// (statistics.py:36-126) as in the other engines.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "resident.cuh"
#include "tma.cuh"

namespace lgx {

namespace {

// twiddle tables of every size used here, 3 tables of N entries each
constexpr int TW32 = 0, TW64 = TW32 + 3 * 32, TW128 = TW64 + 3 * 64, TW256 = TW128 + 3 * 128,
              TW64G2 = TW256 + 3 * 256, TW32G2 = TW64G2 + 64, TW_END = TW32G2 + 32;

constexpr int kBigRed = 16 * 16 + 16;  // floats: per-warp partials + shift

template <int N, int G>
constexpr size_t big_smem() {
  return (size_t)(512 / G) * Geo<N, G>::SCR * sizeof(float2) + kBigRed * sizeof(float);
}

constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }

template <int N, int LG>
struct Big3D {
  static constexpr int G = 4;
  using GE = Geo<N, G>;
  using GZ = Geo<N, LG>;
  static constexpr int HW = N / 2 + 1;
  static constexpr int NT = (N / 2) * G;  // threads per plane slice
  static constexpr int SL = 512 / NT;     // planes in flight
  static constexpr int PITCH = N + G;
  static constexpr int BUF = (N / 2) * PITCH, CSCR = (N / 2) * GE::SCR;
  static constexpr int XS = N * HW;               // one half-spectrum plane, staged per slice (phase C)
  static constexpr int XSOFF = SL * (BUF + CSCR);
  static constexpr int PLANES = XSOFF + SL * XS;
  static constexpr int ZSCR = (512 / LG) * GZ::SCR;
  static constexpr int REGION = PLANES > ZSCR ? PLANES : ZSCR;  // float2, phases A/C and B share it
  static_assert(NT % 32 == 0 && 512 % NT == 0 && N % SL == 0, "plane slices");
};

constexpr int kBigBars = 8;  // mbarriers after the reduction area (one per plane slice)

template <int N, int LG>
constexpr size_t big3d_smem() {
  return (size_t)Big3D<N, LG>::REGION * sizeof(float2) + kBigRed * sizeof(float) + kBigBars * sizeof(uint64_t);
}

constexpr size_t kWorkBytes =
    cmax(cmax(cmax(resident_work_bytes<128, 8>(), resident_work_bytes<64, 4>()), resident_work_bytes<32, 4>()),
         cmax(big_smem<256, 8>(), cmax(cmax(big3d_smem<64, 4>(), big3d_smem<64, 2>()),
                                       cmax(big3d_smem<32, 4>(), big3d_smem<32, 2>()))));
constexpr size_t kMixedSmem = (size_t)TW_END * sizeof(float2) + kWorkBytes;
static_assert(kMixedSmem <= 227 * 1024, "mixed kernel shared memory");

template <int GF>
__device__ __forceinline__ GrowthP big_growth(const BigArgs& a, int sol) {
  GrowthP g;
  g.m = __ldg(a.gf + 2 * sol);
  g.s = __ldg(a.gf + 2 * sol + 1);
  g.id = a.gf_id;
  g.a = GF == GF_FAST_GAUSSIAN ? 0.84932180028801904272f / g.s : (GF == GF_FAST_POLY4 ? 1.f / (9.f * g.s * g.s) : 0.f);
  return g;
}

// acc layout == raw slots 0..13: M00, G00, CNT_POT, CNT_MASS, CNT_GROW,
// MX[3], GX[3], MX2[3] (axes outermost first).  Block reduction, record of the
// step's raw moments by warp 0 (lane i writes raw slot i), shift update.
__device__ __forceinline__ void big_finish_step(const BigArgs& a, int world, int step, int nd, const int (&sizes)[3],
                                                float (&acc)[14], bool border, float* red, int* shv) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 14; ++i) acc[i] = warp_sum(acc[i]);
  const bool anyb = __any_sync(0xffffffffu, border);
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 14; ++i) red[wid * 16 + i] = acc[i];
    red[wid * 16 + 14] = anyb ? 1.f : 0.f;
  }
  __syncthreads();
  if (wid == 0) {
    float v = 0.f;
    if (lane < 15)
      for (int w = 0; w < 16; ++w) v += red[w * 16 + lane];
    const int sh0 = shv[0], sh1 = shv[1], sh2 = shv[2];
    const float m00 = __shfl_sync(0xffffffffu, v, RAW_M00);
    const float mx0 = __shfl_sync(0xffffffffu, v, RAW_MX + 0);
    const float mx1 = __shfl_sync(0xffffffffu, v, RAW_MX + 1);
    const float mx2 = __shfl_sync(0xffffffffu, v, RAW_MX + 2);
    const int sol = world / a.n_init, init = world - sol * a.n_init;
    float* rw = a.raw + (((size_t)sol * a.steps + step) * a.n_init + init) * raw_stride(1);
    if (lane < RAW_BORDER) rw[lane] = v;
    else if (lane == RAW_BORDER) rw[lane] = v > 0.f ? 1.f : 0.f;
    else if (lane < RAW_CM) rw[lane] = (float)(lane == RAW_SHIFT ? sh0 : (lane == RAW_SHIFT + 1 ? sh1 : sh2));
    else if (lane == RAW_CM) rw[lane] = m00;
    __syncwarp();
    if (lane == 0) {
      const float den = m00 + kEps;
      shv[0] = pmod(sh0 + (int)(mx0 / den), sizes[0]);
      if (nd > 1) shv[1] = pmod(sh1 + (int)(mx1 / den), sizes[1]);
      if (nd > 2) shv[2] = pmod(sh2 + (int)(mx2 / den), sizes[2]);
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------ big 2D
// Euler rate of a big item's world (BigArgs::dt_mode).
__device__ __forceinline__ float big_dt(const BigArgs& a, int world, int sol) {
  return a.dt_mode == 1 ? __ldg(a.dt) : (a.dt_mode == 2 ? __ldg(a.dt + world) : 1.f / __ldg(a.T + sol));
}

template <int N, int GF>
__device__ __noinline__ void big2d_item(const BigArgs& a, int world, const float2* tw, float2* work) {
  constexpr int G = 8;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q, NG = 512 / G, KP = N / 2 + 2;
  const float2 *tw_std = tw, *tw_colf = tw + N, *tw_rowi = tw + 2 * N;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  float2* scr = work + grp * GE::SCR;
  float* red = reinterpret_cast<float*>(work + NG * GE::SCR);
  int* shv = reinterpret_cast<int*>(red + 16 * 16);
  float2* spec = a.scratch + (size_t)blockIdx.x * a.scratch_per_cta;  // [N/2][N]
  const int sol = world / a.n_init;
  const float2* kp = a.kp + (size_t)sol * N * KP;
  const float* c0 = a.cells0 + (size_t)world * N * N;
  float* st = a.state + (size_t)world * N * N;
  const GrowthP gq = big_growth<GF>(a, sol);
  const float wk = __ldg(a.w + sol), wf = a.mean ? wk / wk : wk;
  const float dt = big_dt(a, world, sol);
  const int sizes[3] = {N, N, 1};
  if (threadIdx.x == 0) shv[0] = shv[1] = shv[2] = 0;
  __syncthreads();
  for (int step = 0; step < a.steps; ++step) {
    const float* src = step == 0 ? c0 : st;
    for (int r = grp; r < N / 2; r += NG) {  // row pass
      float2 v[P];
#pragma unroll
      for (int n2 = 0; n2 < P; ++n2) v[n2] = make_float2(src[(2 * r) * N + t + G * n2], src[(2 * r + 1) * N + t + G * n2]);
      float2 u[Q][G];
      fft_standard<GE, false, false>(v, u, scr, tw_std, t, gmask);
#pragma unroll
      for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int k1 = 0; k1 < G; ++k1) spec[r * N + pa_pos<N>(t + G * q + P * k1)] = u[q][k1];
    }
    __syncthreads();
    for (int c = grp; c < N / 2; c += NG) {  // column pass
      float2 v[Q][G];
#pragma unroll
      for (int jp = 0; jp < Q / 2; ++jp) {
        const int m = t + G * jp;
#pragma unroll
        for (int n2 = 0; n2 < G; ++n2) {
          const int r = m + (P / 2) * n2;
          // pair c of packed row r: (slot c, slot N - c); pair 0: (slot 0, slot N/2)
          const float4 q = reinterpret_cast<const float4*>(spec + r * N)[c];
          const float2 z1 = make_float2(q.x, q.y), z2 = make_float2(q.z, q.w);
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
      float2 w[P];
      fft_mirrored<GE, false, false>(v, w, scr, tw_colf, t, gmask);
      if (c != 0) {
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) w[k1] = cmul(w[k1], __ldg(kp + (t + G * k1) * KP + c));
      } else {
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) scr[t + G * k1] = w[k1];
        __syncwarp(gmask);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          const int ky = t + G * k1;
          const float2 mir = scr[(N - ky) & (N - 1)];
          w[k1] = cadd(cmul(w[k1], __ldg(kp + ky * KP)), cmul(conjf2(mir), __ldg(kp + ky * KP + N / 2)));
        }
        __syncwarp(gmask);
      }
      float2 u[Q][G];
      fft_standard<GE, true, true>(w, u, scr, tw_std, t, gmask);
      // rows 2r and 2r+1 of column pair c -> pair c of packed row r
#pragma unroll
      for (int a = 0; a < Q / 2; ++a) {
        const int m = t + G * a;
#pragma unroll
        for (int k1 = 0; k1 < G; ++k1)
          reinterpret_cast<float4*>(spec + (m + (P / 2) * k1) * N)[c] =
              make_float4(u[2 * a][k1].x, u[2 * a][k1].y, u[2 * a + 1][k1].x, u[2 * a + 1][k1].y);
      }
    }
    __syncthreads();
    float acc[14];
#pragma unroll
    for (int i = 0; i < 14; ++i) acc[i] = 0.f;
    bool border = false;
    const int sy = shv[0], sx = shv[1];
    for (int r = grp; r < N / 2; r += NG) {  // row inverse, growth, update, moments
      float2 v[Q][G];
      unpack_row_pair_pa<GE>(spec + r * N, v, t);
      float2 w[P];
      fft_mirrored<GE, true, true>(v, w, scr, tw_rowi, t, gmask);
      const float cya = (float)(((2 * r - sy) & (N - 1)) - N / 2);
      const float cyb = (float)(((2 * r + 1 - sy) & (N - 1)) - N / 2);
      float Sa = 0.f, Sb = 0.f, Ga = 0.f, Gb = 0.f;
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) {
        const int x = t + G * k1;
        const float pa = w[k1].x, pb = w[k1].y;
        const float sa = src[(2 * r) * N + x], sb = src[(2 * r + 1) * N + x];
        const float fa = weighted_growth<GF>(gq, pa, wf), fb = weighted_growth<GF>(gq, pb, wf);
        st[(2 * r) * N + x] = state_fn(a.state_fn, sa, fa, dt);
        st[(2 * r + 1) * N + x] = state_fn(a.state_fn, sb, fb, dt);
        const float fpa = fmaxf(fa, 0.f), fpb = fmaxf(fb, 0.f);
        const float cx = (float)(((x - sx) & (N - 1)) - N / 2);
        Sa += sa;
        Sb += sb;
        Ga += fpa;
        Gb += fpb;
        const float ss = sa + sb, gg = fpa + fpb;
        acc[RAW_MX + 1] = fmaf(ss, cx, acc[RAW_MX + 1]);
        acc[RAW_GX + 1] = fmaf(gg, cx, acc[RAW_GX + 1]);
        acc[RAW_MX2 + 1] = fmaf(ss * cx, cx, acc[RAW_MX2 + 1]);
        acc[RAW_CNT_POT] += (pa > kEps ? 1.f : 0.f) + (pb > kEps ? 1.f : 0.f);
        const bool la = sa > kEps, lb = sb > kEps;
        acc[RAW_CNT_MASS] += (la ? 1.f : 0.f) + (lb ? 1.f : 0.f);
        acc[RAW_CNT_GROW] += (fpa > kEps ? 1.f : 0.f) + (fpb > kEps ? 1.f : 0.f);
        border |= ((x == 0 || x == N - 1) && (la || lb)) || (r == 0 && la) || (r == N / 2 - 1 && lb);
      }
      acc[RAW_M00] += Sa + Sb;
      acc[RAW_G00] += Ga + Gb;
      acc[RAW_MX + 0] += cya * Sa + cyb * Sb;
      acc[RAW_GX + 0] += cya * Ga + cyb * Gb;
      acc[RAW_MX2 + 0] += cya * cya * Sa + cyb * cyb * Sb;
    }
    big_finish_step(a, world, step, 2, sizes, acc, border, red, shv);
  }
}

// ------------------------------------------------------------------ big 3D
// One N^3 world per CTA.  Per step:
//   A. planes forward: the CTA is cut into SL slices of (N/2)*4 threads; each
//      slice takes one z plane at a time through the resident engine's row
//      and column passes in shared memory (row pairs packed as one complex
//      row, column pairs unpacked) and writes the plane's true half spectrum
//      X[z][ky][kx], kx in [0, N/2], to the per-CTA scratch (the packed
//      DC / Nyquist column is split with its ky mirror);
//   B. z pass over the scratch: lines (ky, kx) on groups of LG lanes, forward
//      FFT, x prepared spectrum (scaled 1/N^3), inverse FFT;
//   C. planes inverse: each slice's spectrum plane arrives by bulk copy into
//      shared memory (issued one plane ahead, mbarrier with a bounded wait);
//      column inverse (DC and Nyquist columns re-packed as DC + i Nyquist),
//      row inverse -> potential, growth, update, moments, and the run_scan
//      trajectories when asked.
// The next state plane (A, C) and the z pass's next round of lines (B) are
// prefetched into L2 with bulk prefetches.
template <int N, int LG, int GF>
__device__ __noinline__ void big3d_item(const BigArgs& a, int world, const float2* tw4, const float2* twz,
                                        float2* work) {
  using B3 = Big3D<N, LG>;
  using GE = typename B3::GE;
  using GZ = typename B3::GZ;
  constexpr int G = B3::G, P = GE::P, Q = GE::Q, HW = B3::HW, NT = B3::NT, SL = B3::SL, PITCH = B3::PITCH;
  constexpr int PZ = GZ::P, QZ = GZ::Q, NGZ = 512 / LG;
  constexpr size_t PLANE = (size_t)N * HW;
  const float2 *tw_std = tw4, *tw_colf = tw4 + N, *tw_rowi = tw4 + 2 * N;
  const int sub = threadIdx.x / NT, tid = threadIdx.x % NT;
  const int grp = tid / G, t = tid % G, lane = threadIdx.x & 31;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int bar_id = 1 + sub;
  float2* buf = work + sub * (B3::BUF + B3::CSCR);
  float2* cs = buf + B3::BUF + grp * GE::SCR;
  float2* rowbuf = buf + grp * PITCH;
  float* red = reinterpret_cast<float*>(work + B3::REGION);
  int* shv = reinterpret_cast<int*>(red + 16 * 16);
  uint64_t* xbar = reinterpret_cast<uint64_t*>(red + kBigRed) + sub;  // this slice's plane copies
  float2* xs = work + B3::XSOFF + sub * B3::XS;                       // this slice's staged plane
  static_assert(SL <= kBigBars, "one mbarrier per slice");
  float2* X = a.scratch + (size_t)blockIdx.x * a.scratch_per_cta;
  const int sol = world / a.n_init;
  const float2* kp = a.kp + (size_t)sol * N * PLANE;  // [N][N][HW], scaled by 1/N^3
  const float* c0 = a.cells0 + (size_t)world * N * N * N;
  float* st = a.state + (size_t)world * N * N * N;
  const GrowthP gq = big_growth<GF>(a, sol);
  const float wk = __ldg(a.w + sol), wf = a.mean ? wk / wk : wk;
  const float dt = big_dt(a, world, sol);
  const int sizes[3] = {N, N, N};
  const int c = grp;  // column pair of the column passes: (c, N-c); c == 0 carries (0, N/2)
  const int c1 = c != 0 ? c : 0, c2 = c != 0 ? N - c : N / 2;
  if (threadIdx.x == 0) shv[0] = shv[1] = shv[2] = 0;
  if (tid == 0) {
    mbar_init(xbar, 1);
    fence_proxy_async();
  }
  unsigned xph = 0;  // phase parity of this slice's next plane copy
  // bulk copy of spectrum plane z into the slice's staging buffer
  auto stage_plane = [&](int z) {
    mbar_arrive_expect_tx(xbar, (unsigned)(PLANE * sizeof(float2)));
    bulk_load(xs, X + (size_t)z * PLANE, (unsigned)(PLANE * sizeof(float2)), xbar);
  };
  __syncthreads();
  for (int step = 0; step < a.steps; ++step) {
    const float* src = step == 0 ? c0 : st;
    // ---------------------------------------------------------- A. planes forward
    for (int zb = 0; zb < N; zb += SL) {
      const int z = zb + sub;
      if (tid == 0 && z + SL < N) prefetch_l2(src + (size_t)(z + SL) * N * N, N * N * sizeof(float));
      {
        const float* pl = src + (size_t)z * N * N;
        float2 v[P];
#pragma unroll
        for (int n2 = 0; n2 < P; ++n2)
          v[n2] = make_float2(pl[(2 * grp) * N + t + G * n2], pl[(2 * grp + 1) * N + t + G * n2]);
        float2 u[Q][G];
        fft_standard<GE, false, false>(v, u, rowbuf, tw_std, t, gmask);
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
          for (int k1 = 0; k1 < G; ++k1) rowbuf[t + G * q + P * k1] = u[q][k1];
      }
      named_bar(bar_id, NT);
      {
        float2 v[Q][G];
#pragma unroll
        for (int jp = 0; jp < Q / 2; ++jp) {
          const int m = t + G * jp;
#pragma unroll
          for (int n2 = 0; n2 < G; ++n2) {
            const int rr = m + (P / 2) * n2;
            const float2 z1 = buf[rr * PITCH + c1], z2 = buf[rr * PITCH + c2];
            if (c != 0) {
              v[2 * jp][n2] = caddc(z1, z2);  // 2 X[2rr][c]
              const float2 d = csubc(z1, z2);  // 2i X[2rr+1][c]
              v[2 * jp + 1][n2] = make_float2(d.y, -d.x);
            } else {
              v[2 * jp][n2] = make_float2(z1.x, z2.x);
              v[2 * jp + 1][n2] = make_float2(z1.y, z2.y);
            }
          }
        }
        float2 w[P];
        fft_mirrored<GE, false, false>(v, w, cs, tw_colf, t, gmask);  // w[k1]: ky = t + G*k1
        float2* xz = X + (size_t)z * PLANE;
        if (c != 0) {
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) xz[(t + G * k1) * HW + c] = make_float2(0.5f * w[k1].x, 0.5f * w[k1].y);
        } else {
          // w = X0 + i XN (x-DC and x-Nyquist columns); X0[ky] = (w[ky] + conj w[-ky]) / 2,
          // XN[ky] = -i (w[ky] - conj w[-ky]) / 2
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) cs[t + G * k1] = w[k1];
          __syncwarp(gmask);
#pragma unroll
          for (int k1 = 0; k1 < P; ++k1) {
            const int ky = t + G * k1;
            const float2 mr = cs[(N - ky) & (N - 1)];
            xz[ky * HW] = make_float2(0.5f * (w[k1].x + mr.x), 0.5f * (w[k1].y - mr.y));
            xz[ky * HW + N / 2] = make_float2(0.5f * (w[k1].y + mr.y), -0.5f * (w[k1].x - mr.x));
          }
          __syncwarp(gmask);
        }
      }
      named_bar(bar_id, NT);
    }
    __syncthreads();
    // ---------------------------------------------------------- B. z pass
    {
      const int zg = threadIdx.x / LG, zt = threadIdx.x % LG;
      const unsigned zmask = ((1u << LG) - 1u) << (lane & ~(LG - 1));
      float2* zs = work + zg * GZ::SCR;
      for (int l = zg; l < N * HW; l += NGZ) {
        // L2 prefetch of the next round of lines: z row zg of the scratch and of the spectrum
        const int next = l - zg + NGZ;
        if (zt == 0 && zg < N && next < N * HW) {
          const unsigned bytes = (unsigned)(min(NGZ, N * HW - next) * sizeof(float2));
          prefetch_l2(X + (size_t)zg * PLANE + next, bytes);
          prefetch_l2(kp + (size_t)zg * PLANE + next, bytes);
        }
        float2* base = X + l;  // l = ky * HW + kx
        const float2* kb = kp + l;
        float2 v[PZ];
#pragma unroll
        for (int n2 = 0; n2 < PZ; ++n2) v[n2] = base[(size_t)(zt + LG * n2) * PLANE];
        float2 u[QZ][LG];
        fft_standard<GZ, false, false>(v, u, zs, twz, zt, zmask);
#pragma unroll
        for (int q = 0; q < QZ; ++q)
#pragma unroll
          for (int k1 = 0; k1 < LG; ++k1) {
            const int kz = zt + LG * q + PZ * k1;
            u[q][k1] = cmul(u[q][k1], __ldg(kb + (size_t)kz * PLANE));
          }
#pragma unroll
        for (int q = 0; q < QZ; ++q)
#pragma unroll
          for (int k1 = 0; k1 < LG; ++k1) zs[zt + LG * q + PZ * k1] = u[q][k1];
        __syncwarp(zmask);
#pragma unroll
        for (int n2 = 0; n2 < PZ; ++n2) v[n2] = zs[zt + LG * n2];
        __syncwarp(zmask);
        fft_standard<GZ, true, false>(v, u, zs, twz, zt, zmask);
#pragma unroll
        for (int q = 0; q < QZ; ++q)
#pragma unroll
          for (int k1 = 0; k1 < LG; ++k1) base[(size_t)(zt + LG * q + PZ * k1) * PLANE] = u[q][k1];
      }
    }
    __syncthreads();
    // ---------------------------------------------------------- C. planes inverse
    // Each slice's spectrum planes arrive by bulk copy into its staging
    // buffer: plane z + SL is issued once every thread of the slice is past
    // its reads of plane z (the slice barrier between the column and row
    // inverses), so it lands during plane z's row inverse.
    if (tid == 0) {
      fence_proxy_async();
      stage_plane(sub);
    }
    float acc[14];
#pragma unroll
    for (int i = 0; i < 14; ++i) acc[i] = 0.f;
    bool border = false;
    const int sz = shv[0], sy = shv[1], sx = shv[2];
    for (int zb = 0; zb < N; zb += SL) {
      const int z = zb + sub;
      if (tid == 0 && z + SL < N) prefetch_l2(src + (size_t)(z + SL) * N * N, N * N * sizeof(float));
      if (!mbar_wait(xbar, xph)) {  // the plane never landed: record it, give it a bounded second wait
        if (tid == 0 && a.status) atomicExch(a.status, kStatusCopyTimeout);
        mbar_wait(xbar, xph);
      }
      xph ^= 1u;
      {
        const float2* xz = xs;
        float2 w[P];
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          const int ky = t + G * k1;
          if (c != 0) {
            w[k1] = xz[ky * HW + c];
          } else {
            const float2 a0 = xz[ky * HW], an = xz[ky * HW + N / 2];
            w[k1] = make_float2(a0.x - an.y, a0.y + an.x);  // DC + i Nyquist
          }
        }
        float2 u[Q][G];
        fft_standard<GE, true, true>(w, u, cs, tw_std, t, gmask);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int m = t + G * (q >> 1);
          const int col = (q & 1) ? c2 : c1;
#pragma unroll
          for (int k1 = 0; k1 < G; ++k1) buf[(m + (P / 2) * k1) * PITCH + col] = u[q][k1];
        }
      }
      named_bar(bar_id, NT);
      if (tid == 0 && z + SL < N) {  // the slice is done with xs: stage its next plane
        fence_proxy_async();
        stage_plane(z + SL);
      }
      {
        const int r = grp;
        float2 v[Q][G];
        unpack_row_pair<GE>(rowbuf, v, t);
        __syncwarp(gmask);
        float2 w[P];
        fft_mirrored<GE, true, true>(v, w, rowbuf, tw_rowi, t, gmask);  // w[k1]: x = t + G*k1
        const float cz = (float)(((z - sz) & (N - 1)) - N / 2);
        const float cya = (float)(((2 * r - sy) & (N - 1)) - N / 2);
        const float cyb = (float)(((2 * r + 1 - sy) & (N - 1)) - N / 2);
        const float* sra = src + ((size_t)z * N + 2 * r) * N;
        float* dsa = st + ((size_t)z * N + 2 * r) * N;
        float Sa = 0.f, Sb = 0.f, Ga = 0.f, Gb = 0.f;
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          const int x = t + G * k1;
          const float pa = w[k1].x, pb = w[k1].y;
          const float sa = sra[x], sb = sra[N + x];
          const float fa = weighted_growth<GF>(gq, pa, wf), fb = weighted_growth<GF>(gq, pb, wf);
          dsa[x] = state_fn(a.state_fn, sa, fa, dt);
          dsa[N + x] = state_fn(a.state_fn, sb, fb, dt);
          if (a.traj_cells || a.traj_field || a.traj_pot) {  // run_scan trajectories (runner.py:119-164)
            const size_t tb = ((size_t)step * a.n_worlds + world) * N * N * N + ((size_t)z * N + 2 * r) * N + x;
            if (a.traj_cells) {
              a.traj_cells[tb] = sa;
              a.traj_cells[tb + N] = sb;
            }
            if (a.traj_field) {
              a.traj_field[tb] = fa;
              a.traj_field[tb + N] = fb;
            }
            if (a.traj_pot) {
              a.traj_pot[tb] = pa;
              a.traj_pot[tb + N] = pb;
            }
          }
          const float fpa = fmaxf(fa, 0.f), fpb = fmaxf(fb, 0.f);
          const float cx = (float)(((x - sx) & (N - 1)) - N / 2);
          Sa += sa;
          Sb += sb;
          Ga += fpa;
          Gb += fpb;
          const float ss = sa + sb, gg = fpa + fpb;
          acc[RAW_MX + 2] = fmaf(ss, cx, acc[RAW_MX + 2]);
          acc[RAW_GX + 2] = fmaf(gg, cx, acc[RAW_GX + 2]);
          acc[RAW_MX2 + 2] = fmaf(ss * cx, cx, acc[RAW_MX2 + 2]);
          acc[RAW_CNT_POT] += (pa > kEps ? 1.f : 0.f) + (pb > kEps ? 1.f : 0.f);
          const bool la = sa > kEps, lb = sb > kEps;
          acc[RAW_CNT_MASS] += (la ? 1.f : 0.f) + (lb ? 1.f : 0.f);
          acc[RAW_CNT_GROW] += (fpa > kEps ? 1.f : 0.f) + (fpb > kEps ? 1.f : 0.f);
          border |= ((x == 0 || x == N - 1 || z == 0 || z == N - 1) && (la || lb)) || (r == 0 && la) ||
                    (r == N / 2 - 1 && lb);
        }
        const float S = Sa + Sb, Gs = Ga + Gb;
        acc[RAW_M00] += S;
        acc[RAW_G00] += Gs;
        acc[RAW_MX + 0] += cz * S;
        acc[RAW_GX + 0] += cz * Gs;
        acc[RAW_MX2 + 0] += cz * cz * S;
        acc[RAW_MX + 1] += cya * Sa + cyb * Sb;
        acc[RAW_GX + 1] += cya * Ga + cyb * Gb;
        acc[RAW_MX2 + 1] += cya * cya * Sa + cyb * cyb * Sb;
      }
      named_bar(bar_id, NT);
    }
    big_finish_step(a, world, step, 3, sizes, acc, border, red, shv);
  }
  __syncthreads();
  if (tid == 0) mbar_inval(xbar);  // the area holds other items' data next
}

template <int N, int G, int GF>
__device__ __noinline__ void resident_item_call(const ResidentArgs& a, int item, const float2* tw, float2* work) {
  int loaded = -1;
  resident_item<N, G, GF>(a, item, tw, work, loaded);
}

template <int GF>
__device__ __forceinline__ void dispatch_gf(const BatchClassArgs& c, int item, float2* sm, float2* work) {
  switch (c.kind) {
    case BK_R32: resident_item_call<32, 4, GF>(c.r, item, sm + TW32, work); break;
    case BK_R64: resident_item_call<64, 4, GF>(c.r, item, sm + TW64, work); break;
    case BK_R128: resident_item_call<128, 8, GF>(c.r, item, sm + TW128, work); break;
    case BK_B2D256: big2d_item<256, GF>(c.b, item, sm + TW256, work); break;
    case BK_B3D32:
      if (c.line_group == 2) big3d_item<32, 2, GF>(c.b, item, sm + TW32, sm + TW32G2, work);
      else big3d_item<32, 4, GF>(c.b, item, sm + TW32, sm + TW32, work);
      break;
    case BK_B3D64:
      if (c.line_group == 2) big3d_item<64, 2, GF>(c.b, item, sm + TW64, sm + TW64G2, work);
      else big3d_item<64, 4, GF>(c.b, item, sm + TW64, sm + TW64, work);
      break;
  }
}

__global__ void __launch_bounds__(512, 1) mixed_kernel(MixedArgs ma) {
  extern __shared__ __align__(16) float2 sm[];
  init_twiddles<Geo<32, 4>>(sm + TW32, sm + TW32 + 32, sm + TW32 + 64, threadIdx.x, blockDim.x);
  init_twiddles<Geo<64, 4>>(sm + TW64, sm + TW64 + 64, sm + TW64 + 128, threadIdx.x, blockDim.x);
  init_twiddles<Geo<128, 8>>(sm + TW128, sm + TW128 + 128, sm + TW128 + 256, threadIdx.x, blockDim.x);
  init_twiddles<Geo<256, 8>>(sm + TW256, sm + TW256 + 256, sm + TW256 + 512, threadIdx.x, blockDim.x);
  // G = 2 line transforms use only the standard table
  for (int i = threadIdx.x; i < 64; i += blockDim.x) sm[TW64G2 + i] = reinterpret_cast<const float2*>(kTwiddles<64, 2>.v)[i];
  for (int i = threadIdx.x; i < 32; i += blockDim.x) sm[TW32G2 + i] = reinterpret_cast<const float2*>(kTwiddles<32, 2>.v)[i];
  __syncthreads();
  __shared__ BatchClassArgs s_cls[kMaxBatchClasses];
  __shared__ int s_item;
  {
    const int* src = reinterpret_cast<const int*>(ma.cls);
    int* dst = reinterpret_cast<int*>(s_cls);
    const int n = ma.n_cls * (int)(sizeof(BatchClassArgs) / sizeof(int));
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  float2* work = sm + TW_END;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(ma.head, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= ma.n_items) break;
    const int2 w = ma.items[it];
    const BatchClassArgs& c = s_cls[w.x];
    if (c.gf_variant == GF_FAST_GAUSSIAN) dispatch_gf<GF_FAST_GAUSSIAN>(c, w.y, sm, work);
    else if (c.gf_variant == GF_FAST_POLY4) dispatch_gf<GF_FAST_POLY4>(c, w.y, sm, work);
    else dispatch_gf<GF_GENERIC>(c, w.y, sm, work);
  }
}

template <int N>
__global__ void prepare_3d_kernel(long n, const float2* __restrict__ kh, float2* __restrict__ kp) {
  const long total = n * (long)N * N * (N / 2 + 1);
  const float scale = 1.f / ((float)N * (float)N * (float)N);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const float2 k = kh[i];
    kp[i] = make_float2(k.x * scale, k.y * scale);
  }
}

__global__ void batch_setup_kernel(BatchSetup s) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0) {
    const int* src = reinterpret_cast<const int*>(s.cls);
    int* dst = reinterpret_cast<int*>(s.cls_out);
    const int n = s.n_cls * (int)(sizeof(BatchClassArgs) / sizeof(int));
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
    if (threadIdx.x == 0) *s.head = 0;
  }
  for (int i = tid; i < s.n_items; i += gridDim.x * blockDim.x) {
    int r = 0;
    while (r + 1 < s.n_cls && s.first_item[r + 1] <= i) ++r;
    s.items[i] = make_int2(s.cls_of_rank[r], i - s.first_item[r]);
  }
}

}  // namespace

cudaError_t launch_batch_setup(const BatchSetup& s, cudaStream_t st) {
  const int blocks = (int)std::min<long>((s.n_items + 255) / 256 + 1, 1024);
  batch_setup_kernel<<<blocks, 256, 0, st>>>(s);
  return cudaGetLastError();
}

size_t mixed_smem_bytes() { return kMixedSmem; }

long batch_scratch_per_cta(int kind) {
  switch (kind) {
    case BK_B2D256: return 128L * 256;
    case BK_B3D32: return 32L * 32 * 17;
    case BK_B3D64: return 64L * 64 * 33;
  }
  return 0;
}

int batch_worlds_per_item(int kind) {
  switch (kind) {
    case BK_R32: return RCfg<32, 4>::WPC;
    case BK_R64: return RCfg<64, 4>::WPC;
    case BK_R128: return RCfg<128, 8>::WPC;
  }
  return 1;
}

int batch_kind_gf_variant(int gf_id) {
  return gf_id == LGX_GF_GAUSSIAN ? GF_FAST_GAUSSIAN : (gf_id == LGX_GF_POLY_QUAD4 ? GF_FAST_POLY4 : GF_GENERIC);
}

cudaError_t launch_mixed(const MixedArgs& a, int grid, cudaStream_t st) {
  // set once per device, before any stream capture of a launch (the first
  // launch on a device happens uncaptured: UnevenBatch.capture warms up first)
  static std::mutex mu;
  static bool attr_set[64] = {false};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!attr_set[dev]) {
      e = cudaFuncSetAttribute(mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMixedSmem);
      if (e != cudaSuccess) return e;
      attr_set[dev] = true;
    }
  }
  mixed_kernel<<<grid, 512, kMixedSmem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_prepare_3d_spectrum(int N, long n, const float2* k_half, float2* kp, cudaStream_t st) {
  const long total = n * (long)N * N * (N / 2 + 1);
  const int blocks = (int)std::min<long>((total + 255) / 256, 8192);
  switch (N) {
    case 32: prepare_3d_kernel<32><<<blocks, 256, 0, st>>>(n, k_half, kp); break;
    case 64: prepare_3d_kernel<64><<<blocks, 256, 0, st>>>(n, k_half, kp); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace lgx
