// Streamed Lenia step for any channel/kernel topology (2D, square power-of-two
// worlds of side 32..512): the spectra of a step travel through HBM/L2
// between its kernels.
//
//   row_fwd  : per (world, channel, packed row) N-point FFT of rows (2r, 2r+1)
//              packed as one complex row -> spec[n][c][r][.] in the
//              pair-adjacent layout (pa_pos, fft.cuh); first step only
//   col_conv : per (world, channel, block of column pairs) the block's column
//              tile arrives by TMA (2D tensor copies, 128-byte swizzle); per
//              pair: unpack + N-point FFT, then for every kernel reading that
//              channel: x prepared spectrum (column-major planes, so a
//              transform's lanes read consecutive ky; bulk-staged up to
//              N = 128), inverse FFT -> prod[n][k] (same pair-adjacent
//              layout), written back through the tile by TMA stores
//   row_inv  : per (world, block of packed rows) the block's rows of every
//              kernel's product plane arrive by bulk copies into a staging
//              ring (the next kernel's rows land while this kernel's are
//              transformed), each channel's state rows by one bulk copy;
//              inverse row FFTs -> potential, growth, weighted field in
//              registers (core.py:163-242), state update (core.py:245-319),
//              per-block raw statistics moments, and the next step's forward
//              row FFT of the new rows
//   reduce   : per world: block moments -> raw moments of the step, carried
//              torus shift update (statistics.py:117-119)
//
// This is leniax core.update with get_potential_fft (core.py:52-102), the
// true-kernel selection (tc_indices, core.py:97-98) being the (c_in, slot)
// table of the plan.
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "engine.h"
#include "fft.cuh"
#include "tma.cuh"

namespace lgx {

namespace {

constexpr int kThreads = 256;  // row_fwd blocks

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
struct SCfg<256> { static constexpr int G = 16; };  // P = 16 points per lane (Q == 1 transforms)
template <>
struct SCfg<512> { static constexpr int G = 16; };

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
    for (int k1 = 0; k1 < G; ++k1) dst[pa_pos<N>(t + G * q + P * k1)] = u[q][k1];
}

// ----------------------------------------------------------------- col_conv
template <int N>
struct ColCfg {
  static constexpr int G = SCfg<N>::G;
  static constexpr int T = ((N / 2) * G < 128) ? (N / 2) * G : 128;  // threads per block
  static constexpr int GPB = T / G;                // column pairs per block (one per group)
  static constexpr int BPP = (N / 2) / GPB;        // blocks per plane
  static constexpr int BOXES = GPB / 8;            // TMA boxes: 8 pairs (128 bytes) x N/2 rows
  static constexpr int BOX_BYTES = (N / 2) * 128;
  static constexpr int TILE_BYTES = BOXES * BOX_BYTES;
  // kernel spectrum columns staged by bulk copy (GPB columns + the Nyquist
  // column for the block holding pair 0) up to N = 128; from N = 256 on the
  // staging buffer would cost a resident block per SM, which measured slower
  // than the (coalesced, column-major) direct loads
  static constexpr bool KSTAGE = N <= 128;
  static constexpr int KB_BYTES = KSTAGE ? (GPB + 1) * N * 8 : 0;
  static_assert(GPB % 8 == 0 && (N / 2) % GPB == 0, "column tile");
};

template <int N>
constexpr size_t col_conv_smem() {
  using CC = ColCfg<N>;
  using GE = Geo<N, CC::G>;
  // 1024 bytes of alignment slack for the swizzled tile, tile (the column
  // input, then the output staging), staged kernel columns, twiddles, group
  // scratch, DC/Nyquist mirror, two mbarriers
  return 1024 + (size_t)CC::TILE_BYTES + (size_t)CC::KB_BYTES + (size_t)3 * N * sizeof(float2) +
         (size_t)CC::GPB * GE::SCR * sizeof(float2) + (size_t)N * sizeof(float2) + 16;
}

// Next kernel after k (or K) reading channel ch.
__device__ __forceinline__ int next_kernel(const KTab& tab, int k, int ch) {
  for (++k; k < tab.K; ++k)
    if (tab.cin[k] == ch) break;
  return k;
}

// One block: GPB column pairs of one (world, channel) plane.  The column tile
// arrives by TMA; per kernel reading the channel, the kernel's GPB spectrum
// columns arrive by bulk copy (issued one kernel ahead), and the product
// columns leave through the same swizzled tile by TMA stores, so the kernel's
// global traffic bypasses the load/store pipe.
template <int N>
__global__ void __launch_bounds__(ColCfg<N>::T) col_conv_kernel(const __grid_constant__ CUtensorMap spec_map,
                                                               const __grid_constant__ CUtensorMap prod_map,
                                                               int n_worlds, int n_init, KTab tab,
                                                               const float2* __restrict__ kp, long kp_sol_stride,
                                                               int* __restrict__ status) {
  using CC = ColCfg<N>;
  constexpr int G = CC::G, GPB = CC::GPB, BPP = CC::BPP;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q;
  constexpr int KPITCH = N / 2 + 2;
  extern __shared__ __align__(16) unsigned char smraw[];
  unsigned char* tile = smraw + ((1024u - (smem_u32(smraw) & 1023u)) & 1023u);
  float2* kb = reinterpret_cast<float2*>(tile + CC::TILE_BYTES);  // [GPB + 1][N] kernel columns
  float2* sm = reinterpret_cast<float2*>(tile + CC::TILE_BYTES + CC::KB_BYTES);
  float2* scr = sm + 3 * N;
  float2* mirror = scr + GPB * GE::SCR;
  uint64_t* bar = reinterpret_cast<uint64_t*>(mirror + N);  // [0]: column tile, [1]: kernel columns
  const int plane = blockIdx.x / BPP;  // n*C + c
  if (plane >= n_worlds * tab.C) return;
  const int j0 = (blockIdx.x % BPP) * GPB;
  const int n = plane / tab.C, ch = plane % tab.C;
  const int sol = n / n_init;
  auto kplane = [&](int k) {
    return kp + sol * kp_sol_stride + ((size_t)(ch * tab.max_k + tab.slot[k]) * N) * KPITCH;
  };
  // kernel k's columns j0 .. j0 + GPB - 1 (+ column N/2 for pair 0) -> kb
  auto issue_kernel = [&](int k) {
    const unsigned main = GPB * N * sizeof(float2), nyq = j0 == 0 ? N * sizeof(float2) : 0u;
    mbar_arrive_expect_tx(&bar[1], main + nyq);
    const float2* kk = kplane(k);
    bulk_load(kb, kk + (size_t)j0 * N, main, &bar[1]);
    if (nyq) bulk_load(kb + GPB * N, kk + (size_t)(N / 2) * N, nyq, &bar[1]);
  };
  const int k_first = next_kernel(tab, -1, ch);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_proxy_async();
    mbar_arrive_expect_tx(&bar[0], CC::TILE_BYTES);
    for (int b = 0; b < CC::BOXES; ++b)
      tma_load_2d(tile + b * CC::BOX_BYTES, &spec_map, (j0 + 8 * b) * 4, plane * (N / 2), &bar[0]);
    if (CC::KSTAGE && k_first < tab.K) issue_kernel(k_first);
  }
  init_twiddles<GE>(sm, sm + N, sm + 2 * N, threadIdx.x, blockDim.x);
  __syncthreads();
  if (__syncthreads_or(!mbar_wait(&bar[0], 0))) {  // the tile never landed: record, drain, leave
    if (threadIdx.x == 0) {
      if (status) atomicExch(status, kStatusCopyTimeout);
      mbar_wait(&bar[0], 0);
      if (CC::KSTAGE && k_first < tab.K) mbar_wait(&bar[1], 0);
    }
    return;
  }
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31;
  const int j = j0 + grp;  // column pair (j, N-j); j == 0 carries (0, N/2)
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  float2* cs = scr + grp * GE::SCR;
  unsigned char* tb = tile + (grp >> 3) * CC::BOX_BYTES;
  const int chunk = grp & 7;

  float2 v[Q][G];
  if constexpr (Q == 1) {
    // lane t carries the unpacked rows n = t + P*n2: packed row n >> 1, the
    // even row's value for even n, the odd row's for odd n (lanes 2m, 2m+1
    // read the same 16-byte pair)
#pragma unroll
    for (int n2 = 0; n2 < G; ++n2) {
      const int r = t + P * n2;
      const float4 q = *reinterpret_cast<const float4*>(tb + swz128(r >> 1, chunk));
      if (j != 0) v[0][n2] = (r & 1) ? make_float2(q.y + q.w, q.z - q.x) : make_float2(q.x + q.z, q.y - q.w);
      else v[0][n2] = (r & 1) ? make_float2(q.y, q.w) : make_float2(q.x, q.z);
    }
  } else {
#pragma unroll
    for (int jp = 0; jp < Q / 2; ++jp) {
      const int m = t + G * jp;
#pragma unroll
      for (int n2 = 0; n2 < G; ++n2) {
        const int r = m + (P / 2) * n2;
        const float4 q = *reinterpret_cast<const float4*>(tb + swz128(r, chunk));
        if (j != 0) {
          v[2 * jp][n2] = make_float2(q.x + q.z, q.y - q.w);      // 2 X[2r][j]
          v[2 * jp + 1][n2] = make_float2(q.y + q.w, q.z - q.x);  // 2 X[2r+1][j]
        } else {
          v[2 * jp][n2] = make_float2(q.x, q.z);  // X[2r][0] + i X[2r][N/2]
          v[2 * jp + 1][n2] = make_float2(q.y, q.w);
        }
      }
    }
  }
  float2 w0[P];
  fft_mirrored<GE, false, false>(v, w0, cs, sm + N, t, gmask);
  // the packed DC / Nyquist column keeps its spectrum in the block's mirror
  // buffer: Q[ky] needs A[-ky] for every kernel
  if (j == 0) {
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) mirror[t + G * k1] = w0[k1];
    __syncwarp(gmask);
  }
  int it = 0;
  for (int k = k_first; k < tab.K; k = next_kernel(tab, k, ch), ++it) {
    bool ok = true;
    if constexpr (CC::KSTAGE) ok = mbar_wait(&bar[1], it & 1);
    float2 w[P];
    if (ok) {
      const float2* kc = CC::KSTAGE ? kb + grp * N : kplane(k) + (size_t)j * N;
      const float2* kn = CC::KSTAGE ? kb + GPB * N : kplane(k) + (size_t)(N / 2) * N;
      if (j != 0) {
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) w[k1] = cmul(w0[k1], kc[t + G * k1]);
      } else {
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
          const int ky = t + G * k1;
          const float2 A = kc[ky], B = kn[ky];
          w[k1] = cadd(cmul(w0[k1], A), cmul(conjf2(mirror[(N - ky) & (N - 1)]), B));
        }
      }
    }
    // past this barrier: kb is free for the next kernel, and the previous
    // product's store has read the tile
    if (threadIdx.x == 0) bulk_wait_read_all();
    if (__syncthreads_or(!ok)) {  // a kernel column copy never landed
      if (threadIdx.x == 0) {
        if (status) atomicExch(status, kStatusCopyTimeout);
        mbar_wait(&bar[1], it & 1);
        bulk_wait_all();
      }
      return;
    }
    const int k_next = next_kernel(tab, k, ch);
    if (CC::KSTAGE && threadIdx.x == 0 && k_next < tab.K) issue_kernel(k_next);
    float2 u[Q][G];
    if constexpr (Q == 1) {
      // unpacked row r = t + P*k1 -> its half of pair j of packed row r >> 1
      fft_standard<GE, true, false>(w, u, cs, sm, t, gmask);
#pragma unroll
      for (int k1 = 0; k1 < G; ++k1) {
        const int r = t + P * k1;
        *reinterpret_cast<float2*>(tb + swz128(r >> 1, chunk) + (r & 1) * 8) = u[0][k1];
      }
    } else {
      fft_standard<GE, true, true>(w, u, cs, sm, t, gmask);
#pragma unroll
      for (int a = 0; a < Q / 2; ++a) {
        const int m = t + G * a;
#pragma unroll
        for (int k1 = 0; k1 < G; ++k1) {
          const int r = m + (P / 2) * k1;
          *reinterpret_cast<float4*>(tb + swz128(r, chunk)) =
              make_float4(u[2 * a][k1].x, u[2 * a][k1].y, u[2 * a + 1][k1].x, u[2 * a + 1][k1].y);
        }
      }
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int b = 0; b < CC::BOXES; ++b)
        tma_store_2d(&prod_map, (j0 + 8 * b) * 4, (n * tab.K + k) * (N / 2), tile + b * CC::BOX_BYTES);
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

// ------------------------------------------------------------------ row_inv
// Block = GPB groups = GPB packed rows of one world.  Work items are the
// (output channel, kernel) pairs with a nonzero weight, channel by channel,
// then the kernels that feed no channel (their potentials still count in
// potential_volume).  Item i's GPB product rows are bulk-copied into buffer
// i & 1 (row pitch N + G) while item i-1 is transformed; after unpacking its
// row, a group reuses that row as its FFT exchange scratch.  The weighted
// field of the current channel stays in registers (2*P values per thread); a
// kernel feeding several channels is transformed once per channel, its
// potential counted (and written) at the first.
template <int N>
struct RowInvCfg {
  static constexpr int G = SCfg<N>::G;
  static constexpr int T = ((N / 2) * G < 128) ? (N / 2) * G : 128;  // threads per block
  static constexpr int GPB = T / G;
  static constexpr int BPW = (N / 2) / GPB;  // blocks per world
  static constexpr int ROWP = N + G;         // staged row pitch (float2) == Geo<N, G>::SCR
  static constexpr int BUF = GPB * ROWP;     // float2 per buffer
  static constexpr int NBUF = 2;             // staging ring depth (items in flight: NBUF - 1)
  static constexpr int SSTP = 2 * N + 16;    // staged state rows (2r, 2r+1) pitch per group (floats)
};

// item word: bit 16 = count the potential, bits 8..15 = output channel + 1 (0: none), bits 0..7 = kernel
__device__ __forceinline__ int item_k(int it) { return it & 255; }
__device__ __forceinline__ int item_co(int it) { return ((it >> 8) & 255) - 1; }
__device__ __forceinline__ bool item_count(int it) { return (it >> 16) & 1; }

template <int N>
size_t row_inv_smem(int C, int K) {
  using RC = RowInvCfg<N>;
  return (size_t)RC::NBUF * RC::BUF * sizeof(float2) + (size_t)RC::GPB * RC::SSTP * sizeof(float) +
         (size_t)3 * N * sizeof(float2) +
         (size_t)(RC::T / 32) * (RAW_CM + kMaxChannels) * sizeof(float) + 16 * sizeof(uint64_t) +
         (size_t)kMaxChannels * sizeof(float) + (size_t)(C * K + K + 1) * sizeof(int) +
         (size_t)(C * K + K + 1) * sizeof(float4) + (size_t)(C * K + 2 * K) * sizeof(float);
}

template <int N, int GF>
__global__ void __launch_bounds__(RowInvCfg<N>::T) row_inv_kernel(
    int n_worlds, int n_init, KTab tab, const float2* __restrict__ prod, const float* __restrict__ gfp,
    long gf_sol_stride, const float* __restrict__ wts, long w_sol_stride, const float* __restrict__ dtp,
    const float* __restrict__ state, float* __restrict__ state_out, float* __restrict__ field_out,
    float* __restrict__ pot_out, const int* __restrict__ shift, float* __restrict__ partial, int* __restrict__ status,
    float2* __restrict__ spec_next) {
  using RC = RowInvCfg<N>;
  constexpr int G = RC::G, GPB = RC::GPB, BPW = RC::BPW, ROWP = RC::ROWP, NBUF = RC::NBUF;
  using GE = Geo<N, G>;
  constexpr int P = GE::P, Q = GE::Q;
  constexpr int RAWS_MAX = RAW_CM + kMaxChannels;
  constexpr int NWARPS = RC::T / 32;
  static_assert(ROWP == GE::SCR, "a staged row doubles as the group's FFT scratch");
  extern __shared__ __align__(16) float2 sm[];
  float2* bufs = sm;                    // [NBUF][GPB][ROWP] staging ring
  float* sst = reinterpret_cast<float*>(bufs + NBUF * RC::BUF);  // [GPB][SSTP] the channel's state rows
  float2* tw = reinterpret_cast<float2*>(sst + GPB * RC::SSTP);  // 3N twiddles
  float* red = reinterpret_cast<float*>(tw + 3 * N);  // [warps][RAWS_MAX]
  uint64_t* bars = reinterpret_cast<uint64_t*>(red + NWARPS * RAWS_MAX);  // NBUF ring + 1 state (16 reserved)
  float* wsum_s = reinterpret_cast<float*>(bars + 16);  // [kMaxChannels]
  float4* ipar = reinterpret_cast<float4*>(wsum_s + kMaxChannels);  // [C*K + K + 1] per item: weight, m, s, a
  __shared__ int s_nitems;

  const int n = blockIdx.x / BPW;
  if (n >= n_worlds) return;
  const int sol = n / n_init;
  const int grp = threadIdx.x / G, t = threadIdx.x % G, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r0 = (blockIdx.x % BPW) * GPB;
  const int r = r0 + grp;
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int C = tab.C, K = tab.K;
  const float* gf = gfp + sol * gf_sol_stride;
  const float* wt = wts + sol * w_sol_stride;
  int* items = reinterpret_cast<int*>(ipar + (C * K + K + 1));  // [C*K + K + 1] item words
  float* wgf = reinterpret_cast<float*>(items + (C * K + K + 1));  // [C*K] weights, then [K][2] (m, s)

  // the solution's weights and growth parameters, one coalesced pass
  for (int q = threadIdx.x; q < C * K + 2 * K; q += blockDim.x)
    wgf[q] = q < C * K ? __ldg(wt + q) : __ldg(gf + (q - C * K));
  init_twiddles<GE>(tw, tw + N, tw + 2 * N, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int b = 0; b <= NBUF; ++b) mbar_init(&bars[b], 1);
    fence_proxy_async();
    // work items with their growth parameters, and per-channel weight sums
    int ni = 0;
    unsigned long long seen = 0ull;
    auto param = [&](float w, int k) {
      const float m = wgf[C * K + 2 * k], sg = wgf[C * K + 2 * k + 1];
      const float a = GF == GF_FAST_GAUSSIAN ? 0.84932180028801904272f / sg
                                             : (GF == GF_FAST_POLY4 ? 1.f / (9.f * (sg * sg)) : 0.f);
      return make_float4(w, m, sg, a);
    };
    for (int co = 0; co < C; ++co) {
      float ws = 0.f;
      for (int k = 0; k < K; ++k) {
        const float w = wgf[co * K + k];
        ws += w;
        if (w == 0.f) continue;
        const bool first = !((seen >> k) & 1ull);
        seen |= 1ull << k;
        ipar[ni] = param(w, k);
        items[ni++] = (first ? (1 << 16) : 0) | ((co + 1) << 8) | k;
      }
      wsum_s[co] = ws;
    }
    for (int k = 0; k < K; ++k)
      if (!((seen >> k) & 1ull)) {
        ipar[ni] = param(0.f, k);
        items[ni++] = (1 << 16) | k;
      }
    s_nitems = ni;
  }
  __syncthreads();
  const int nit = s_nitems;

  // warp 0 stages item i's GPB product rows into ring slot i % NBUF
  auto issue = [&](int i) {
    const int b = i % NBUF;
    const float2* src = prod + (((size_t)n * K + item_k(items[i])) * (N / 2) + r0) * N;
    float2* dst = bufs + b * RC::BUF;
    if (lane == 0) mbar_arrive_expect_tx(&bars[b], (unsigned)(GPB * N * sizeof(float2)));
    __syncwarp();
    for (int g = lane; g < GPB; g += 32) bulk_load(dst + g * ROWP, src + (size_t)g * N, N * sizeof(float2), &bars[b]);
  };
  // warp 0 stages channel co's state rows (2r, 2r+1) of every group into sst
  auto issue_state = [&](int co) {
    const float* src = state + (((size_t)n * C + co) * N + 2 * r0) * N;
    if (lane == 0) mbar_arrive_expect_tx(&bars[NBUF], (unsigned)(GPB * 2 * N * sizeof(float)));
    __syncwarp();
    for (int g = lane; g < GPB; g += 32)
      bulk_load(sst + g * RC::SSTP, src + (size_t)g * 2 * N, 2 * N * sizeof(float), &bars[NBUF]);
  };
  if (wid == 0)
    for (int q = 0; q < NBUF - 1 && q < nit; ++q) issue(q);
  int st_issued = 0, st_done = 0;  // state-row copies issued / waited for (block-uniform)

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
  float2 acc[P];
  bool failed = false;
  int failed_at = 0;

  // item i: wait for its rows, inverse row transform, count / write the
  // potential, accumulate the weighted growth of channel co (co >= 0)
  // One block barrier per item: past it, item i has landed for every thread
  // and every group is done with slot (i - 1) % NBUF (item i - 1, or the
  // fused row FFT's scratch), so warp 0 refills that slot with item
  // i + NBUF - 1.
  auto process = [&](int i) {
    if (__syncthreads_or(!mbar_wait(&bars[i % NBUF], (i / NBUF) & 1))) {
      failed = true;
      failed_at = i;
      return;
    }
    const int it = items[i], k = item_k(it), co = item_co(it);
    // a channel's first item: its state rows start moving (the previous
    // channel's epilogue, the last reader of sst, is behind the barrier)
    const bool first = co >= 0 && (i == 0 || item_co(items[i - 1]) != co);
    st_issued += first ? 1 : 0;
    if (wid == 0) {
      fence_proxy_async();
      if (i + NBUF - 1 < nit) issue(i + NBUF - 1);
      if (first) issue_state(co);
    }
    float2* row = bufs + (i % NBUF) * RC::BUF + grp * ROWP;
    float2 v[Q][G];
    if constexpr (Q == 1) {
      // lane t needs Z[k], k = t + P*n2: one pair load each (k < N/2 for n2 < G/2)
      const float4* p4 = reinterpret_cast<const float4*>(row);
#pragma unroll
      for (int n2 = 0; n2 < G; ++n2) {
        const int k = t + P * n2;
        if (n2 < G / 2) {
          const float4 q = p4[k];  // k == 0: pair 0 = (DC, Nyquist)
          v[0][n2] = k == 0 ? make_float2(q.x, q.z) : make_float2(q.x - q.w, q.y + q.z);
        } else {
          const float4 q = p4[k == N / 2 ? 0 : N - k];
          v[0][n2] = k == N / 2 ? make_float2(q.y, q.w) : make_float2(q.x + q.w, q.z - q.y);
        }
      }
    } else {
      unpack_row_pair_pa<GE>(row, v, t);
    }
    __syncwarp(gmask);
    float2 w[P];
    fft_mirrored<GE, true, true>(v, w, row, tw + 2 * N, t, gmask);
    if (item_count(it)) {
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
    if (co >= 0) {
      const float4 ip = ipar[i];
      const float wk = ip.x;
      GrowthP g;
      g.m = ip.y;
      g.s = ip.z;
      g.a = ip.w;
      g.id = tab.gf[k];
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) {
        if constexpr (GF == GF_GENERIC) {
          acc[k1].x = fmaf(wk, growth_cell<GF>(g, w[k1].x), acc[k1].x);
          acc[k1].y = fmaf(wk, growth_cell<GF>(g, w[k1].y), acc[k1].y);
        } else {  // w (2 e - 1) summed as 2 w e here, minus the channel's weight sum below
          acc[k1] = __ffma2_rn(make_float2(2.f * wk, 2.f * wk), growth_core2<GF>(g, w[k1]), acc[k1]);
        }
      }
    }
  };

  int i = 0;
  for (int co = 0; co < C && !failed; ++co) {
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) acc[k1] = make_float2(0.f, 0.f);
    const int i_begin = i;
    while (!failed && i < nit && item_co(items[i]) == co) process(i++);
    if (failed) break;
    if (i == i_begin) {  // a channel no kernel feeds: fetch its state rows here
      __syncthreads();
      ++st_issued;
      if (wid == 0) {
        fence_proxy_async();
        issue_state(co);
      }
    }
    if (__syncthreads_or(!mbar_wait(&bars[NBUF], (st_issued - 1) & 1))) {
      failed = true;
      failed_at = i;
      break;
    }
    st_done = st_issued;
    // field (weighted_sum / weighted_mean, core.py:202-242), state update, moments
    const float wsum = wsum_s[co];
    const size_t base = ((size_t)n * C + co) * N * N;
    const float* sa_row = sst + grp * RC::SSTP;
    float* da_row = state_out + base + (size_t)(2 * r) * N;
    float* fa_row = field_out ? field_out + base + (size_t)(2 * r) * N : nullptr;
    float Sa = 0.f, Sb = 0.f, Ga = 0.f, Gb = 0.f;
    float2 nsv[P];  // the new rows (2r, 2r+1) at x = t + G*k1: the next step's row-FFT input comb
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      const int x = t + G * k1;
      float fa = acc[k1].x, fb = acc[k1].y;
      if constexpr (GF != GF_GENERIC) {
        fa -= wsum;
        fb -= wsum;
      }
      if (tab.mean) {
        fa = fa / wsum;
        fb = fb / wsum;
      }
      const float sa = sa_row[x], sb = sa_row[N + x];
      nsv[k1] = make_float2(state_fn(tab.state_fn, sa, fa, dt), state_fn(tab.state_fn, sb, fb, dt));
      da_row[x] = nsv[k1].x;
      da_row[N + x] = nsv[k1].y;
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
    if (spec_next) {
      // the next step's row pass, fused: FFT of the packed new rows -> its
      // spectrum plane.  Exchange scratch: this group's row of ring slot
      // (i - 1) % NBUF, the one slot with no copy in flight (items i ..
      // i + NBUF - 2 are); the next process() barrier orders it before reuse.
      float2 u[Q][G];
      fft_standard<GE, false, false>(nsv, u, bufs + ((i + NBUF - 1) % NBUF) * RC::BUF + grp * ROWP, tw, t, gmask);
      float2* dst = spec_next + (((size_t)n * C + co) * (N / 2) + r) * N;
#pragma unroll
      for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int k1 = 0; k1 < G; ++k1) dst[pa_pos<N>(t + G * q + P * k1)] = u[q][k1];
    }
  }
  while (!failed && i < nit) process(i++);  // kernels that feed no channel
  if (failed) {
    // a staged copy never landed: record it, give the copies in flight a
    // bounded time to drain, leave without writing moments
    if (threadIdx.x == 0 && status) atomicExch(status, kStatusCopyTimeout);
    const int f = failed_at;
    for (int q = f; q < f + NBUF - 1 && q < nit; ++q) mbar_wait(&bars[q % NBUF], (q / NBUF) & 1);  // issued: <= f + NBUF - 2
    if (st_issued > st_done) mbar_wait(&bars[NBUF], (st_issued - 1) & 1);
    return;
  }
  // block reduction: warp shuffles then shared memory
  float accm[11] = {m00, g00, cpot, cmass, cgrow, mxy, mxx, gxy, gxx, m2y, m2x};
#pragma unroll
  for (int q = 0; q < 11; ++q) accm[q] = warp_sum(accm[q]);
  const bool anyb = __any_sync(0xffffffffu, border);
  if (lane == 0) {
    float* rd = red + wid * RAWS_MAX;
    rd[RAW_M00] = accm[0];
    rd[RAW_G00] = accm[1];
    rd[RAW_CNT_POT] = accm[2];
    rd[RAW_CNT_MASS] = accm[3];
    rd[RAW_CNT_GROW] = accm[4];
    rd[RAW_MX + 0] = accm[5];
    rd[RAW_MX + 1] = accm[6];
    rd[RAW_MX + 2] = 0.f;
    rd[RAW_GX + 0] = accm[7];
    rd[RAW_GX + 1] = accm[8];
    rd[RAW_GX + 2] = 0.f;
    rd[RAW_MX2 + 0] = accm[9];
    rd[RAW_MX2 + 1] = accm[10];
    rd[RAW_MX2 + 2] = 0.f;
    rd[RAW_BORDER] = anyb ? 1.f : 0.f;
    rd[RAW_SHIFT + 0] = rd[RAW_SHIFT + 1] = rd[RAW_SHIFT + 2] = 0.f;
  }
  __syncthreads();
  const int RAWS = raw_stride(C);
  if (threadIdx.x < RAWS) {
    float sum = 0.f;
    for (int w = 0; w < NWARPS; ++w) sum += red[w * RAWS_MAX + threadIdx.x];
    if (threadIdx.x == RAW_BORDER) sum = sum > 0.f ? 1.f : 0.f;
    partial[((size_t)n * BPW + (blockIdx.x % BPW)) * RAWS + threadIdx.x] = sum;
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
  // column-major planes: element (ky, c) at c * N + ky, so the lanes of a
  // column transform read consecutive ky
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int ky = (int)(i % N);
    const long pc = i / N;
    const int c = (int)(pc % KP);
    const float2* src = kh + ((pc / KP) * N + ky) * HW;
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

template <int N, int GF>
cudaError_t launch_row_inv(const StreamedStep& s, const KTab& tab, cudaStream_t st) {
  using RC = RowInvCfg<N>;
  const size_t sm_inv = row_inv_smem<N>(tab.C, tab.K);
  cudaError_t e = cudaFuncSetAttribute(row_inv_kernel<N, GF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_inv);
  if (e != cudaSuccess) return e;
  row_inv_kernel<N, GF><<<(unsigned)((long)s.n_worlds * RC::BPW), RC::T, sm_inv, st>>>(
      s.n_worlds, s.n_init, tab, s.prod, s.gf, s.gf_sol_stride, s.w, s.w_sol_stride, s.dt, s.state, s.state_out,
      s.field_out, s.pot_out, s.shift, s.partial, s.status, s.emit_spec ? s.spec : nullptr);
  return cudaGetLastError();
}

// cuTensorMapEncodeTiled, fetched once from the driver through the runtime.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// Tensor map of the packed spectrum planes seen as rows of 2N floats:
// boxes of 32 floats (8 column pairs, 128 bytes) x N/2 packed rows,
// 128-byte swizzle.
template <int N>
bool encode_spec_map(CUtensorMap* map, const float2* spec, long planes) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)(2 * N), (cuuint64_t)(planes * (N / 2))};
  const cuuint64_t strides[1] = {(cuuint64_t)(2 * N * sizeof(float))};
  const cuuint32_t box[2] = {32, (cuuint32_t)(N / 2)};
  const cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2*>(spec), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
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
  using CC = ColCfg<N>;
  constexpr size_t sm_col = col_conv_smem<N>();
  cudaError_t e;
  e = cudaFuncSetAttribute(row_fwd_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_fwd);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(col_conv_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_col);
  if (e != cudaSuccess) return e;
  const long planes = (long)s.n_worlds * m.C;
  alignas(64) CUtensorMap spec_map, prod_map;
  if (!encode_spec_map<N>(&spec_map, s.spec, planes)) return cudaErrorInvalidValue;
  if (!encode_spec_map<N>(&prod_map, s.prod, (long)s.n_worlds * m.K)) return cudaErrorInvalidValue;
  if (!s.spec_ready)  // otherwise the previous step's row inverse already wrote this step's row spectra
    row_fwd_kernel<N><<<(unsigned)(planes * BPP), kThreads, sm_fwd, st>>>(s.n_worlds, m.C, s.state, s.spec);
  col_conv_kernel<N><<<(unsigned)(planes * CC::BPP), CC::T, sm_col, st>>>(spec_map, prod_map, s.n_worlds, s.n_init,
                                                                          tab, s.kp, s.kp_sol_stride, s.status);
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
  return launch_streamed_reduce(s, RC::BPW, st);
}

}  // namespace

bool streamed_supported(const Model& m) {
  if (m.nb_dims != 2 || m.H != m.W) return false;
  if (m.C > kMaxChannels || m.K > kMaxKernels) return false;
  if (!(m.H == 32 || m.H == 64 || m.H == 128 || m.H == 256 || m.H == 512) && !generic_size(m.H)) return false;
  return true;
}

int streamed_blocks_per_world(const Model& m) {
  switch (m.H) {
    case 32: return RowInvCfg<32>::BPW;
    case 64: return RowInvCfg<64>::BPW;
    case 128: return RowInvCfg<128>::BPW;
    case 256: return RowInvCfg<256>::BPW;
    case 512: return RowInvCfg<512>::BPW;
  }
  return generic_blocks_per_world(m.H);  // generic sizes: a few packed rows per block
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

cudaError_t launch_streamed_reduce(const StreamedStep& s, int bpw, cudaStream_t st) {
  const int wpb = 8;
  reduce_kernel<<<(s.n_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(s.n_worlds, s.n_init, bpw, s.m->C, s.m->H, s.m->W,
                                                                  s.partial, s.raw, s.raw_sol_stride,
                                                                  s.raw_world_stride, s.shift);
  return cudaGetLastError();
}

cudaError_t launch_streamed_step(const StreamedStep& s, cudaStream_t st) {
  // the row inverse bulk-copies state rows: the state base must be 16-byte aligned
  if ((reinterpret_cast<uintptr_t>(s.state) & 15u) != 0) return cudaErrorMisalignedAddress;
  switch (s.m->H) {
    case 32: return step_n<32>(s, st);
    case 64: return step_n<64>(s, st);
    case 128: return step_n<128>(s, st);
    case 256: return step_n<256>(s, st);
    case 512: return step_n<512>(s, st);
  }
  if (generic_size(s.m->H)) return launch_generic_step(s, st);
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
    case 512: prepare_streamed_kernel<512><<<blocks, threads, 0, st>>>(planes, k_half, kp); break;
    default:
      if (generic_size(m.H)) return launch_prepare_generic_spectrum(m, n_sols, k_half, kp, st);
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace lgx
