// Streamed step for square 2D worlds whose side is even and factors into 2,
// 3, 5 and 7 without being a power of two (leniax worlds of side 48, 72, 96,
// 112, ...).  Same data flow as the power-of-two streamed engine:
//
//   rows forward  : per (world, channel, packed row r) the complex row
//                   row(2r) + i row(2r+1) -> its N-point FFT -> spec
//   column conv   : per (world, channel, column pair c): the column spectra
//                   X[n][c], n < N, unpacked from packed rows (c and N - c),
//                   N-point FFT over n, then per kernel reading the channel:
//                   x prepared spectrum, inverse FFT -> prod (column 0 also
//                   carries column N/2: both are real after the inverse)
//   rows inverse  : per (world, packed row r): for every kernel, the packed
//                   row's full spectrum rebuilt from prod (Hermitian
//                   extension), inverse FFT -> potential rows 2r, 2r+1,
//                   growth, weighted field per channel (core.py:163-242),
//                   state update (core.py:245-319), raw statistics moments
//   reduce        : the power-of-two engine's reducer
//
// Each line transform is a mixed-radix Stockham FFT (radices 4, 2, 3, 5, 7,
// self-sorting, ping-pong between two shared buffers) run by a whole block,
// one stage per barrier; the row passes transform several packed rows per
// block (gen_lines).  Growth uses leniax's operation order (growth_fn).
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "engine.h"
#include "fft.cuh"
#include "fft_mixed.cuh"

namespace lgx {
namespace {

constexpr int kGT = 128;  // threads per block
// Packed rows per block of the row passes: the largest of 8, 4, 2, 1 that
// divides N/2 with at most 1024 points in flight.
__host__ __device__ inline int gen_lines(int N) {
  for (int nl = 8; nl > 1; nl >>= 1)
    if ((N / 2) % nl == 0 && nl * N <= 1024) return nl;
  return 1;
}

struct GTab {  // per-plan kernel table, passed by value
  int C, K, max_k, mean, state_fn, dt_mode;
  int cin[kMaxKernels];
  int slot[kMaxKernels];
  int gf[kMaxKernels];
};

// ------------------------------------------------------------ rows forward
__global__ void __launch_bounds__(kGT) gen_row_fwd_kernel(GPlan p, const float* __restrict__ state,
                                                          float2* __restrict__ spec) {
  extern __shared__ __align__(16) float2 gsm[];
  const int N = p.n, H = N / 2, NL = gen_lines(N), BPP = H / NL;
  float2* tw = gsm;
  float2* A = tw + N;
  float2* B = A + NL * N;
  const long plane = blockIdx.x / BPP;
  const int r0 = (blockIdx.x % BPP) * NL;  // packed rows r0 .. r0 + NL - 1: state rows 2 r0 .. 2 r0 + 2 NL - 1
  fill_twiddles(tw, N);
  const float* src = state + (size_t)plane * N * N + (size_t)(2 * r0) * N;
  for (int i = threadIdx.x; i < NL * N; i += blockDim.x) {
    const int l = i / N, x = i - l * N;
    A[i] = make_float2(src[(size_t)(2 * l) * N + x], src[(size_t)(2 * l + 1) * N + x]);
  }
  __syncthreads();
  const float2* res = fft_line<false>(A, B, p, tw, NL);
  float2* dst = spec + ((size_t)plane * H + r0) * N;  // NL consecutive rows
  for (int i = threadIdx.x; i < NL * N; i += blockDim.x) dst[i] = res[i];
}

// ------------------------------------------------------------ column conv
// prod[(world K + k) H + r][c] (float4) holds (P[2r][c], P[2r+1][c]) for
// 0 < c < N/2 and, at c = 0, (P[2r][0] + i P[2r][N/2], P[2r+1][0] + i P[2r+1][N/2]).
__global__ void __launch_bounds__(kGT) gen_col_conv_kernel(GPlan p, int n_worlds, int n_init, GTab tab,
                                                           const float2* __restrict__ spec,
                                                           const float2* __restrict__ kp, long kp_sol_stride,
                                                           float2* __restrict__ prod) {
  extern __shared__ __align__(16) float2 gsm[];
  const int N = p.n, H = N / 2, KP = N / 2 + 2;
  float2* tw = gsm;
  float2* F0 = tw + N;   // forward spectrum of column c
  float2* FN = F0 + N;   // forward spectrum of column N/2 (block c = 0)
  float2* P0 = FN + N;   // inverse of column 0 (block c = 0)
  float2* A = P0 + N;
  float2* B = A + N;
  const int plane = blockIdx.x / H, c = blockIdx.x % H;
  if (plane >= n_worlds * tab.C) return;
  const int n = plane / tab.C, ch = plane % tab.C, sol = n / n_init;
  fill_twiddles(tw, N);
  const float2* sp = spec + (size_t)plane * H * N;
  // column spectra X[2r][cc], X[2r+1][cc] from packed rows (slots cc and N - cc)
  auto load_column = [&](int cc) {
    for (int rr = threadIdx.x; rr < H; rr += blockDim.x) {
      const float2 z1 = sp[(size_t)rr * N + cc], z2 = sp[(size_t)rr * N + (N - cc) % N];
      A[2 * rr] = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
      const float2 d = make_float2(z1.x - z2.x, z1.y + z2.y);  // z1 - conj(z2) = 2i X[2r+1]
      A[2 * rr + 1] = make_float2(0.5f * d.y, -0.5f * d.x);
    }
    __syncthreads();
  };
  load_column(c);
  {
    const float2* f = fft_line<false>(A, B, p, tw);
    for (int ky = threadIdx.x; ky < N; ky += blockDim.x) F0[ky] = f[ky];
  }
  if (c == 0) {
    __syncthreads();
    load_column(H);
    const float2* f = fft_line<false>(A, B, p, tw);
    for (int ky = threadIdx.x; ky < N; ky += blockDim.x) FN[ky] = f[ky];
  }
  __syncthreads();
  float4* pd4 = reinterpret_cast<float4*>(prod);
  for (int k = 0; k < tab.K; ++k) {
    if (tab.cin[k] != ch) continue;
    const float2* kk = kp + sol * kp_sol_stride + (size_t)(ch * tab.max_k + tab.slot[k]) * N * KP;
    for (int ky = threadIdx.x; ky < N; ky += blockDim.x) A[ky] = cmul(F0[ky], kk[(size_t)ky * KP + c]);
    __syncthreads();
    const float2* pc = fft_line<true>(A, B, p, tw);
    float4* dst = pd4 + (((size_t)n * tab.K + k) * H) * H;
    if (c != 0) {
      for (int rr = threadIdx.x; rr < H; rr += blockDim.x)
        dst[(size_t)rr * H + c] = make_float4(pc[2 * rr].x, pc[2 * rr].y, pc[2 * rr + 1].x, pc[2 * rr + 1].y);
    } else {
      for (int x = threadIdx.x; x < N; x += blockDim.x) P0[x] = pc[x];
      __syncthreads();
      for (int ky = threadIdx.x; ky < N; ky += blockDim.x) A[ky] = cmul(FN[ky], kk[(size_t)ky * KP + H]);
      __syncthreads();
      const float2* pn = fft_line<true>(A, B, p, tw);
      for (int rr = threadIdx.x; rr < H; rr += blockDim.x)
        dst[(size_t)rr * H] = make_float4(P0[2 * rr].x, pn[2 * rr].x, P0[2 * rr + 1].x, pn[2 * rr + 1].x);
    }
    __syncthreads();  // A / B / P0 free for the next kernel
  }
}

// ------------------------------------------------------------ rows inverse
// One block per (world, NL consecutive packed rows).
__global__ void __launch_bounds__(kGT) gen_row_inv_kernel(
    GPlan p, int n_worlds, int n_init, GTab tab, const float2* __restrict__ prod, const float* __restrict__ gfp,
    long gf_sol_stride, const float* __restrict__ wts, long w_sol_stride, const float* __restrict__ dtp,
    const float* __restrict__ state, float* __restrict__ state_out, float* __restrict__ field_out,
    float* __restrict__ pot_out, const int* __restrict__ shift, float* __restrict__ partial) {
  extern __shared__ __align__(16) float2 gsm[];
  constexpr int NWARPS = kGT / 32, RAWS_MAX = RAW_CM + kMaxChannels;
  const int N = p.n, H = N / 2, NL = gen_lines(N), BPW = H / NL;
  float2* tw = gsm;
  float2* A = tw + N;
  float2* B = A + NL * N;
  float* fld = reinterpret_cast<float*>(B + NL * N);  // [NL][2N] field of the current channel, rows 2r, 2r+1
  float* red = fld + 2 * NL * N;                      // [warps][RAWS_MAX]
  const int n = blockIdx.x / BPW, r0 = (blockIdx.x % BPW) * NL;
  if (n >= n_worlds) return;
  const int sol = n / n_init, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int C = tab.C, K = tab.K;
  const float* gf = gfp + sol * gf_sol_stride;
  const float* wt = wts + sol * w_sol_stride;
  fill_twiddles(tw, N);
  float dt;
  if (tab.dt_mode == 0) dt = __ldg(dtp);
  else if (tab.dt_mode == 1) dt = __ldg(dtp + n);
  else dt = 1.f / __ldg(dtp + sol);
  const int sy = shift[3 * n], sx = shift[3 * n + 1];
  for (int i = threadIdx.x; i < NWARPS * RAWS_MAX; i += blockDim.x) red[i] = 0.f;
  float cpot = 0.f, m00 = 0.f, g00 = 0.f, cmass = 0.f, cgrow = 0.f, mxy = 0.f, mxx = 0.f, gxy = 0.f, gxx = 0.f,
        m2y = 0.f, m2x = 0.f;
  bool border = false;
  unsigned long long counted = 0ull;
  const float4* pr = reinterpret_cast<const float4*>(prod);

  // kernel k's potential rows into the returned buffer: element l N + x holds
  // (row 2(r0+l), row 2(r0+l)+1) at column x
  auto potential = [&](int k) -> const float2* {
    for (int i = threadIdx.x; i < NL * N; i += blockDim.x) {
      const int l = i / N, kx = i - l * N;
      const float4* row = pr + (((size_t)n * K + k) * H + r0 + l) * H;
      float2 z;
      if (kx == 0 || kx == H) {
        const float4 q = row[0];  // (P[2r][0] + i P[2r][N/2], P[2r+1][0] + i P[2r+1][N/2])
        z = kx == 0 ? make_float2(q.x, q.z) : make_float2(q.y, q.w);
      } else if (kx < H) {
        const float4 q = row[kx];  // Z = P[2r][kx] + i P[2r+1][kx]
        z = make_float2(q.x - q.w, q.y + q.z);
      } else {
        const float4 q = row[N - kx];  // conj(P[2r][N-kx]) + i conj(P[2r+1][N-kx])
        z = make_float2(q.x + q.w, q.z - q.y);
      }
      A[i] = z;
    }
    __syncthreads();
    return fft_line<true>(A, B, p, tw, NL);
  };
  auto count = [&](int k, const float2* pot) {
    for (int i = threadIdx.x; i < NL * N; i += blockDim.x) {
      const int l = i / N, x = i - l * N;
      const float pa = pot[i].x, pb = pot[i].y;
      cpot += (pa > kEps ? 1.f : 0.f) + (pb > kEps ? 1.f : 0.f);
      if (pot_out) {
        float* po = pot_out + ((size_t)n * K + k) * N * N + (size_t)(2 * (r0 + l)) * N;
        po[x] = pa;
        po[N + x] = pb;
      }
    }
  };

  for (int co = 0; co < C; ++co) {
    float wsum = 0.f;
    for (int k = 0; k < K; ++k) wsum += __ldg(wt + co * K + k);
    for (int i = threadIdx.x; i < 2 * NL * N; i += blockDim.x) fld[i] = 0.f;
    __syncthreads();
    for (int k = 0; k < K; ++k) {
      const float wk = __ldg(wt + co * K + k);
      if (wk == 0.f) continue;
      const float2* pot = potential(k);
      if (!((counted >> k) & 1ull)) count(k, pot);
      counted |= 1ull << k;
      const float m = __ldg(gf + 2 * k), s = __ldg(gf + 2 * k + 1);
      const int id = tab.gf[k];
      for (int i = threadIdx.x; i < NL * N; i += blockDim.x) {
        const int l = i / N, x = i - l * N;
        float* fl = fld + (size_t)l * 2 * N;
        fl[x] = fmaf(wk, growth_fn(id, pot[i].x, m, s), fl[x]);
        fl[N + x] = fmaf(wk, growth_fn(id, pot[i].y, m, s), fl[N + x]);
      }
      __syncthreads();
    }
    // field, state update and moments of channel co (statistics.py:64-100)
    float cm = 0.f;
    for (int i = threadIdx.x; i < NL * N; i += blockDim.x) {
      const int l = i / N, x = i - l * N, r = r0 + l;
      const size_t base = ((size_t)n * C + co) * N * N + (size_t)(2 * r) * N;
      const float cx = (float)(pmod(x - sx, N) - N / 2);
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        float f = fld[(size_t)l * 2 * N + e * N + x];
        if (tab.mean) f = f / wsum;
        const float sv = __ldg(state + base + (size_t)e * N + x);
        state_out[base + (size_t)e * N + x] = state_fn(tab.state_fn, sv, f, dt);
        if (field_out) field_out[base + (size_t)e * N + x] = f;
        const int y = 2 * r + e;
        const float fp = fmaxf(f, 0.f), cy = (float)(pmod(y - sy, N) - N / 2);
        m00 += sv;
        g00 += fp;
        cm += sv;
        mxy = fmaf(cy, sv, mxy);
        mxx = fmaf(cx, sv, mxx);
        gxy = fmaf(cy, fp, gxy);
        gxx = fmaf(cx, fp, gxx);
        m2y = fmaf(cy * cy, sv, m2y);
        m2x = fmaf(cx * cx, sv, m2x);
        const bool live = sv > kEps;
        cmass += live ? 1.f : 0.f;
        cgrow += fp > kEps ? 1.f : 0.f;
        border |= live && (x == 0 || x == N - 1 || y == 0 || y == N - 1);
      }
    }
    cm = warp_sum(cm);
    if (lane == 0) red[wid * RAWS_MAX + RAW_CM + co] = cm;
    __syncthreads();
  }
  for (int k = 0; k < K; ++k)  // kernels that feed no channel: their potential still counts
    if (!((counted >> k) & 1ull)) {
      const float2* pot = potential(k);
      count(k, pot);
      __syncthreads();
    }
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
    rd[RAW_GX + 0] = accm[7];
    rd[RAW_GX + 1] = accm[8];
    rd[RAW_MX2 + 0] = accm[9];
    rd[RAW_MX2 + 1] = accm[10];
    rd[RAW_BORDER] = anyb ? 1.f : 0.f;
  }
  __syncthreads();
  const int RAWS = raw_stride(C);
  if (threadIdx.x < RAWS) {
    float sum = 0.f;
    for (int w = 0; w < NWARPS; ++w) sum += red[w * RAWS_MAX + threadIdx.x];
    if (threadIdx.x == RAW_BORDER) sum = sum > 0.f ? 1.f : 0.f;
    partial[((size_t)n * BPW + blockIdx.x % BPW) * RAWS + threadIdx.x] = sum;
  }
}

// prepared spectra: k_half [planes][N][N/2+1] scaled by 1/N^2, row pitch N/2+2
__global__ void gen_prepare_kernel(long planes, int N, const float2* __restrict__ kh, float2* __restrict__ kp) {
  const int HW = N / 2 + 1, KP = N / 2 + 2;
  const float scale = 1.f / ((float)N * (float)N);
  const long total = planes * N * KP;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % KP);
    const long row = i / KP;  // plane * N + ky
    float2 o = make_float2(0.f, 0.f);
    if (c < HW) {
      const float2 k = kh[row * HW + c];
      o = make_float2(k.x * scale, k.y * scale);
    }
    kp[i] = o;
  }
}

}  // namespace

bool generic_size(int n) {
  if (n < 8 || n > kGMaxN || (n & 1) || (n & (n - 1)) == 0) return false;
  return make_plan(n).stages > 0;
}

cudaError_t launch_prepare_generic_spectrum(const Model& m, int n_sols, const float2* k_half, float2* kp,
                                            cudaStream_t st) {
  const long planes = (long)n_sols * m.C * m.max_k;
  const long total = planes * m.H * (m.W / 2 + 2);
  const int threads = 256;
  const int blocks = (int)std::min<long>((total + threads - 1) / threads, 8192);
  gen_prepare_kernel<<<blocks, threads, 0, st>>>(planes, m.H, k_half, kp);
  return cudaGetLastError();
}

cudaError_t launch_generic_step(const StreamedStep& s, cudaStream_t st) {
  const Model& m = *s.m;
  const int N = m.H, H = N / 2;
  const GPlan p = make_plan(N);
  if (p.stages == 0 || m.H != m.W) return cudaErrorInvalidValue;
  GTab tab;
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
  const long planes = (long)s.n_worlds * m.C;
  const int NL = gen_lines(N), BPW = H / NL;
  const size_t sm_fwd = (size_t)(1 + 2 * NL) * N * sizeof(float2);
  const size_t sm_col = (size_t)6 * N * sizeof(float2);
  const size_t sm_inv = (size_t)(1 + 2 * NL) * N * sizeof(float2) + (size_t)2 * NL * N * sizeof(float) +
                        (size_t)(kGT / 32) * (RAW_CM + kMaxChannels) * sizeof(float);
  // the row spectra are recomputed every step (no fused next-step transform here)
  gen_row_fwd_kernel<<<(unsigned)(planes * BPW), kGT, sm_fwd, st>>>(p, s.state, s.spec);
  gen_col_conv_kernel<<<(unsigned)(planes * H), kGT, sm_col, st>>>(p, s.n_worlds, s.n_init, tab, s.spec, s.kp,
                                                                     s.kp_sol_stride, s.prod);
  gen_row_inv_kernel<<<(unsigned)((long)s.n_worlds * BPW), kGT, sm_inv, st>>>(
      p, s.n_worlds, s.n_init, tab, s.prod, s.gf, s.gf_sol_stride, s.w, s.w_sol_stride, s.dt, s.state, s.state_out,
      s.field_out, s.pot_out, s.shift, s.partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_streamed_reduce(s, BPW, st);
}

int generic_blocks_per_world(int N) { return (N / 2) / gen_lines(N); }

}  // namespace lgx
