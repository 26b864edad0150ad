// Mixed-radix line FFTs in shared memory (radices 4, 2, 3, 5, 7): a
// self-sorting Stockham transform run by a whole block, one stage per
// barrier, ping-ponging between two shared buffers.  Used by the even-side 2D
// engine (generic.cu) and the general N-D engine (nd.cu).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "fft.cuh"

namespace lgx {

// n / d for 0 <= n < 2^31 by a multiply-high and a shift (the round-up
// method of Granlund and Montgomery, "Division by invariant integers using
// multiplication", 1994): s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1,
// n / d = (umulhi(n, m) + n) >> s.
struct FastDivU {
  unsigned m, s;
  __device__ __forceinline__ int div(int n) const {
    return (int)((__umulhi((unsigned)n, m) + (unsigned)n) >> s);
  }
};
inline FastDivU make_fastdiv(unsigned d) {
  FastDivU f;
  f.s = 0;
  while ((1ull << f.s) < d) ++f.s;
  f.m = (unsigned)(((1ull << 32) * ((1ull << f.s) - d)) / d + 1);
  return f;
}

constexpr int kGMaxStages = 12;
constexpr int kGMaxN = 512;

struct GPlan {  // radices of one N-point transform, passed by value
  int n, stages;
  int r[kGMaxStages];
};

// exp(-2 pi i m / L) in float: the octant reduction of cx_trig on exact
// integers, then sincospif of a reduced fraction (one rounding).
__device__ __forceinline__ float2 tw_entry(int m, int L) {
  int n = m % L;
  if (n < 0) n += L;
  float ss = 1.f, cs = 1.f;
  if (2 * n > L) {
    n = L - n;
    ss = -1.f;
  }
  int mm = n, D = L;
  if (4 * n > L) {
    mm = L - 2 * n;
    D = 2 * L;
    cs = -1.f;
  }
  float c, s;
  if (8 * mm > D) {  // the complementary angle pi/2 - a
    float sb, cb;
    sincospif((float)(D - 4 * mm) / (float)(2 * D), &sb, &cb);
    c = sb;
    s = cb;
  } else {
    sincospif((float)(2 * mm) / (float)D, &s, &c);
  }
  return make_float2(cs * c, -(ss * s));
}

__device__ __forceinline__ void fill_twiddles(float2* tw, int N) {
  for (int j = threadIdx.x; j < N; j += blockDim.x) tw[j] = tw_entry(j, N);
}

// One Stockham stage of radix R: butterfly j reads in[j + q N/R], twiddles
// by W_{Ns R}^{q (j mod Ns)}, takes the R-point DFT and writes
// out[(j / Ns) Ns R + (j mod Ns) + t Ns].
// Point i of the line is in[i * pitch] / out[i * pitch] (pitch 1: a
// contiguous line; the row pitch: a column of a row-major tile).
template <bool INV, int R>
__device__ __forceinline__ void stockham_butterfly(const float2* in, float2* out, int nb, int Ns, int j, int k,
                                                   int stride, const float2* tw, int pitch = 1) {
  float2 v[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const float2 x = in[(j + q * nb) * pitch];
    const float2 w = tw[q * k * stride];  // q k stride < N
    v[q] = q == 0 ? x : (INV ? cmulc(x, w) : cmul(x, w));
  }
  float2 y[R];
  if constexpr (R == 2) {
    y[0] = cadd(v[0], v[1]);
    y[1] = csub(v[0], v[1]);
  } else if constexpr (R == 4) {
    // W_4 = -i forward, +i inverse: the products are swaps and sign flips
    const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    const float2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
    const float2 rot = INV ? make_float2(-d13.y, d13.x) : make_float2(d13.y, -d13.x);
    y[0] = cadd(s02, s13);
    y[1] = cadd(d02, rot);
    y[2] = csub(s02, s13);
    y[3] = csub(d02, rot);
  } else {
#pragma unroll
    for (int t = 0; t < R; ++t) {
      float2 acc = v[0];
#pragma unroll
      for (int q = 1; q < R; ++q) {
        const float2 w = tw[((q * t) % R) * nb];  // W_R^{q t} = W_N^{(q t mod R) N / R}
        acc = cadd(acc, INV ? cmulc(v[q], w) : cmul(v[q], w));
      }
      y[t] = acc;
    }
  }
  const int base = (j - k) * R + k;  // (j / Ns) Ns R + k
#pragma unroll
  for (int t = 0; t < R; ++t) out[(base + t * Ns) * pitch] = y[t];
}

template <bool INV, int R>
__device__ __forceinline__ void stockham_stage(const float2* in_all, float2* out_all, int N, int Ns, const float2* tw,
                                               int nl) {
  const int nb = N / R, stride = N / (Ns * R);
  for (int jj = threadIdx.x; jj < nl * nb; jj += blockDim.x) {
    const int line = jj / nb, j = jj - line * nb;  // lines of N points, contiguous
    stockham_butterfly<INV, R>(in_all + line * N, out_all + line * N, nb, Ns, j, j % Ns, stride, tw);
  }
}

// The same stage over ncols columns of a row-major tile (N rows, row pitch
// `pitch`): consecutive threads take consecutive columns, so every access of
// a warp is to consecutive addresses.  cdiv divides by ncols.
template <bool INV, int R>
__device__ __forceinline__ void stockham_stage_cols(const float2* in_all, float2* out_all, int N, int Ns,
                                                    const float2* tw, int ncols, int pitch, const FastDivU& cdiv) {
  const int nb = N / R, stride = N / (Ns * R);
  for (int jj = threadIdx.x; jj < ncols * nb; jj += blockDim.x) {
    const int j = cdiv.div(jj), col = jj - j * ncols;
    stockham_butterfly<INV, R>(in_all + col, out_all + col, nb, Ns, j, j % Ns, stride, tw, pitch);
  }
}

// N-point FFTs of the ncols columns of a row-major tile in a (N rows, row
// pitch `pitch`), into a or b (returned); unnormalised for INV.  Every thread
// of the block calls it; it ends on a barrier.
template <bool INV>
__device__ __forceinline__ float2* fft_cols(float2* a, float2* b, const GPlan& p, const float2* tw, int ncols,
                                            int pitch, const FastDivU& cdiv) {
  const int N = p.n;
  float2* in = a;
  float2* out = b;
  int Ns = 1;
  for (int s = 0; s < p.stages; ++s) {
    switch (p.r[s]) {
      case 2: stockham_stage_cols<INV, 2>(in, out, N, Ns, tw, ncols, pitch, cdiv); break;
      case 3: stockham_stage_cols<INV, 3>(in, out, N, Ns, tw, ncols, pitch, cdiv); break;
      case 4: stockham_stage_cols<INV, 4>(in, out, N, Ns, tw, ncols, pitch, cdiv); break;
      case 5: stockham_stage_cols<INV, 5>(in, out, N, Ns, tw, ncols, pitch, cdiv); break;
      default: stockham_stage_cols<INV, 7>(in, out, N, Ns, tw, ncols, pitch, cdiv); break;
    }
    __syncthreads();
    Ns *= p.r[s];
    float2* t = in;
    in = out;
    out = t;
  }
  return in;
}

// N-point FFTs of the block's nl contiguous lines in a into a or b
// (returned); unnormalised for INV.  Every thread of the block calls it; it
// ends on a barrier.
template <bool INV>
__device__ __forceinline__ float2* fft_line(float2* a, float2* b, const GPlan& p, const float2* tw, int nl = 1) {
  const int N = p.n;
  float2* in = a;
  float2* out = b;
  int Ns = 1;
  for (int s = 0; s < p.stages; ++s) {
    const int R = p.r[s];
    switch (R) {
      case 2: stockham_stage<INV, 2>(in, out, N, Ns, tw, nl); break;
      case 3: stockham_stage<INV, 3>(in, out, N, Ns, tw, nl); break;
      case 4: stockham_stage<INV, 4>(in, out, N, Ns, tw, nl); break;
      case 5: stockham_stage<INV, 5>(in, out, N, Ns, tw, nl); break;
      default: stockham_stage<INV, 7>(in, out, N, Ns, tw, nl); break;
    }
    __syncthreads();
    Ns *= R;
    float2* t = in;
    in = out;
    out = t;
  }
  return in;
}

// Radices of an N-point transform (0 stages when N has a prime factor above 7).
inline GPlan make_plan(int N) {
  GPlan p;
  p.n = N;
  p.stages = 0;
  int n = N;
  while (n % 4 == 0 && p.stages < kGMaxStages) {
    p.r[p.stages++] = 4;
    n /= 4;
  }
  while (n % 2 == 0 && p.stages < kGMaxStages) {
    p.r[p.stages++] = 2;
    n /= 2;
  }
  for (int f : {3, 5, 7})
    while (n % f == 0 && p.stages < kGMaxStages) {
      p.r[p.stages++] = f;
      n /= f;
    }
  if (n != 1) p.stages = 0;
  return p;
}

}  // namespace lgx
