// Register/shared-memory FFT building blocks for the Lenia step kernels (sm_103a).
//
// A complex N-point transform (N = G * P, powers of two) is computed by a
// "group" of G consecutive lanes of one warp, each lane holding P points in
// registers.  Two Cooley-Tukey factorisations are used:
//
//  * standard  : input  n = t + G*n2   (lane t owns a stride-G comb)
//                stage 1: P-point DFT over n2 in registers, twiddle W_N^(t*k2),
//                exchange through the group's shared scratch, stage 2: G-point
//                DFTs over t.  Output k = k2 + P*k1.
//  * mirrored  : input  n = n1 + P*n2  (lane owns a set of n1 rows)
//                stage 1: G-point DFTs over n2, twiddle W_N^(n1*k2), exchange,
//                stage 2: P-point DFT over n1.  Output k = t + G*k1, i.e. the
//                standard factorisation's input comb.
//
// Chaining a standard forward with a mirrored inverse (or the reverse) keeps a
// lane's data on the same index comb, so world states can stay in registers
// across Euler steps.  Scratch layouts are padded / permuted so every 64-bit
// shared access of an exchange is bank-conflict free (checked for G in {4,8,16}).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include <utility>

namespace lgx {

// ---------------------------------------------------------------- utilities
template <int I>
using ic = std::integral_constant<int, I>;

template <class F, int... Is>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, Is...>) {
  (f(ic<Is>{}), ...);
}
// Compile-time loop: f(ic<0>{}), ..., f(ic<N-1>{}).
template <int N, class F>
__device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// Complex add/sub on Blackwell's packed FP32x2 pipe (one instruction per
// complex value; a - b is fma(b, -1, a), exact to one rounding like a - b).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
// a + conj(b) and a - conj(b)
__device__ __forceinline__ float2 caddc(float2 a, float2 b) { return __ffma2_rn(b, make_float2(1.f, -1.f), a); }
__device__ __forceinline__ float2 csubc(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, 1.f), a); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// ------------------------------------------- compile-time twiddle constants
// cos/sin of 2*pi*k/L evaluated at compile time: exact octant reduction on the
// integers (k, L), then Taylor series on [0, pi/4] in double precision.
__host__ __device__ constexpr double cx_sin_series(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int i = 1; i < 14; ++i) {
    term *= -x2 / double((2 * i) * (2 * i + 1));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double cx_cos_series(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int i = 1; i < 14; ++i) {
    term *= -x2 / double((2 * i - 1) * (2 * i));
    sum += term;
  }
  return sum;
}
constexpr double kTwoPi = 6.283185307179586476925286766559;
// returns cos(2*pi*k/L) (want_sin=false) or sin(2*pi*k/L) (want_sin=true)
__host__ __device__ constexpr double cx_trig(long k, long L, bool want_sin) {
  long n = ((k % L) + L) % L;
  double ssign = 1.0, csign = 1.0;
  if (2 * n > L) {  // angle in (pi, 2pi): 2pi - a keeps cos, flips sin
    n = L - n;
    ssign = -1.0;
  }
  long m = n, D = L;  // angle = 2*pi*m/D
  if (4 * n > L) {    // angle in (pi/2, pi]: pi - a flips cos, keeps sin
    m = L - 2 * n;
    D = 2 * L;
    csign = -1.0;
  }
  double a = kTwoPi * double(m) / double(D);  // [0, pi/2]
  double c = 0.0, s = 0.0;
  if (8 * m > D) {  // (pi/4, pi/2]: use the complementary angle
    double b = kTwoPi / 4.0 - a;
    c = cx_sin_series(b);
    s = cx_cos_series(b);
  } else {
    c = cx_cos_series(a);
    s = cx_sin_series(a);
  }
  return want_sin ? ssign * s : csign * c;
}

// x * W_L^k (forward, W = exp(-2*pi*i/L)) or x * W_L^-k (inverse)
template <int K, int L, bool INV>
__device__ __forceinline__ float2 tw_mul(float2 x) {
  constexpr int k = ((K % L) + L) % L;
  if constexpr (k == 0) {
    return x;
  } else if constexpr (4 * k == L) {  // -i (fwd) / +i (inv)
    return INV ? make_float2(-x.y, x.x) : make_float2(x.y, -x.x);
  } else if constexpr (2 * k == L) {
    return make_float2(-x.x, -x.y);
  } else if constexpr (4 * k == 3 * L) {  // +i (fwd) / -i (inv)
    return INV ? make_float2(x.y, -x.x) : make_float2(-x.y, x.x);
  } else {
    constexpr float c = (float)cx_trig(k, L, false);
    constexpr float s0 = (float)cx_trig(k, L, true);
    constexpr float s = INV ? s0 : -s0;
    return make_float2(fmaf(x.x, c, -x.y * s), fmaf(x.x, s, x.y * c));
  }
}

// In-register DFT of L points, natural order in and out (radix-2 DIT).
template <int L, bool INV>
__device__ __forceinline__ void fft_reg(float2 (&v)[L]) {
  if constexpr (L == 1) {
  } else if constexpr (L == 2) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else {
    float2 e[L / 2], o[L / 2];
#pragma unroll
    for (int i = 0; i < L / 2; ++i) {
      e[i] = v[2 * i];
      o[i] = v[2 * i + 1];
    }
    fft_reg<L / 2, INV>(e);
    fft_reg<L / 2, INV>(o);
    sfor<L / 2>([&](auto I) {
      constexpr int k = decltype(I)::value;
      float2 t = tw_mul<k, L, INV>(o[k]);
      v[k] = cadd(e[k], t);
      v[k + L / 2] = csub(e[k], t);
    });
  }
}

// ------------------------------------------------------------- geometry
// One square-axis FFT geometry: N points, G lanes per transform, P points per lane.
template <int N_, int G_>
struct Geo {
  static constexpr int N = N_;
  static constexpr int G = G_;
  static constexpr int P = N / G;
  static constexpr int Q = P / G;         // comb members per lane after an exchange
  static constexpr int SCR = N + G;       // float2 per group scratch (padded)
  static_assert(G == 2 || G == 4 || G == 8 || G == 16, "group size");
  // Q even: the pair-preserving exchanges (a lane holds rows / columns in
  // pairs); Q == 1: one index per lane (the "identity" sets below)
  static_assert(P % G == 0 && (Q == 1 || Q % 2 == 0), "need P/G even, or P == G");
};

// Per-thread twiddle tables kept in shared memory, one N-entry table per
// factorisation.  Layouts are [slot][t] so a warp reads consecutive entries.
//   std   : tw[k2*G + t]              = W_N^(t*k2),             k2 < P
//   colf  : tw[(q*G + k2)*G + t]      = W_N^(n1c(t,q)*k2),      q < Q, k2 < G
//   rowi  : tw[(q*G + k2)*G + t]      = W_N^(n1r(t,q)*k2),      q < Q, k2 < G
// where n1c / n1r are the lane's row sets of the column-forward (adjacent
// pairs) and row-inverse (mirror pairs) mirrored factorisations.
// With Q == 1 (P == G) both sets are the identity: lane t holds n1 = t.
template <class GE>
__device__ __forceinline__ int n1_pairs(int t, int q) {  // q-th n1 of lane t: {2m, 2m+1}, m = t + G*(q/2)
  if constexpr (GE::Q == 1) return t;
  int m = t + GE::G * (q >> 1);
  return 2 * m + (q & 1);
}
template <class GE>
__device__ __forceinline__ int n1_mirror(int t, int q) {  // {m, P-m} (m>0) or {0, P/2} (m==0), m = t + G*(q/2)
  if constexpr (GE::Q == 1) return t;
  int m = t + GE::G * (q >> 1);
  if (m == 0) return (q & 1) ? GE::P / 2 : 0;
  return (q & 1) ? GE::P - m : m;
}

// The three tables of every (N, G), evaluated at compile time with the
// octant-reduced series above (exact zeros and ones at the quarter points,
// like sincospi) and stored once in global memory; blocks copy them into
// shared memory at start.  Evaluating them per block with double-precision
// sincospi cost more than the transforms in short-lived blocks: the FP64
// pipe of this part is narrow.
struct alignas(8) TwEntry {
  float x, y;
};
template <int N, int G>
struct TwiddleTables {
  static constexpr int P = N / G, Q = P / G;
  TwEntry v[3 * N];
  static constexpr TwEntry entry(int m) {  // W_N^m = exp(-2 pi i m / N)
    return TwEntry{(float)cx_trig(m, N, false), (float)(-cx_trig(m, N, true))};
  }
  static constexpr int pairs(int t, int q) {  // n1_pairs
    if (Q == 1) return t;
    const int m = t + G * (q >> 1);
    return 2 * m + (q & 1);
  }
  static constexpr int mirror(int t, int q) {  // n1_mirror
    if (Q == 1) return t;
    const int m = t + G * (q >> 1);
    if (m == 0) return (q & 1) ? P / 2 : 0;
    return (q & 1) ? P - m : m;
  }
  constexpr TwiddleTables() : v{} {
    for (int i = 0; i < N; ++i) {
      const int t = i % G, k2 = i / G, kk = (i / G) % G, q = i / (G * G);
      v[i] = entry((t * k2) % N);
      v[N + i] = entry((pairs(t, q) * kk) % N);
      v[2 * N + i] = entry((mirror(t, q) * kk) % N);
    }
  }
};
template <int N, int G>
__device__ const TwiddleTables<N, G> kTwiddles{};

template <class GE>
__device__ void init_twiddles(float2* tw_std, float2* tw_colf, float2* tw_rowi, int tid, int nthreads) {
  constexpr int N = GE::N;
  const float2* src = reinterpret_cast<const float2*>(kTwiddles<GE::N, GE::G>.v);
  for (int i = tid; i < N; i += nthreads) {
    tw_std[i] = __ldg(src + i);
    tw_colf[i] = __ldg(src + N + i);
    tw_rowi[i] = __ldg(src + 2 * N + i);
  }
}

// ---------------------------------------------------- standard factorisation
// v[n2] holds x[t + G*n2].  On return u[q][k1] holds X[k2 + P*k1] with
// k2 = kset(t, q); kset is strided {t + G*q} (PAIRS=false) or adjacent pairs
// {2m, 2m+1}, m = t + G*(q/2) (PAIRS=true).  scr: the group's scratch (SCR).
template <class GE, bool INV, bool PAIRS>
__device__ __forceinline__ void fft_standard(float2 (&v)[GE::P], float2 (&u)[GE::Q][GE::G], float2* scr,
                                             const float2* tw_std, int t, unsigned gmask) {
  constexpr int G = GE::G, P = GE::P, Q = GE::Q;
  static_assert(!PAIRS || Q % 2 == 0, "the pair output sets need Q even");
  fft_reg<P, INV>(v);
#pragma unroll
  for (int k2 = 1; k2 < P; ++k2) {
    float2 w = tw_std[k2 * G + t];
    v[k2] = INV ? cmulc(v[k2], w) : cmul(v[k2], w);
  }
  // write Y[t][k2] at t*(P+1) + pi(k2)
#pragma unroll
  for (int k2 = 0; k2 < P; ++k2) {
    int pk = PAIRS ? ((k2 >> 1) + (k2 & 1) * (P / 2)) : k2;
    scr[t * (P + 1) + pk] = v[k2];
  }
  __syncwarp(gmask);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    int k2 = PAIRS ? (2 * (t + G * (q >> 1)) + (q & 1)) : (t + G * q);
    int pk = PAIRS ? ((k2 >> 1) + (k2 & 1) * (P / 2)) : k2;
#pragma unroll
    for (int n1 = 0; n1 < G; ++n1) u[q][n1] = scr[n1 * (P + 1) + pk];
  }
  __syncwarp(gmask);
#pragma unroll
  for (int q = 0; q < Q; ++q) fft_reg<G, INV>(u[q]);
}

// ---------------------------------------------------- mirrored factorisation
// v[q][n2] holds x[n1(t,q) + P*n2] (n1 from the pairs or mirror set, MIRROR
// selects).  On return w[k1] holds X[t + G*k1].
template <class GE, bool INV, bool MIRROR>
__device__ __forceinline__ void fft_mirrored(float2 (&v)[GE::Q][GE::G], float2 (&w)[GE::P], float2* scr,
                                             const float2* tw_tab, int t, unsigned gmask) {
  constexpr int G = GE::G, P = GE::P, Q = GE::Q;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    fft_reg<G, INV>(v[q]);
#pragma unroll
    for (int k2 = 1; k2 < G; ++k2) {
      float2 tw = tw_tab[(q * G + k2) * G + t];
      v[q][k2] = INV ? cmulc(v[q][k2], tw) : cmul(v[q][k2], tw);
    }
  }
  // write Y[n1][k2] at k2*(P+1) + pi(n1)
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    int n1 = MIRROR ? n1_mirror<GE>(t, q) : n1_pairs<GE>(t, q);
    int pn = (MIRROR || Q == 1) ? n1 : ((n1 >> 1) + (n1 & 1) * (P / 2));
#pragma unroll
    for (int k2 = 0; k2 < G; ++k2) scr[k2 * (P + 1) + pn] = v[q][k2];
  }
  __syncwarp(gmask);
#pragma unroll
  for (int n1 = 0; n1 < P; ++n1) {
    int pn = (MIRROR || Q == 1) ? n1 : ((n1 >> 1) + (n1 & 1) * (P / 2));
    w[n1] = scr[t * (P + 1) + pn];
  }
  __syncwarp(gmask);
  fft_reg<P, INV>(w);
}

// Pair-adjacent layout of a packed-row spectrum Z[0..N-1]: pair j (16 bytes)
// holds (Z[j], Z[N-j]) for 0 < j < N/2 and pair 0 holds (Z[0], Z[N/2]).  The
// column pass reads and writes whole pairs, and its tiles start on 16-byte
// boundaries, as TMA requires.  After the column pass, pair j of packed row r
// holds (column j at row 2r, column j at row 2r+1); pair 0 the DC and Nyquist
// columns packed as DC + i Nyquist.
template <int N>
__host__ __device__ __forceinline__ int pa_pos(int k) {
  return k == 0 ? 0 : (k == N / 2 ? 1 : (k < N / 2 ? 2 * k : 2 * (N - k) + 1));
}

// Row-inverse input of a packed row pair.  `pr` holds the N-point packed row r
// of a real 2D transform after the column pass: slot k < N/2 carries
// P[2r][k] and slot N - k carries P[2r+1][k] (P the half spectra of rows 2r
// and 2r+1; slots 0 and N/2 carry the DC / Nyquist columns packed together).
// Fills v[q][n2] = Z[n1 + P*n2] with n1 from the mirror set of lane t, where
// Z = P[2r] + i P[2r+1] over the full row, ready for
// fft_mirrored<GE, true, true>, whose output w[k1] is then
// (row 2r, row 2r+1) at x = t + G*k1.
template <class GE>
__device__ __forceinline__ void unpack_row_pair(const float2* pr, float2 (&v)[GE::Q][GE::G], int t) {
  constexpr int N = GE::N, G = GE::G, P = GE::P, Q = GE::Q;
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
}

// Row-inverse input of a packed row pair stored in the pair-adjacent layout:
// pair j (one 16-byte float4) holds (slot j, slot N - j) of the packed row,
// pair 0 holds (slot 0, slot N/2).  Same result as unpack_row_pair on the
// plain layout, with one 16-byte load per (slot k, slot N - k).
template <class GE>
__device__ __forceinline__ void unpack_row_pair_pa(const float2* pr, float2 (&v)[GE::Q][GE::G], int t) {
  constexpr int N = GE::N, G = GE::G, P = GE::P, Q = GE::Q;
  const float4* p4 = reinterpret_cast<const float4*>(pr);
#pragma unroll
  for (int jp = 0; jp < Q / 2; ++jp) {
    const int m = t + G * jp;
    if (m != 0) {
#pragma unroll
      for (int n2 = 0; n2 < G; ++n2) {
        const int kx = m + P * n2;
        // s1 = slot min(kx, N-kx), s2 = slot max(kx, N-kx)
        const float4 q = p4[n2 < G / 2 ? kx : N - kx];
        const float2 a = make_float2(q.x - q.w, q.y + q.z);  // s1 + i s2
        const float2 b = make_float2(q.x + q.w, q.z - q.y);  // conj(s1) + i conj(s2)
        if (n2 < G / 2) {
          v[2 * jp][n2] = a;
          v[2 * jp + 1][G - 1 - n2] = b;
        } else {
          v[2 * jp][n2] = b;
          v[2 * jp + 1][G - 1 - n2] = a;
        }
      }
    } else {
      const float4 q0 = p4[0];  // (slot 0, slot N/2)
      v[2 * jp][0] = make_float2(q0.x, q0.z);
      v[2 * jp][G / 2] = make_float2(q0.y, q0.w);
#pragma unroll
      for (int n2 = 1; n2 < G / 2; ++n2) {
        const float4 q = p4[P * n2];
        v[2 * jp][n2] = make_float2(q.x - q.w, q.y + q.z);
        v[2 * jp][G - n2] = make_float2(q.x + q.w, q.z - q.y);
      }
#pragma unroll
      for (int n2 = 0; n2 < G / 2; ++n2) {
        const float4 q = p4[P / 2 + P * n2];
        v[2 * jp + 1][n2] = make_float2(q.x - q.w, q.y + q.z);
        v[2 * jp + 1][G - 1 - n2] = make_float2(q.x + q.w, q.z - q.y);
      }
    }
  }
}

}  // namespace lgx
