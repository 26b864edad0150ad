// General N-D engine: any 2D or 3D torus whose sides factor into 2, 3, 5
// and 7 (odd, non-square and non-power-of-two sides included, e.g. 48^3),
// any number of channels and kernels -- the forward Euler step and its
// adjoint.  leniax's get_potential_fft transforms every world axis
// (core.py:74-87); here each axis is one pass of mixed-radix line FFTs over
// complex planes in HBM:
//
//   forward step : x pass (real state in), y pass, z pass   -> state spectra S
//                  S[c_in(k)] x prepared spectrum[k]           -> products P
//                  z, y, x inverse passes (real part out)      -> potentials u_k
//                  growth, weighted field, state update and the statistics
//                  moments per block (core.py:163-319, statistics.py:36-126)
//                  per-world reduction of the moments, carried torus shift
//   adjoint step : clip / state-function gradient, dL/df, dL/dg, growth
//                  derivative -> a_k = dL/du_k; forward passes of a_k and of
//                  the state; kernel gradient A_k conj(S) accumulated; the
//                  correlation sum_k A_k conj(K_k) per input channel through
//                  the inverse passes added to lambda; growth-parameter and
//                  weight gradients reduced per (world, kernel)
//
// A pass stages a tile of lines in shared memory (consecutive lines of the
// same group so that global loads and stores are coalesced), runs the
// Stockham transform of fft_mixed.cuh and writes the tile back in place.
// Spectra are full complex (no Hermitian packing), so odd sides need no
// special case.  This engine serves the worlds the specialised engines do not
// (resident: 2D 32..128 C = K = 1; streamed: square 2D; one world per CTA:
// 3D 32^3 / 64^3 C = K = 1) and every differentiated model beyond C = K = 1.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "fft_mixed.cuh"

namespace lgx {
namespace {

constexpr int kNT = 256;          // threads per block
constexpr int kNdMaxN = 4096;     // longest world axis (one 4096-point line per pass tile)
constexpr int kBluesteinMaxN = 2048;  // longest axis with a prime factor above 7 (M <= 4096)
constexpr int kMaxPts = 4096;     // complex points of one pass tile (two buffers in shared memory)
// Launches smaller than this many blocks (two on each of GB300's 152 SMs)
// get smaller tiles / chunks so that one small world still spreads over the
// whole GPU; large batches keep the full-size tiles.  Measured on one 48^3
// world (forward + adjoint): 1, 2, 4 and 8 blocks per SM gave 8.45, 8.7,
// 6.25 and 5.6 thousand fwd+bwd world-steps/s (more, smaller blocks pay
// more per-block start-up than they gain in parallelism).
constexpr long kFillBlocks = 2 * 152;
constexpr int kRawMax = RAW_CM + kMaxChannels;

struct NdTab {  // kernel table of a model, passed by value
  int C, K, max_k, mean, state_fn, dt_mode, nd;
  int D, H, W;
  long cells;
  int cin[kMaxKernels];
  int slot[kMaxKernels];
  int gf[kMaxKernels];
};

NdTab make_tab(const Model& m, int dt_mode) {
  NdTab t;
  t.C = m.C;
  t.K = m.K;
  t.max_k = m.max_k;
  t.mean = m.mean;
  t.state_fn = m.state_fn;
  t.dt_mode = dt_mode;
  t.nd = m.nb_dims;
  t.D = m.D;
  t.H = m.H;
  t.W = m.W;
  t.cells = m.cells;
  for (int k = 0; k < kMaxKernels; ++k) {
    t.cin[k] = k < m.K ? m.cin[k] : 0;
    t.slot[k] = k < m.K ? m.slot[k] : 0;
    t.gf[k] = k < m.K ? m.gf[k] : 0;
  }
  return t;
}

// ------------------------------------------------------------------ passes
// Lines of a pass: line (g, i) starts at g * gstride + i and has L points
// `stride` apart; g < G, i < I.  I == 1: a tile is nl consecutive groups
// (rows of the x pass, contiguous); I > 1: nl consecutive i of one group.
// The smallest M >= 2L - 1 whose prime factors are 2, 3, 5, 7 (the
// Bluestein transform length of an L-point line), or 0 past the tile size.
inline int bluestein_size(int L) {
  if (L < 2 || L > kBluesteinMaxN) return 0;
  for (int m = 2 * L - 1; m <= kMaxPts; ++m)
    if (make_plan(m).stages > 0) return m;
  return 0;
}

struct Pass {
  float2* data;          // complex planes (in and out, in place)
  const float* src_real;  // IN_REAL: real input of the same geometry
  float* dst_real;        // OUT_REAL: Re(result) * scale (stored, or added when accumulate)
  long G, I, gstride, stride;
  int L, nl;
  int M;                  // Bluestein lines: the transform length M >= 2L - 1 (0: an L-point transform)
  FastDivU fnl;            // division by nl
  int in_real, out_real, accumulate;
  float scale;
};

// Bluestein's chirp-z transform (L. Bluestein, "A linear filtering approach
// to the computation of discrete Fourier transform", 1970) for lines whose
// length has a prime factor above 7: with c_n = exp(-i pi n^2 / L),
// X_k = c_k sum_n (x_n c_n) conj(c_{k-n}), a cyclic convolution of length
// M >= 2L - 1 done with M-point transforms (the inverse transform uses
// conj(c)).  The tile holds nl lines of M points (x_n c_n, then zeros);
// `chirp` c_n (n < L) and `bhat` = FFT_M(b), b_m = conj(c_|m|) for |m| < L
// (indices mod M), are in shared memory.  b is even, so FFT_M(conj(b)) =
// conj(bhat).  Unnormalised like fft_line; returns the buffer holding X.
template <bool INV>
__device__ float2* bluestein_lines(float2* A, float2* B, const GPlan& p, const float2* tw, const float2* chirp,
                                   const float2* bhat, int nl, int L) {
  const int M = p.n;
  for (int l = 0; l < nl; ++l)
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
      const float2 c = chirp[j];
      A[l * M + j] = INV ? cmulc(A[l * M + j], c) : cmul(A[l * M + j], c);
    }
  __syncthreads();
  float2* r = fft_line<false>(A, B, p, tw, nl);
  for (int l = 0; l < nl; ++l)
    for (int k = threadIdx.x; k < M; k += blockDim.x)
      r[l * M + k] = INV ? cmulc(r[l * M + k], bhat[k]) : cmul(r[l * M + k], bhat[k]);
  __syncthreads();
  float2* q = fft_line<true>(r, r == A ? B : A, p, tw, nl);
  const float inv_m = 1.f / (float)M;
  for (int l = 0; l < nl; ++l)
    for (int k = threadIdx.x; k < L; k += blockDim.x) {
      const float2 v = INV ? cmulc(q[l * M + k], chirp[k]) : cmul(q[l * M + k], chirp[k]);
      q[l * M + k] = make_float2(v.x * inv_m, v.y * inv_m);
    }
  __syncthreads();
  return q;
}

// chirp c_n = exp(-2 pi i (n^2 mod 2L) / 2L) and bhat = FFT_M(b), computed by
// the block in shared memory with A and B as the transform's scratch
__device__ void bluestein_tables(float2* chirp, float2* bhat, float2* A, float2* B, const GPlan& p,
                                 const float2* tw, int L) {
  const int M = p.n;
  for (int n = threadIdx.x; n < L; n += blockDim.x) chirp[n] = tw_entry((int)(((long)n * n) % (2L * L)), 2 * L);
  __syncthreads();
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const int d = m < L ? m : (M - m < L ? M - m : -1);
    A[m] = d >= 0 ? conjf2(chirp[d]) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* r = fft_line<false>(A, B, p, tw, 1);
  for (int m = threadIdx.x; m < M; m += blockDim.x) bhat[m] = r[m];
  __syncthreads();
}

template <bool INV, bool BL>
__global__ void __launch_bounds__(kNT, 3) nd_pass_kernel(Pass a, GPlan p) {
  extern __shared__ __align__(16) float2 ndsm[];
  const int L = a.L, nl = a.nl;
  const int S = BL ? a.M : L;  // points per line in the tile
  float2* tw = ndsm;
  float2* A = tw + S;
  float2* B = A + (size_t)nl * S;
  float2* chirp = B + (size_t)nl * S;  // Bluestein tables (BL only)
  float2* bhat = chirp + L;
  long g0, i0;
  int lines;
  if (a.I == 1) {
    g0 = (long)blockIdx.x * nl;
    i0 = 0;
    lines = (int)min((long)nl, a.G - g0);
  } else {
    const long tiles = (a.I + nl - 1) / nl;
    g0 = blockIdx.x / tiles;
    i0 = (blockIdx.x % tiles) * nl;
    lines = (int)min((long)nl, a.I - i0);
  }
  fill_twiddles(tw, S);
  if (BL) {
    __syncthreads();
    bluestein_tables(chirp, bhat, A, B, p, tw, L);
  }
  const int pts = nl * L;
  // A tile of the x pass is nl whole rows, contiguous in memory and in the
  // tile (point idx at row-block offset idx); a strided pass's tile holds
  // nl adjacent lines, point idx = j nl + l of the global walk landing at
  // l L + j in the tile.
  const bool rows = a.I == 1;
  const long gbase = rows ? g0 * a.gstride : g0 * a.gstride + i0;
  const int valid = rows ? lines * L : pts;
  // kLoadBatch independent global loads in flight per thread before their
  // shared-memory stores (one load per iteration would serialise on latency)
  constexpr int kLoadBatch = 8;
  for (int base = threadIdx.x; base < pts; base += kLoadBatch * blockDim.x) {
    float2 v[kLoadBatch];
    int dst[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = base + u * blockDim.x;
      long off;
      bool in;
      if (rows && !BL) {
        dst[u] = idx < pts ? idx : -1;
        in = idx < valid;
        off = gbase + idx;
      } else if (rows) {  // Bluestein rows: tile lines of M points
        const int l = idx / L, j = idx - l * L;
        dst[u] = idx < pts ? l * S + j : -1;
        in = idx < valid;
        off = gbase + idx;
      } else {
        const int j = a.fnl.div(idx), l = idx - j * nl;
        dst[u] = idx < pts ? l * S + j : -1;
        in = idx < pts && l < lines;
        off = gbase + l + (long)j * a.stride;
      }
      v[u] = make_float2(0.f, 0.f);
      if (in) v[u] = a.in_real ? make_float2(__ldg(a.src_real + off), 0.f) : a.data[off];
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u)
      if (dst[u] >= 0) A[dst[u]] = v[u];
  }
  if (BL)  // the zero padding of every tile line
    for (int l = 0; l < nl; ++l)
      for (int j = L + threadIdx.x; j < S; j += blockDim.x) A[l * S + j] = make_float2(0.f, 0.f);
  __syncthreads();
  const float2* res = BL ? bluestein_lines<INV>(A, B, p, tw, chirp, bhat, nl, L) : fft_line<INV>(A, B, p, tw, nl);
  for (int idx = threadIdx.x; idx < valid; idx += blockDim.x) {
    long off;
    int src;
    if (rows && !BL) {
      off = gbase + idx;
      src = idx;
    } else if (rows) {
      const int l = idx / L;
      off = gbase + idx;
      src = l * S + (idx - l * L);
    } else {
      const int j = a.fnl.div(idx), l = idx - j * nl;
      if (l >= lines) continue;
      off = gbase + l + (long)j * a.stride;
      src = l * S + j;
    }
    const float2 v = res[src];
    if (a.out_real) {
      const float r = v.x * a.scale;
      a.dst_real[off] = a.accumulate ? a.dst_real[off] + r : r;
    } else {
      a.data[off] = v;
    }
  }
}

// Raise the N-D kernels' dynamic shared-memory limits once per CUDA context
// (the attribute belongs to the context: a context created later, after a
// device reset for example, gets them again).
cudaError_t allow_nd_smem();

// One axis pass over `planes` planes of D x H x W points.  axis 0 = x
// (contiguous), 1 = y, 2 = z.
cudaError_t run_pass(bool inv, int axis, const NdTab& t, long planes, float2* data, const float* src_real,
                     float* dst_real, bool accumulate, float scale, cudaStream_t st) {
  Pass a;
  a.data = data;
  a.src_real = src_real;
  a.dst_real = dst_real;
  a.in_real = src_real != nullptr;
  a.out_real = dst_real != nullptr;
  a.accumulate = accumulate ? 1 : 0;
  a.scale = scale;
  const long HW = (long)t.H * t.W;
  if (axis == 0) {
    a.L = t.W;
    a.G = planes * t.D * t.H;
    a.I = 1;
    a.gstride = t.W;
    a.stride = 1;
  } else if (axis == 1) {
    a.L = t.H;
    a.G = planes * t.D;
    a.I = t.W;
    a.gstride = HW;
    a.stride = t.W;
  } else {
    a.L = t.D;
    a.G = planes;
    a.I = HW;
    a.gstride = HW * t.D;
    a.stride = HW;
  }
  GPlan p = make_plan(a.L);
  a.M = 0;
  if (p.stages == 0) {  // Bluestein lines
    a.M = bluestein_size(a.L);
    if (a.M == 0) return cudaErrorInvalidValue;
    p = make_plan(a.M);
  }
  const bool bl = a.M > 0;
  const int S = bl ? a.M : a.L;
  const int cap = std::max(1, kMaxPts / S);
  // lines per tile: the full tile, or fewer when the pass has too few lines
  // to fill the GPU (at least 4 adjacent lines of a strided pass, so each
  // load still covers a 32-byte sector)
  const long fill = (a.G * a.I + kFillBlocks - 1) / kFillBlocks;
  const long want = std::max<long>(a.I == 1 ? 1 : 4, fill);
  a.nl = (int)std::min<long>(std::min<long>(cap, want), a.I == 1 ? a.G : a.I);
  a.fnl = make_fastdiv((unsigned)a.nl);
  const long tiles = a.I == 1 ? (a.G + a.nl - 1) / a.nl : a.G * ((a.I + a.nl - 1) / a.nl);
  const size_t smem = (size_t)(S + 2L * a.nl * S + (bl ? a.L + S : 0)) * sizeof(float2);
  cudaError_t e = allow_nd_smem();
  if (e != cudaSuccess) return e;
  if (tiles >= (1L << 31)) return cudaErrorInvalidConfiguration;
  if (bl) {
    if (inv) nd_pass_kernel<true, true><<<(unsigned)tiles, kNT, smem, st>>>(a, p);
    else nd_pass_kernel<false, true><<<(unsigned)tiles, kNT, smem, st>>>(a, p);
  } else {
    if (inv) nd_pass_kernel<true, false><<<(unsigned)tiles, kNT, smem, st>>>(a, p);
    else nd_pass_kernel<false, false><<<(unsigned)tiles, kNT, smem, st>>>(a, p);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- plane passes
// 3D worlds whose z-planes fit one tile (H W <= kMaxPts): the x and y
// transforms of a plane in one block -- rows as contiguous lines, then the
// columns of the same row-major tile -- one global read and write per plane
// instead of one per axis.  The line transforms and their order are those of
// the axis passes: x then y forward, y then x inverse.
struct PlaneArgs {
  float2* data;           // complex planes (in and out, in place)
  const float* src_real;  // forward: real input of the same geometry, or null
  float* dst_real;        // inverse: Re(result) * scale (stored, or added when accumulate), or null
  int accumulate;
  float scale;
  int H, W;
  FastDivU wdiv;  // division by W
};

template <bool INV>
__global__ void __launch_bounds__(kNT, 3) nd_plane_kernel(PlaneArgs a, GPlan px, GPlan py) {
  extern __shared__ __align__(16) float2 ndsm[];
  const int H = a.H, W = a.W, pts = H * W;
  float2* twx = ndsm;
  float2* twy = twx + W;
  float2* A = twy + H;
  float2* B = A + pts;
  const long base = (long)blockIdx.x * pts;
  fill_twiddles(twx, W);
  fill_twiddles(twy, H);
  constexpr int kLoadBatch = 8;
  for (int b0 = threadIdx.x; b0 < pts; b0 += kLoadBatch * blockDim.x) {
    float2 v[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = b0 + u * blockDim.x;
      v[u] = make_float2(0.f, 0.f);
      if (idx < pts) v[u] = a.src_real ? make_float2(__ldg(a.src_real + base + idx), 0.f) : a.data[base + idx];
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = b0 + u * blockDim.x;
      if (idx < pts) A[idx] = v[u];
    }
  }
  __syncthreads();
  float2* r;
  if (!INV) {
    r = fft_line<false>(A, B, px, twx, H);                          // x: H rows of W points
    r = fft_cols<false>(r, r == A ? B : A, py, twy, W, W, a.wdiv);  // y: W columns of H points
  } else {
    r = fft_cols<true>(A, B, py, twy, W, W, a.wdiv);
    r = fft_line<true>(r, r == A ? B : A, px, twx, H);
  }
  for (int idx = threadIdx.x; idx < pts; idx += blockDim.x) {
    const float2 v = r[idx];
    if (a.dst_real) {
      const float x = v.x * a.scale;
      a.dst_real[base + idx] = a.accumulate ? a.dst_real[base + idx] + x : x;
    } else {
      a.data[base + idx] = v;
    }
  }
}

bool plane_ok(const NdTab& t) {
  return t.D > 1 && (long)t.H * t.W <= kMaxPts && make_plan(t.H).stages > 0 && make_plan(t.W).stages > 0;
}

// Shared memory of the fused plane epilogue (twiddles, two tiles, the
// channels' fields), or 0 when the world does not take it.
constexpr size_t kPlaneEpiSmemMax = 200 * 1024;
size_t plane_epi_smem(const NdTab& t) {
  if (!plane_ok(t)) return 0;
  const size_t pts = (size_t)t.H * t.W;
  const size_t bytes = (t.W + t.H + 2 * pts) * sizeof(float2) + (size_t)t.C * pts * sizeof(float);
  return bytes <= kPlaneEpiSmemMax ? bytes : 0;
}

// The x and y transforms of `planes` 3D planes (each D z-planes of H x W).
cudaError_t run_plane(bool inv, const NdTab& t, long planes, float2* data, const float* src_real, float* dst_real,
                      bool accumulate, float scale, cudaStream_t st) {
  PlaneArgs a;
  a.data = data;
  a.src_real = src_real;
  a.dst_real = dst_real;
  a.accumulate = accumulate ? 1 : 0;
  a.scale = scale;
  a.H = t.H;
  a.W = t.W;
  a.wdiv = make_fastdiv((unsigned)t.W);
  const GPlan px = make_plan(t.W), py = make_plan(t.H);
  if (px.stages == 0 || py.stages == 0) return cudaErrorInvalidValue;
  const long blocks = planes * t.D;
  if (blocks >= (1L << 31)) return cudaErrorInvalidConfiguration;
  const size_t smem = (size_t)(t.W + t.H + 2L * t.H * t.W) * sizeof(float2);
  cudaError_t e = allow_nd_smem();
  if (e != cudaSuccess) return e;
  if (inv) nd_plane_kernel<true><<<(unsigned)blocks, kNT, smem, st>>>(a, px, py);
  else nd_plane_kernel<false><<<(unsigned)blocks, kNT, smem, st>>>(a, px, py);
  return cudaGetLastError();
}

// Full forward transform of real planes (src) into complex planes (dst).
cudaError_t forward_real(const NdTab& t, long planes, const float* src, float2* dst, cudaStream_t st) {
  cudaError_t e;
  if (plane_ok(t)) {
    e = run_plane(false, t, planes, dst, src, nullptr, false, 1.f, st);
  } else {
    e = run_pass(false, 0, t, planes, dst, src, nullptr, false, 1.f, st);
    if (e == cudaSuccess) e = run_pass(false, 1, t, planes, dst, nullptr, nullptr, false, 1.f, st);
  }
  if (e == cudaSuccess && t.D > 1) e = run_pass(false, 2, t, planes, dst, nullptr, nullptr, false, 1.f, st);
  return e;
}

// Unnormalised inverse transform of complex planes; the real part times
// `scale` is stored into (or added to) dst.
cudaError_t inverse_real(const NdTab& t, long planes, float2* data, float* dst, bool accumulate, float scale,
                         cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (t.D > 1) e = run_pass(true, 2, t, planes, data, nullptr, nullptr, false, 1.f, st);
  if (e != cudaSuccess) return e;
  if (plane_ok(t)) return run_plane(true, t, planes, data, nullptr, dst, accumulate, scale, st);
  e = run_pass(true, 1, t, planes, data, nullptr, nullptr, false, 1.f, st);
  if (e == cudaSuccess) e = run_pass(true, 0, t, planes, data, nullptr, dst, accumulate, scale, st);
  return e;
}

// ------------------------------------------------------------------ spectra
// Prepared spectra: the Hermitian half [planes, D, H, W/2+1] extended to the
// full spectrum [planes, D, H, W] and scaled by 1/cells (the inverse passes
// are unnormalised).
__global__ void nd_prepare_kernel(long planes, int D, int H, int W, float scale, const float2* __restrict__ kh,
                                  float2* __restrict__ kf) {
  const int HWH = W / 2 + 1;
  const long cells = (long)D * H * W, total = planes * cells;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long pl = i / cells;
    long r = i - pl * cells;
    const int x = (int)(r % W);
    r /= W;
    const int y = (int)(r % H), z = (int)(r / H);
    float2 v;
    if (x < HWH) {
      v = kh[((pl * D + z) * H + y) * HWH + x];
    } else {  // K[z, y, x] = conj(K[-z, -y, W - x])
      const int zz = z == 0 ? 0 : D - z, yy = y == 0 ? 0 : H - y;
      const float2 c = kh[((pl * D + zz) * H + yy) * HWH + (W - x)];
      v = make_float2(c.x, -c.y);
    }
    kf[i] = make_float2(v.x * scale, v.y * scale);
  }
}

// Hermitian half of full spectra: [planes, D, H, W] -> [planes, D, H, W/2+1].
__global__ void nd_half_kernel(long planes, int D, int H, int W, const float2* __restrict__ full,
                               float2* __restrict__ half) {
  const int HWH = W / 2 + 1;
  const long rows = planes * D * H, total = rows * HWH;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long row = i / HWH;
    const int x = (int)(i - row * HWH);
    half[i] = full[row * W + x];
  }
}

inline int grid_for(long total) { return (int)std::max(1L, std::min<long>((total + kNT - 1) / kNT, 1L << 16)); }

// ------------------------------------------------------------------ separate last-axis passes
// For worlds whose fused-pass tile set does not fit (long last axes with many
// channels): the last forward axis, these products, then the first inverse
// axis run as three launches.
// P[w, k] = S[w, c_in(k)] * prepared[sol(w), c_in(k), slot(k)]
__global__ void nd_multiply_kernel(NdTab t, int n_worlds, int n_init, const float2* __restrict__ S,
                                   const float2* __restrict__ kf, long kf_sol_stride, float2* __restrict__ P) {
  const long total = (long)n_worlds * t.K * t.cells;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long cell = i % t.cells;
    const long wk = i / t.cells;
    const int k = (int)(wk % t.K), w = (int)(wk / t.K);
    const int sol = w / n_init, c = t.cin[k];
    const float2 s = S[((long)w * t.C + c) * t.cells + cell];
    const float2 kk = __ldg(kf + sol * kf_sol_stride + ((long)c * t.max_k + t.slot[k]) * t.cells + cell);
    P[i] = cmul(s, kk);
  }
}

// gk[w, k] += A_k conj(S_cin(k)) (kernel gradient), Q[w, c] = sum_{k: c_in(k)
// = c} A_k conj(prepared K_k)
__global__ void nd_adj_spectral_kernel(NdTab t, int n_worlds, int n_init, const float2* __restrict__ A,
                                       const float2* __restrict__ S, const float2* __restrict__ kf,
                                       long kf_sol_stride, float2* __restrict__ gk, float2* __restrict__ Q) {
  const long total = (long)n_worlds * t.cells;
  const int C = t.C, K = t.K;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int w = (int)(i / t.cells);
    const long cell = i - (long)w * t.cells;
    const int sol = w / n_init;
    float2 q[kMaxChannels];
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) q[c] = make_float2(0.f, 0.f);
    for (int k = 0; k < K; ++k) {
      const int c = t.cin[k];
      const float2 ak = A[((long)w * K + k) * t.cells + cell];
      const float2 sc = S[((long)w * C + c) * t.cells + cell];
      float2* g = gk + ((long)w * K + k) * t.cells + cell;
      *g = cadd(*g, cmulc(ak, sc));
      const float2 kk = __ldg(kf + sol * kf_sol_stride + ((long)c * t.max_k + t.slot[k]) * t.cells + cell);
      const float2 pr = cmulc(ak, kk);
#pragma unroll
      for (int cc = 0; cc < kMaxChannels; ++cc)
        if (cc == c) q[cc] = cadd(q[cc], pr);
    }
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      Q[((long)w * C + c) * t.cells + cell] = q[c];
    }
  }
}

// ------------------------------------------------------------------ fused convolution pass
// Along the last world axis (z in 3D, y in 2D) line i of a plane holds the
// points i + j I, j < L, with I = cells / L lines per plane.  One block takes
// a tile of nl adjacent lines of one world: the forward transform along the
// axis of each channel, the spectrum products, the inverse transform of each
// product -- the last forward pass, the multiply and the first inverse pass
// in one launch, with the channel spectra kept in shared memory.  The
// arithmetic is that of the separate passes, in the same order.
struct ConvArgs {
  int n_init, L, nl, tiles;  // points per line, lines per tile, tiles per plane
  FastDivU fnl;               // division by nl
  long I;                    // lines per plane (= point stride along the axis)
  const float2* kf;          // prepared full spectra [Ns, C, max_k, cells]
  long kf_sol_stride;
  const float2* S;           // forward: [nw, C] planes, the other axes transformed
  float2* P;                 // forward: [nw, K] product planes out
  const float2* A;           // adjoint: [nw, K] planes of a = dL/du, the other axes transformed
  float2* gk;                // adjoint: [nw, K] kernel-gradient spectra (accumulated)
  float2* Q;                 // adjoint: [nw, C] correlation planes out
};

// nl lines of a plane (points src[l + j I]) into a line-major tile (lines
// past `lines` read as zero); kLoadBatch loads in flight per thread
__device__ __forceinline__ void load_lines(float2* dst, const float2* __restrict__ src, long I, int L, int nl,
                                           FastDivU fnl, int lines) {
  const int pts = nl * L;
  constexpr int kLoadBatch = 8;
  for (int base = threadIdx.x; base < pts; base += kLoadBatch * blockDim.x) {
    float2 v[kLoadBatch];
    int d[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = base + u * blockDim.x;
      const int j = fnl.div(idx), l = idx - j * nl;
      d[u] = idx < pts ? l * L + j : -1;
      v[u] = make_float2(0.f, 0.f);
      if (idx < pts && l < lines) v[u] = src[l + (long)j * I];
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u)
      if (d[u] >= 0) dst[d[u]] = v[u];
  }
}

__device__ __forceinline__ void store_lines(float2* __restrict__ dst, const float2* src, long I, int L, int nl,
                                            FastDivU fnl, int lines) {
  for (int idx = threadIdx.x; idx < nl * L; idx += blockDim.x) {
    const int j = fnl.div(idx), l = idx - j * nl;
    if (l < lines) dst[l + (long)j * I] = src[l * L + j];
  }
}

// forward: P[w, k] = IFFT_axis(FFT_axis(S[w, c_in(k)]) * prepared[sol, c_in(k), slot(k)])
__global__ void __launch_bounds__(kNT) nd_conv_kernel(NdTab t, ConvArgs a, GPlan p) {
  extern __shared__ __align__(16) float2 ndsm[];
  const int L = a.L, nl = a.nl, pts = nl * L;
  float2* tw = ndsm;
  float2* Sc = tw + L;  // [C][pts] channel spectra along the axis
  float2* A = Sc + (size_t)t.C * pts;
  float2* B = A + pts;
  const int w = blockIdx.x / a.tiles;
  const long i0 = (long)(blockIdx.x % a.tiles) * nl;
  const int lines = (int)min((long)nl, a.I - i0);
  const int sol = w / a.n_init;
  fill_twiddles(tw, L);
  for (int c = 0; c < t.C; ++c) {
    load_lines(A, a.S + ((long)w * t.C + c) * t.cells + i0, a.I, L, nl, a.fnl, lines);
    __syncthreads();
    const float2* r = fft_line<false>(A, B, p, tw, nl);
    for (int x = threadIdx.x; x < pts; x += blockDim.x) Sc[c * pts + x] = r[x];
    __syncthreads();
  }
  for (int k = 0; k < t.K; ++k) {
    const int c = t.cin[k];
    load_lines(A, a.kf + sol * a.kf_sol_stride + ((long)c * t.max_k + t.slot[k]) * t.cells + i0, a.I, L, nl, a.fnl, lines);
    __syncthreads();
    for (int x = threadIdx.x; x < pts; x += blockDim.x) A[x] = cmul(Sc[c * pts + x], A[x]);
    __syncthreads();
    const float2* r = fft_line<true>(A, B, p, tw, nl);
    store_lines(a.P + ((long)w * t.K + k) * t.cells + i0, r, a.I, L, nl, a.fnl, lines);
    __syncthreads();
  }
}

// adjoint: with A_k = FFT(a_k), S_c = FFT(state_c) along the axis,
// gk[w, k] += A_k conj(S_c_in(k)) and Q[w, c] = IFFT_axis(sum_{k: c_in(k) = c}
// A_k conj(prepared_k)) -- the last forward passes of a and of the state, the
// spectral products and the first inverse pass of Q in one launch
__global__ void __launch_bounds__(kNT) nd_adj_conv_kernel(NdTab t, ConvArgs a, GPlan p) {
  extern __shared__ __align__(16) float2 ndsm[];
  const int L = a.L, nl = a.nl, pts = nl * L;
  float2* tw = ndsm;
  float2* Sc = tw + L;                    // [C][pts]
  float2* Qc = Sc + (size_t)t.C * pts;    // [C][pts]
  float2* A = Qc + (size_t)t.C * pts;
  float2* B = A + pts;
  const int w = blockIdx.x / a.tiles;
  const long i0 = (long)(blockIdx.x % a.tiles) * nl;
  const int lines = (int)min((long)nl, a.I - i0);
  const int sol = w / a.n_init;
  fill_twiddles(tw, L);
  for (int c = 0; c < t.C; ++c) {
    load_lines(A, a.S + ((long)w * t.C + c) * t.cells + i0, a.I, L, nl, a.fnl, lines);
    __syncthreads();
    const float2* r = fft_line<false>(A, B, p, tw, nl);
    for (int x = threadIdx.x; x < pts; x += blockDim.x) {
      Sc[c * pts + x] = r[x];
      Qc[c * pts + x] = make_float2(0.f, 0.f);
    }
    __syncthreads();
  }
  for (int k = 0; k < t.K; ++k) {
    const int c = t.cin[k];
    load_lines(A, a.A + ((long)w * t.K + k) * t.cells + i0, a.I, L, nl, a.fnl, lines);
    __syncthreads();
    const float2* r = fft_line<false>(A, B, p, tw, nl);
    float2* o = r == A ? B : A;  // the free buffer takes the prepared spectrum's lines
    load_lines(o, a.kf + sol * a.kf_sol_stride + ((long)c * t.max_k + t.slot[k]) * t.cells + i0, a.I, L, nl, a.fnl,
               lines);
    __syncthreads();
    float2* g = a.gk + ((long)w * t.K + k) * t.cells + i0;
    for (int idx = threadIdx.x; idx < pts; idx += blockDim.x) {
      const int j = a.fnl.div(idx), l = idx - j * nl;
      if (l >= lines) continue;
      const int x = l * L + j;
      const float2 ak = r[x];
      float2* gp = g + l + (long)j * a.I;
      *gp = cadd(*gp, cmulc(ak, Sc[c * pts + x]));
      Qc[c * pts + x] = cadd(Qc[c * pts + x], cmulc(ak, o[x]));
    }
    __syncthreads();
  }
  for (int c = 0; c < t.C; ++c) {
    for (int x = threadIdx.x; x < pts; x += blockDim.x) A[x] = Qc[c * pts + x];
    __syncthreads();
    const float2* r = fft_line<true>(A, B, p, tw, nl);
    store_lines(a.Q + ((long)w * t.C + c) * t.cells + i0, r, a.I, L, nl, a.fnl, lines);
    __syncthreads();
  }
}

// Tile and shared memory of a fused convolution pass; `bufs` complex tiles
// besides the twiddles (C + 2 forward, 2C + 2 adjoint).
constexpr long kConvSmemPts = 96 * 1024 / 8;  // 96 KB of tiles: two blocks per SM
// the largest tile set a fused pass may take; worlds whose one-line tile set
// is larger (long last axes with many channels) take the separate passes
constexpr int kConvSmemMax = 200 * 1024;

// Lines per tile and shared memory of the fused pass along the last axis, or
// 0 when even one line per tile does not fit.
size_t conv_smem(const NdTab& t, bool adjoint, long nw, int* nl_out) {
  const long L = t.nd == 3 ? t.D : t.H;
  if (make_plan((int)L).stages == 0) return 0;  // Bluestein lines take the separate passes
  const long I = t.cells / L;
  const long bufs = adjoint ? 2L * t.C + 2 : (long)t.C + 2;
  const long cap_pts = std::min<long>(kMaxPts, (kConvSmemPts - L) / bufs);
  const long cap = std::max<long>(1, cap_pts / L);
  const long fill = (nw * I + kFillBlocks - 1) / kFillBlocks;
  const long nl = std::min<long>(std::min<long>(cap, std::max<long>(4, fill)), I);
  const size_t smem = (size_t)(L + bufs * nl * L) * sizeof(float2);
  if (nl_out) *nl_out = (int)nl;
  return smem <= (size_t)kConvSmemMax ? smem : 0;
}

cudaError_t run_conv(bool adjoint, const NdTab& t, long nw, ConvArgs a, cudaStream_t st) {
  a.L = t.nd == 3 ? t.D : t.H;
  a.I = t.cells / a.L;
  const GPlan p = make_plan(a.L);
  if (p.stages == 0) return cudaErrorInvalidValue;
  const size_t smem = conv_smem(t, adjoint, nw, &a.nl);
  if (smem == 0) return cudaErrorInvalidConfiguration;
  a.tiles = (int)((a.I + a.nl - 1) / a.nl);
  a.fnl = make_fastdiv((unsigned)a.nl);
  const long blocks = nw * a.tiles;
  if (blocks >= (1L << 31)) return cudaErrorInvalidConfiguration;
  cudaError_t e = allow_nd_smem();
  if (e != cudaSuccess) return e;
  if (adjoint) nd_adj_conv_kernel<<<(unsigned)blocks, kNT, smem, st>>>(t, a, p);
  else nd_conv_kernel<<<(unsigned)blocks, kNT, smem, st>>>(t, a, p);
  return cudaGetLastError();
}


// The axis passes before and after the fused one: forward x (real input)
// and, in 3D, y; inverse y (3D) and x (real part out).
cudaError_t forward_real_head(const NdTab& t, long planes, const float* src, float2* dst, cudaStream_t st) {
  if (plane_ok(t)) return run_plane(false, t, planes, dst, src, nullptr, false, 1.f, st);
  cudaError_t e = run_pass(false, 0, t, planes, dst, src, nullptr, false, 1.f, st);
  if (e == cudaSuccess && t.D > 1) e = run_pass(false, 1, t, planes, dst, nullptr, nullptr, false, 1.f, st);
  return e;
}

cudaError_t inverse_real_tail(const NdTab& t, long planes, float2* data, float* dst, bool accumulate, float scale,
                              cudaStream_t st) {
  if (plane_ok(t)) return run_plane(true, t, planes, data, nullptr, dst, accumulate, scale, st);
  cudaError_t e = cudaSuccess;
  if (t.D > 1) e = run_pass(true, 1, t, planes, data, nullptr, nullptr, false, 1.f, st);
  if (e == cudaSuccess) e = run_pass(true, 0, t, planes, data, nullptr, dst, accumulate, scale, st);
  return e;
}

// ------------------------------------------------------------------ forward epilogue
struct EpiArgs {
  int n_worlds, n_init, bpw;
  const float* state;   // [nw, C, cells]
  float* state_out;     // [nw, C, cells]
  const float* pot;     // [nw, K, cells]
  float* pot_out;       // [nw, K, cells] potential trajectory (fused plane epilogue), or null
  const float* gf;      // [Ns, K, 2] (sol stride gf_sol_stride)
  long gf_sol_stride;
  const float* w;       // [Ns, C, K]
  long w_sol_stride;
  const float* dt;
  float* field_out;     // [nw, C, cells] or null
  float* state_copy;    // [nw, C, cells] copy of the entering state (trajectory), or null
  int* shift;           // [nw, 3] read by every block, advanced by the world's last block
  int* done;            // [nw] blocks finished this step (zero between steps)
  float* partial;       // [nw, bpw, RAWS]
  float* raw;           // the step's raw record, or null
  long raw_sol_stride, raw_init_stride;
};

// per-cell centred coordinate on one axis (statistics.py:64-81 on the world
// rolled by the carried shift): ((i - shift) mod n) - n // 2
// (for 0 <= i, sh < n: a carried shift is always reduced mod n)
__device__ __forceinline__ float centred_in(int i, int sh, int n) {
  const int d = i - sh;
  return (float)((d < 0 ? d + n : d) - n / 2);
}

// Per-thread statistics moments of one block of cells (statistics.py:64-100
// in the centred frame), then the block's partial and, in the world's last
// block, the step's raw record and the carried shift.
struct Moments {
  float m00 = 0.f, g00 = 0.f, cpot = 0.f, cmass = 0.f, cgrow = 0.f;
  float mx0 = 0.f, mx1 = 0.f, mx2 = 0.f, gx0 = 0.f, gx1 = 0.f, gx2 = 0.f, q0 = 0.f, q1 = 0.f, q2 = 0.f;
  float cm[kMaxChannels];
  bool border = false;
  __device__ Moments() {
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) cm[c] = 0.f;
  }
  // one channel of one cell: entering state sv, field f, centred coordinates
  __device__ __forceinline__ void add(int c, float sv, float f, float ca, float cb, float cc, bool edge) {
    const float fp = fmaxf(f, 0.f);
    m00 += sv;
    g00 += fp;
    cm[c] += sv;
    mx0 = fmaf(ca, sv, mx0);
    mx1 = fmaf(cb, sv, mx1);
    mx2 = fmaf(cc, sv, mx2);
    gx0 = fmaf(ca, fp, gx0);
    gx1 = fmaf(cb, fp, gx1);
    gx2 = fmaf(cc, fp, gx2);
    q0 = fmaf(ca * ca, sv, q0);
    q1 = fmaf(cb * cb, sv, q1);
    q2 = fmaf(cc * cc, sv, q2);
    const bool live = sv > kEps;
    cmass += live ? 1.f : 0.f;
    cgrow += fp > kEps ? 1.f : 0.f;
    border |= live && edge;
  }
};

// Block b of world w: reduce the threads' moments into the block's partial;
// the world's last block to finish (a ticket on the world's counter; no block
// waits) reduces all of the world's block partials in a fixed order into the
// step's raw record (with the shift s0..s2 that centred it), then advances
// the carried shift by the integer part of the centred-frame centroid
// (statistics.py:117-124).  Every thread of the block calls it.
__device__ __forceinline__ void epi_finish(const NdTab& t, const EpiArgs& a, int w, int b, int bpw, Moments& mo,
                                           int s0, int s1, int s2) {
  constexpr int NWARP = kNT / 32;
  __shared__ float red[NWARP][kRawMax];
  __shared__ int last;
  __shared__ float tot[kRawMax];
  const int C = t.C, nd = t.nd;
  const int sol = w / a.n_init, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float v[14] = {mo.m00, mo.g00, mo.cpot, mo.cmass, mo.cgrow, mo.mx0, mo.mx1,
                 mo.mx2, mo.gx0, mo.gx1, mo.gx2, mo.q0,   mo.q1,   mo.q2};
#pragma unroll
  for (int i = 0; i < 14; ++i) v[i] = warp_sum(v[i]);
  const bool anyb = __any_sync(0xffffffffu, mo.border);
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) {
    if (c >= C) break;
    mo.cm[c] = warp_sum(mo.cm[c]);
  }
  if (lane == 0) {
    float* rd = red[wid];
    rd[RAW_M00] = v[0];
    rd[RAW_G00] = v[1];
    rd[RAW_CNT_POT] = v[2];
    rd[RAW_CNT_MASS] = v[3];
    rd[RAW_CNT_GROW] = v[4];
    for (int i = 0; i < 3; ++i) {
      rd[RAW_MX + i] = v[5 + i];
      rd[RAW_GX + i] = v[8 + i];
      rd[RAW_MX2 + i] = v[11 + i];
    }
    rd[RAW_BORDER] = anyb ? 1.f : 0.f;
    for (int i = 0; i < 3; ++i) rd[RAW_SHIFT + i] = 0.f;
    for (int c = 0; c < C; ++c) rd[RAW_CM + c] = mo.cm[c];
  }
  __syncthreads();
  const int RAWS = raw_stride(C);
  float* pw = a.partial + (long)w * bpw * RAWS;
  if (threadIdx.x < RAWS) {
    float s = 0.f;
    for (int i = 0; i < NWARP; ++i) s += red[i][threadIdx.x];
    if (threadIdx.x == RAW_BORDER) s = s > 0.f ? 1.f : 0.f;
    pw[b * RAWS + threadIdx.x] = s;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(a.done + w, 1) == bpw - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int s = lane; s < RAWS; s += 32) {
    float acc = 0.f;
    for (int bb = wid; bb < bpw; bb += NWARP) acc += __ldcg(pw + bb * RAWS + s);
    red[wid][s] = acc;
  }
  __syncthreads();
  if (threadIdx.x < RAWS) {
    const int s = threadIdx.x;
    float acc = 0.f;
    for (int i = 0; i < NWARP; ++i) acc += red[i][s];
    if (s == RAW_BORDER) acc = acc > 0.f ? 1.f : 0.f;
    if (s == RAW_SHIFT) acc = (float)s0;
    if (s == RAW_SHIFT + 1) acc = (float)s1;
    if (s == RAW_SHIFT + 2) acc = (float)s2;
    tot[s] = acc;
    if (a.raw) a.raw[sol * a.raw_sol_stride + (w - sol * a.n_init) * a.raw_init_stride + s] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int n[3] = {nd == 2 ? t.H : t.D, nd == 2 ? t.W : t.H, t.W};
    const int sh[3] = {s0, s1, s2};
    for (int i = 0; i < nd; ++i) a.shift[3 * w + i] = pmod(sh[i] + (int)(tot[RAW_MX + i] / (tot[RAW_M00] + kEps)), n[i]);
    a.done[w] = 0;
  }
}

__device__ __forceinline__ float step_dt(const NdTab& t, const EpiArgs& a, int w, int sol) {
  if (t.dt_mode == 0) return __ldg(a.dt);
  if (t.dt_mode == 1) return __ldg(a.dt + w);
  return 1.f / __ldg(a.dt + sol);
}

__global__ void __launch_bounds__(kNT, 3) nd_epilogue_kernel(NdTab t, EpiArgs a) {
  const int w = blockIdx.x / a.bpw, b = blockIdx.x % a.bpw;
  const int sol = w / a.n_init;
  const int C = t.C, K = t.K;
  const float* gf = a.gf + sol * a.gf_sol_stride;
  const float* wt = a.w + sol * a.w_sol_stride;
  const float dt = step_dt(t, a, w, sol);
  const int nd = t.nd;
  // axis order of the moments: 2D (y, x), 3D (z, y, x)
  const int s0 = a.shift[3 * w], s1 = a.shift[3 * w + 1], s2 = a.shift[3 * w + 2];
  const long chunk = (t.cells + a.bpw - 1) / a.bpw;
  const long c0 = (long)b * chunk, c1 = min(t.cells, c0 + chunk);
  Moments mo;
  // (x, y, z) of the thread's cell, advanced by the block's stride of kNT
  // cells with one carry per axis (no divisions inside the loop)
  long cell = c0 + threadIdx.x;
  int x = (int)(cell % t.W), y = (int)((cell / t.W) % t.H), z = (int)(cell / ((long)t.W * t.H));
  const int sx = kNT % t.W, sy = (kNT / t.W) % t.H, sz = (int)(kNT / ((long)t.W * t.H));
  for (; cell < c1; cell += kNT) {
    float ca, cb, cc;  // centred coordinates along the moment axes
    if (nd == 2) {
      ca = centred_in(y, s0, t.H);
      cb = centred_in(x, s1, t.W);
      cc = 0.f;
    } else {
      ca = centred_in(z, s0, t.D);
      cb = centred_in(y, s1, t.H);
      cc = centred_in(x, s2, t.W);
    }
    const bool edge = x == 0 || x == t.W - 1 || y == 0 || y == t.H - 1 || (nd == 3 && (z == 0 || z == t.D - 1));
    for (int k = 0; k < K; ++k) mo.cpot += __ldg(a.pot + ((long)w * K + k) * t.cells + cell) > kEps ? 1.f : 0.f;
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      float f = 0.f, wsum = 0.f;
      for (int k = 0; k < K; ++k) {
        const float wk = __ldg(wt + c * K + k);
        wsum += wk;
        if (wk == 0.f) continue;
        const float u = __ldg(a.pot + ((long)w * K + k) * t.cells + cell);
        f = fmaf(wk, growth_fn(t.gf[k], u, __ldg(gf + 2 * k), __ldg(gf + 2 * k + 1)), f);
      }
      if (t.mean) f = f / wsum;
      const long off = ((long)w * C + c) * t.cells + cell;
      const float sv = __ldg(a.state + off);
      a.state_out[off] = state_fn(t.state_fn, sv, f, dt);
      if (a.field_out) a.field_out[off] = f;
      if (a.state_copy) a.state_copy[off] = sv;
      mo.add(c, sv, f, ca, cb, cc, edge);
    }
    x += sx;
    if (x >= t.W) {
      x -= t.W;
      ++y;
    }
    y += sy;
    if (y >= t.H) {
      y -= t.H;
      ++z;
    }
    z += sz;
  }
  epi_finish(t, a, w, b, a.bpw, mo, s0, s1, s2);
}

// 3D worlds whose z-planes fit one tile: the inverse y and x transforms of
// every kernel's product plane and the epilogue in one block per (world,
// z-plane) -- the potentials never leave shared memory (they are stored
// only as a requested trajectory).  Per channel the weighted field is
// accumulated over the kernels in order, as in nd_epilogue_kernel, so the
// results are the same.
__global__ void __launch_bounds__(kNT, 3) nd_plane_epilogue_kernel(NdTab t, EpiArgs a, const float2* __restrict__ P,
                                                                GPlan px, GPlan py, FastDivU wdiv) {
  extern __shared__ __align__(16) float2 ndsm[];
  const int H = t.H, W = t.W, D = t.D, pts = H * W;
  const int C = t.C, K = t.K;
  const int w = blockIdx.x / D, zp = blockIdx.x % D;
  const int sol = w / a.n_init;
  float2* twx = ndsm;
  float2* twy = twx + W;
  float2* A = twy + H;
  float2* B = A + pts;
  float* F = reinterpret_cast<float*>(B + pts);  // [C][pts] weighted fields
  const float* gf = a.gf + sol * a.gf_sol_stride;
  const float* wt = a.w + sol * a.w_sol_stride;
  const float dt = step_dt(t, a, w, sol);
  const int s0 = a.shift[3 * w], s1 = a.shift[3 * w + 1], s2 = a.shift[3 * w + 2];
  const long pbase = (long)zp * pts;  // the plane's first cell
  fill_twiddles(twx, W);
  fill_twiddles(twy, H);
  for (int i = threadIdx.x; i < C * pts; i += kNT) F[i] = 0.f;
  Moments mo;
  for (int k = 0; k < K; ++k) {
    const float2* src = P + ((long)w * K + k) * t.cells + pbase;
    constexpr int kLoadBatch = 8;
    for (int b0 = threadIdx.x; b0 < pts; b0 += kLoadBatch * kNT) {
      float2 v[kLoadBatch];
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u) {
        const int idx = b0 + u * kNT;
        v[u] = idx < pts ? src[idx] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u) {
        const int idx = b0 + u * kNT;
        if (idx < pts) A[idx] = v[u];
      }
    }
    __syncthreads();
    float2* r = fft_cols<true>(A, B, py, twy, W, W, wdiv);
    r = fft_line<true>(r, r == A ? B : A, px, twx, H);
    const int id = t.gf[k];
    const float m = __ldg(gf + 2 * k), sg = __ldg(gf + 2 * k + 1);
    for (int idx = threadIdx.x; idx < pts; idx += kNT) {
      const float u = r[idx].x;
      if (a.pot_out) a.pot_out[((long)w * K + k) * t.cells + pbase + idx] = u;
      mo.cpot += u > kEps ? 1.f : 0.f;
      const float g = growth_fn(id, u, m, sg);
      for (int c = 0; c < C; ++c) {
        const float wk = __ldg(wt + c * K + k);
        if (wk != 0.f) F[c * pts + idx] = fmaf(wk, g, F[c * pts + idx]);
      }
    }
    __syncthreads();  // A and B are reloaded for the next kernel
  }
  float wsum[kMaxChannels];
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) {
    wsum[c] = 0.f;
    if (c < C)
      for (int k = 0; k < K; ++k) wsum[c] += __ldg(wt + c * K + k);
  }
  const float ca = centred_in(zp, s0, D);
  const bool zedge = zp == 0 || zp == D - 1;
  for (int idx = threadIdx.x; idx < pts; idx += kNT) {
    const int y = wdiv.div(idx), x = idx - y * W;
    const float cb = centred_in(y, s1, H), cc = centred_in(x, s2, W);
    const bool edge = zedge || x == 0 || x == W - 1 || y == 0 || y == H - 1;
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      float f = F[c * pts + idx];
      if (t.mean) f = f / wsum[c];
      const long off = ((long)w * C + c) * t.cells + pbase + idx;
      const float sv = __ldg(a.state + off);
      a.state_out[off] = state_fn(t.state_fn, sv, f, dt);
      if (a.field_out) a.field_out[off] = f;
      if (a.state_copy) a.state_copy[off] = sv;
      mo.add(c, sv, f, ca, cb, cc, edge);
    }
  }
  epi_finish(t, a, w, zp, D, mo, s0, s1, s2);
}

// ------------------------------------------------------------------ adjoint
struct AdjArgs {
  int n_worlds, n_init, clip_mask;
  const float* s;      // [nw, C, cells] state entering the step
  const float* s_next;  // [nw, C, cells] state after the step, or null
  const float* u;      // [nw, K, cells] potentials of the step
  const float* lam;    // [nw, C, cells] dL/d(state after the step)
  float* lam_out;      // [nw, C, cells] direct part of dL/d(state before the step)
  float* a;            // [nw, K, cells] dL/du_k
  float* bf;           // [nw, C, cells] dL/df_c
  float* ff;           // [nw, C, cells] f_c
  float* s_copy;       // [nw, C, cells] copy of s, stored right after a
  const float* gf;     // [Ns, K, 2]
  const float* w;      // [Ns, C, K]
  const float* T;      // [Ns]
};

// growth(u) and its derivative in u (growth_functions.py); every family but
// identity is a function of (u - m) / s, so d/dm = -d/du and
// d/ds = -d/du (u - m) / s.
__device__ __forceinline__ float growth_du(int id, float u, float m, float s, float* g) {
  if (id == LGX_GF_GAUSSIAN || id == LGX_GF_GAUSSIAN_TARGET) {
    const float d = (u - m) / s;
    const float e = expf(-(d * d) / 2.f);
    const float amp = id == LGX_GF_GAUSSIAN ? 2.f : 1.f;
    *g = id == LGX_GF_GAUSSIAN ? 2.f * e - 1.f : e;
    return -amp * e * d / s;
  }
  if (id == LGX_GF_POLY_QUAD4) {
    const float d = u - m, c = 9.f * s * s;
    const float q = 1.f - d * d / c;
    if (q > 0.f) {
      const float q3 = q * q * q;
      *g = 2.f * q3 * q - 1.f;
      return 8.f * q3 * (-2.f * d / c);
    }
    *g = -1.f;
    return 0.f;
  }
  *g = growth_fn(id, u, m, s);
  if (id == LGX_GF_IDENTITY) return 1.f;
  if (id == LGX_GF_TRIANGLE) {  // growth_functions.py:234-243: slopes 2/s and -2/s
    if (u >= m - s && u < m) return 2.f / s;
    if (u >= m && u <= m + s) return -2.f / s;
  }
  return 0.f;  // step, staircase: piecewise constant
}

// Pointwise part of the reverse step, one block per (world, chunk of cells):
// the clip / state-function gradient, dL/df per channel, dL/dg per kernel
// (the weighted merge's transpose) and the growth derivative give
// a_k = dL/du_k; the entering state is copied beside a (both are
// transformed by the same passes).  With FK > 0 the model has exactly FK
// kernels and FC channels and the block also adds its parameter partials
// (those of nd_adj_param_kernel) into its slots of pacc.
template <int FK, int FC>
__global__ void __launch_bounds__(kNT) nd_adj_point_kernel(NdTab t, AdjArgs a, int pb, float* __restrict__ pacc) {
  constexpr bool kFused = FK > 0;
  const int C = kFused ? FC : t.C, K = kFused ? FK : t.K;
  const int w = blockIdx.x / pb, b = blockIdx.x % pb;
  const long chunk = (t.cells + pb - 1) / pb;
  const long c0 = (long)b * chunk, c1 = min(t.cells, c0 + chunk);
  const int sol = w / a.n_init;
  const float dt = 1.f / __ldg(a.T + sol);
  const float* gf = a.gf + (long)sol * 2 * K;
  const float* wt = a.w + (long)sol * C * K;
  constexpr int kAcc = kFused ? FK * (2 + FC) : 1;
  float acc[kAcc];
#pragma unroll
  for (int j = 0; j < kAcc; ++j) acc[j] = 0.f;
  for (long cell = c0 + threadIdx.x; cell < c1; cell += blockDim.x) {
    float f[kMaxChannels], bb[kMaxChannels], ws[kMaxChannels];
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      f[c] = 0.f;
      ws[c] = 0.f;
      bb[c] = 0.f;
    }
    for (int k = 0; k < K; ++k) {
      const float u = __ldg(a.u + ((long)w * K + k) * t.cells + cell);
      const float g = growth_fn(t.gf[k], u, __ldg(gf + 2 * k), __ldg(gf + 2 * k + 1));
#pragma unroll
      for (int c = 0; c < kMaxChannels; ++c) {
        if (c >= C) break;
        const float wk = __ldg(wt + c * K + k);
        ws[c] += wk;
        if (wk != 0.f) f[c] = fmaf(wk, g, f[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      if (t.mean) f[c] = f[c] / ws[c];
      const long off = ((long)w * C + c) * t.cells + cell;
      const float lam = __ldg(a.lam + off);
      const float sv = __ldg(a.s + off);
      a.s_copy[off] = sv;
      float dsds, dsdf;  // d state' / d state and d state' / d field (core.py:245-319)
      if (t.state_fn == LGX_STATE_V1) {
        // mask: the forward's clip was inactive where its output lies strictly inside (0, 1)
        const float n = a.s_next ? __ldg(a.s_next + off) : fmaf(dt, f[c], sv);
        const float cg = a.clip_mask ? ((n > 0.f && n < 1.f) ? 1.f : 0.f) : 1.f;  // mask or straight-through
        dsds = cg;
        dsdf = dt * cg;
      } else if (t.state_fn == LGX_STATE_V2) {
        dsds = 1.f - dt;
        dsdf = dt;
      } else {
        dsds = 1.f;
        dsdf = dt;
      }
      a.lam_out[off] = lam * dsds;
      bb[c] = lam * dsdf;
      a.bf[off] = bb[c];
      a.ff[off] = f[c];
    }
    for (int k = 0; k < K; ++k) {
      const int id = t.gf[k];
      const float u = __ldg(a.u + ((long)w * K + k) * t.cells + cell);
      const float m = __ldg(gf + 2 * k), sg = __ldg(gf + 2 * k + 1);
      float g;
      const float gu = growth_du(id, u, m, sg, &g);
      float dg = 0.f;  // dL/dg_k = sum_c dL/df_c * w_ck (/ sum_j w_cj in mean mode)
#pragma unroll
      for (int c = 0; c < kMaxChannels; ++c) {
        if (c >= C) break;
        const float wk = __ldg(wt + c * K + k);
        dg = fmaf(bb[c], t.mean ? wk / ws[c] : wk, dg);
      }
      const float ak = dg * gu;
      a.a[((long)w * K + k) * t.cells + cell] = ak;
      if constexpr (kFused) {
        if (k < FK) {
          float* pk = acc + k * (2 + FC);
          if (id != LGX_GF_IDENTITY) {
            pk[0] -= ak;
            pk[1] -= ak * (u - m) / sg;
          }
#pragma unroll
          for (int c = 0; c < FC; ++c) pk[2 + c] = fmaf(bb[c], t.mean ? (g - f[c]) / ws[c] : g, pk[2 + c]);
        }
      }
    }
  }
  if constexpr (kFused) {
    __shared__ float red[kNT / 32][kAcc];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kAcc; ++j) acc[j] = warp_sum(acc[j]);
    if (lane == 0)
#pragma unroll
      for (int j = 0; j < kAcc; ++j) red[wid][j] = acc[j];
    __syncthreads();
    if (threadIdx.x < kAcc) {
      float v = 0.f;
      for (int i = 0; i < kNT / 32; ++i) v += red[i][threadIdx.x];
      const int k = threadIdx.x / (2 + FC), j = threadIdx.x % (2 + FC);
      pacc[(((long)w * FK + k) * pb + b) * (2 + FC) + j] += v;
    }
  }
}

// Per (world, kernel, chunk of cells): dL/dm_k = -sum a_k,
// dL/ds_k = -sum a_k (u_k - m) / s, dL/dw_ck = sum dL/df_c * (g_k - f_c) /
// sum_j w_cj (mean) or dL/df_c * g_k (sum), added into the block's own slot
// pacc[w, k, b] = {dm, ds, dw_0k .. dw_(C-1)k} (each block owns its slot
// across the reverse steps, so the sums are race-free and deterministic).
__global__ void __launch_bounds__(kNT) nd_adj_param_kernel(NdTab t, int n_init, int pb, const float* __restrict__ u,
                                                           const float* __restrict__ a, const float* __restrict__ bf,
                                                           const float* __restrict__ ff, const float* __restrict__ gfp,
                                                           const float* __restrict__ wts, float* __restrict__ pacc) {
  const int C = t.C, K = t.K;
  const int w = blockIdx.x / (K * pb), k = (blockIdx.x / pb) % K, b = blockIdx.x % pb;
  const long chunk = (t.cells + pb - 1) / pb;
  const long c0 = (long)b * chunk, c1 = min(t.cells, c0 + chunk);
  const int sol = w / n_init;
  const float m = __ldg(gfp + ((long)sol * K + k) * 2), s = __ldg(gfp + ((long)sol * K + k) * 2 + 1);
  const int id = t.gf[k];
  float wsum[kMaxChannels];
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) {
    wsum[c] = 0.f;
    if (c < C)
      for (int j = 0; j < K; ++j) wsum[c] += __ldg(wts + ((long)sol * C + c) * K + j);
  }
  float dm = 0.f, ds = 0.f, dw[kMaxChannels];
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) dw[c] = 0.f;
  for (long cell = c0 + threadIdx.x; cell < c1; cell += blockDim.x) {
    const float uu = __ldg(u + ((long)w * K + k) * t.cells + cell);
    const float ak = __ldg(a + ((long)w * K + k) * t.cells + cell);
    if (id != LGX_GF_IDENTITY) {
      dm -= ak;
      ds -= ak * (uu - m) / s;
    }
    const float g = growth_fn(id, uu, m, s);
#pragma unroll
    for (int c = 0; c < kMaxChannels; ++c) {
      if (c >= C) break;
      const long off = ((long)w * C + c) * t.cells + cell;
      const float b = __ldg(bf + off);
      dw[c] = fmaf(b, t.mean ? (g - __ldg(ff + off)) / wsum[c] : g, dw[c]);
    }
  }
  __shared__ float red[kNT / 32][2 + kMaxChannels];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  dm = warp_sum(dm);
  ds = warp_sum(ds);
#pragma unroll
  for (int c = 0; c < kMaxChannels; ++c) dw[c] = warp_sum(dw[c]);
  if (lane == 0) {
    red[wid][0] = dm;
    red[wid][1] = ds;
    for (int c = 0; c < kMaxChannels; ++c) red[wid][2 + c] = dw[c];
  }
  __syncthreads();
  if (threadIdx.x < 2 + C) {
    float v = 0.f;
    for (int i = 0; i < kNT / 32; ++i) v += red[i][threadIdx.x];
    pacc[(((long)w * K + k) * pb + b) * (2 + C) + threadIdx.x] += v;
  }
}

// per solution: grad_gf[s, k] += sum over its inits and chunks of
// pacc[w, k, b, 0:2], grad_w[s, c, k] += sum of pacc[w, k, b, 2 + c]
__global__ void nd_param_reduce_kernel(int n_sols, int n_init, int K, int C, int pb, const float* __restrict__ pacc,
                                       float* __restrict__ grad_gf, float* __restrict__ grad_w) {
  const int per = 2 * K + C * K;
  const long total = (long)n_sols * per;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int sol = (int)(i / per), j = (int)(i % per);
    const int k = j < 2 * K ? j / 2 : (j - 2 * K) % K;
    const int slot = j < 2 * K ? j % 2 : 2 + (j - 2 * K) / K;
    float v = 0.f;
    for (int n = 0; n < n_init; ++n)
      for (int b = 0; b < pb; ++b) v += pacc[((((long)sol * n_init + n) * K + k) * pb + b) * (2 + C) + slot];
    if (j < 2 * K) grad_gf[(long)sol * 2 * K + j] += v;
    else grad_w[(long)sol * C * K + (j - 2 * K)] += v;
  }
}

// gsum[s, k] = sum over the inits of solution s of gk[w, k]
__global__ void nd_sum_inits_kernel(long per_sol, int n_sols, int n_init, const float2* __restrict__ gk,
                                    float2* __restrict__ gsum) {
  const long total = (long)n_sols * per_sol;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int sol = (int)(i / per_sol);
    const long j = i - (long)sol * per_sol;
    float2 v = make_float2(0.f, 0.f);
    for (int n = 0; n < n_init; ++n) v = cadd(v, gk[((long)sol * n_init + n) * per_sol + j]);
    gsum[i] = v;
  }
}

cudaError_t allow_nd_smem() {
  static std::mutex mu;
  static std::vector<unsigned long long> done;  // contexts already set up
  unsigned long long ctx = 0;
  const bool known = current_context_id(&ctx);
  if (known) {
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), ctx) != done.end()) return cudaSuccess;
  }
  // twiddles, two tiles and, for Bluestein lines, the chirp and its spectrum
  const int pass_bytes = (int)((kNdMaxN + 2 * kMaxPts + kBluesteinMaxN + kMaxPts) * sizeof(float2));
  cudaError_t e = cudaSuccess;
  for (auto f : {nd_pass_kernel<false, false>, nd_pass_kernel<true, false>, nd_pass_kernel<false, true>,
                 nd_pass_kernel<true, true>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, pass_bytes);
  const int plane_bytes = (int)((2 * kMaxPts + 2 * kNdMaxN) * sizeof(float2));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(nd_plane_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, plane_bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(nd_plane_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, plane_bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(nd_plane_epilogue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kPlaneEpiSmemMax);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(nd_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmemMax);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(nd_adj_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmemMax);
  if (e == cudaSuccess && known) {
    std::lock_guard<std::mutex> lk(mu);
    done.push_back(ctx);
  }
  return e;
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// ---------------------------------------------------------------------- API
bool nd_side_ok(int n) {
  return n >= 2 && ((n <= kNdMaxN && make_plan(n).stages > 0) || bluestein_size(n) > 0);
}

int nd_max_side() { return kNdMaxN; }

bool nd_supported(const Model& m) {
  if (m.nb_dims != 2 && m.nb_dims != 3) return false;
  if (m.C > kMaxChannels || m.K > kMaxKernels) return false;
  for (int i = 0; i < m.nb_dims; ++i)
    if (!nd_side_ok(m.world[i])) return false;
  return true;
}

int nd_blocks_per_world(const Model& m, long n_worlds) {
  // 16 cells per thread, or more blocks when the batch is too small to fill
  // the GPU (at least one cell per thread, at most 256 blocks)
  const long by_cells = (m.cells + (long)kNT * 16 - 1) / ((long)kNT * 16);
  const long fill = (kFillBlocks + n_worlds - 1) / std::max(1L, n_worlds);
  const long useful = (m.cells + kNT - 1) / kNT;
  return (int)std::max(1L, std::min<long>(256, std::min(useful, std::max(by_cells, fill))));
}

namespace {
// chunks of cells per world of the adjoint's pointwise kernel, and per
// (world, kernel) of its parameter reduction
int nd_param_blocks(const Model& m, long n_worlds) { return nd_blocks_per_world(m, n_worlds); }
}  // namespace

size_t nd_step_workspace_bytes(const Model& m, int n_worlds) {
  const size_t nw = (size_t)n_worlds, cells = (size_t)m.cells;
  return al256(nw * m.C * cells * sizeof(float2)) + al256(nw * m.K * cells * sizeof(float2)) +
         al256(nw * m.K * cells * sizeof(float)) +
         al256(nw * std::max(nd_blocks_per_world(m, (long)nw), m.D) * raw_stride(m.C) * sizeof(float));
}

size_t nd_prepared_bytes(const Model& m, int n_sols) {
  return al256((size_t)n_sols * m.C * m.max_k * m.cells * sizeof(float2));
}

cudaError_t launch_nd_prepare(const Model& m, int n_sols, const float2* k_half, float2* kf, cudaStream_t st) {
  const long planes = (long)n_sols * m.C * m.max_k;
  nd_prepare_kernel<<<grid_for(planes * m.cells), kNT, 0, st>>>(planes, m.D, m.H, m.W, 1.f / (float)m.cells, k_half,
                                                                kf);
  return cudaGetLastError();
}

cudaError_t launch_nd_step(const NdStep& s, cudaStream_t st) {
  const Model& m = *s.m;
  const NdTab t = make_tab(m, s.dt_mode);
  const size_t nw = (size_t)s.n_worlds, cells = (size_t)m.cells;
  const int bpw = nd_blocks_per_world(m, (long)nw);
  char* p = static_cast<char*>(s.ws);
  float2* S = reinterpret_cast<float2*>(p);
  p += al256(nw * m.C * cells * sizeof(float2));
  float2* P = reinterpret_cast<float2*>(p);
  p += al256(nw * m.K * cells * sizeof(float2));
  float* U = reinterpret_cast<float*>(p);
  p += al256(nw * m.K * cells * sizeof(float));
  float* partial = reinterpret_cast<float*>(p);
  float* pot = s.pot_out ? s.pot_out : U;
  cudaError_t e = forward_real_head(t, (long)nw * m.C, s.state, S, st);
  if (e != cudaSuccess) return e;
  const int last = t.nd == 3 ? 2 : 1;  // the last world axis
  if (conv_smem(t, false, (long)nw, nullptr) > 0) {
    ConvArgs ca{};
    ca.n_init = s.n_init;
    ca.kf = s.kf;
    ca.kf_sol_stride = s.kf_sol_stride;
    ca.S = S;
    ca.P = P;
    if ((e = run_conv(false, t, (long)nw, ca, st)) != cudaSuccess) return e;
  } else {
    if ((e = run_pass(false, last, t, (long)nw * m.C, S, nullptr, nullptr, false, 1.f, st)) != cudaSuccess) return e;
    nd_multiply_kernel<<<grid_for((long)nw * m.K * cells), kNT, 0, st>>>(t, s.n_worlds, s.n_init, S, s.kf,
                                                                          s.kf_sol_stride, P);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = run_pass(true, last, t, (long)nw * m.K, P, nullptr, nullptr, false, 1.f, st)) != cudaSuccess) return e;
  }
  const bool fused = plane_epi_smem(t) > 0;
  if (!fused && (e = inverse_real_tail(t, (long)nw * m.K, P, pot, false, 1.f, st)) != cudaSuccess) return e;
  EpiArgs a;
  a.n_worlds = s.n_worlds;
  a.n_init = s.n_init;
  a.bpw = bpw;
  a.state = s.state;
  a.state_out = s.state_out;
  a.pot = pot;
  a.gf = s.gf;
  a.gf_sol_stride = s.gf_sol_stride;
  a.w = s.w;
  a.w_sol_stride = s.w_sol_stride;
  a.dt = s.dt;
  a.field_out = s.field_out;
  a.state_copy = s.state_copy;
  a.shift = s.shift;
  a.done = s.done;
  a.partial = partial;
  a.raw = s.raw;
  a.raw_sol_stride = s.raw_sol_stride;
  a.raw_init_stride = s.raw_world_stride;
  a.pot_out = s.pot_out;
  if (fused) {
    if ((e = allow_nd_smem()) != cudaSuccess) return e;
    a.bpw = m.D;
    nd_plane_epilogue_kernel<<<(unsigned)(nw * m.D), kNT, plane_epi_smem(t), st>>>(
        t, a, P, make_plan(m.W), make_plan(m.H), make_fastdiv((unsigned)m.W));
  } else {
    nd_epilogue_kernel<<<(unsigned)(nw * bpw), kNT, 0, st>>>(t, a);
  }
  return cudaGetLastError();
}

size_t nd_adjoint_workspace_bytes(const Model& m, int n_sols, int n_init) {
  const size_t nw = (size_t)n_sols * n_init, cells = (size_t)m.cells, KC = (size_t)(m.K + m.C);
  return nd_prepared_bytes(m, n_sols) + al256(nw * KC * cells * sizeof(float2)) +  // kf, [A | S]
         al256(nw * m.C * cells * sizeof(float2)) +                                // Q
         al256(nw * KC * cells * sizeof(float)) +                                  // [a | state copy]
         3 * al256(nw * m.C * cells * sizeof(float)) +                             // bf, ff, lambda ping-pong
         al256(nw * m.K * nd_param_blocks(m, (long)nw) * (2 + m.C) * sizeof(float));  // parameter partials
}

size_t nd_kernel_grad_acc_bytes(const Model& m, int n_sols, int n_init) {
  return (size_t)n_sols * n_init * m.K * m.cells * sizeof(float2);
}

cudaError_t launch_nd_adjoint(const Model& m, const NdAdjoint& j, void* ws, cudaStream_t st) {
  const NdTab t = make_tab(m, 2);
  const int nw = j.n_sols * j.n_init;
  const size_t cells = (size_t)m.cells;
  char* p = static_cast<char*>(ws);
  float2* kf = reinterpret_cast<float2*>(p);
  p += nd_prepared_bytes(m, j.n_sols);
  const size_t KC = (size_t)(m.K + m.C);
  float2* A = reinterpret_cast<float2*>(p);  // the K planes of a, then the C planes of the state
  float2* S = A + (size_t)nw * m.K * cells;
  p += al256((size_t)nw * KC * cells * sizeof(float2));
  float2* Q = reinterpret_cast<float2*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float2));
  float* ar = reinterpret_cast<float*>(p);  // a, then the state copy: one real input for the head passes
  p += al256((size_t)nw * KC * cells * sizeof(float));
  float* bf = reinterpret_cast<float*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float));
  float* ff = reinterpret_cast<float*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float));
  float* lam_tmp = reinterpret_cast<float*>(p);
  p += al256((size_t)nw * m.C * cells * sizeof(float));
  float* pacc = reinterpret_cast<float*>(p);
  const long kf_sol = (long)m.C * m.max_k * m.cells;
  const int pb = nd_param_blocks(m, nw);
  const bool fused = m.K == 1 && m.C == 1;  // parameter partials inside the pointwise kernel
  cudaError_t e = launch_nd_prepare(m, j.n_sols, j.k_half, kf, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(pacc, 0, (size_t)nw * m.K * pb * (2 + m.C) * sizeof(float), st);
  if (e != cudaSuccess) return e;
  const size_t plane_c = (size_t)m.C * cells, plane_k = (size_t)m.K * cells;
  const float* lam_in = j.lambda_in;
  for (int step = j.steps - 1; step >= 0; --step) {
    float* lam_out = (step % 2 == 0) ? j.lambda_out : lam_tmp;  // step 0 lands in lambda_out
    AdjArgs a;
    a.n_worlds = nw;
    a.n_init = j.n_init;
    a.clip_mask = j.clip_mask;
    a.s = j.traj_cells + (size_t)step * nw * plane_c;
    a.s_next = step + 1 < j.steps ? a.s + (size_t)nw * plane_c : j.cells_after;
    a.u = j.traj_potential + (size_t)step * nw * plane_k;
    a.lam = lam_in;
    a.lam_out = lam_out;
    a.a = ar;
    a.bf = bf;
    a.ff = ff;
    a.gf = j.gf_params;
    a.w = j.weights;
    a.T = j.T;
    a.s_copy = ar + (size_t)nw * m.K * cells;
    if (fused) {
      nd_adj_point_kernel<1, 1><<<(unsigned)(nw * pb), kNT, 0, st>>>(t, a, pb, pacc);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    } else {
      nd_adj_point_kernel<0, 0><<<(unsigned)(nw * pb), kNT, 0, st>>>(t, a, pb, pacc);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      nd_adj_param_kernel<<<(unsigned)(nw * m.K * pb), kNT, 0, st>>>(t, j.n_init, pb, a.u, ar, bf, ff, j.gf_params,
                                                                       j.weights, pacc);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = forward_real_head(t, (long)nw * KC, ar, A, st)) != cudaSuccess) return e;
    if (conv_smem(t, true, (long)nw, nullptr) > 0) {
      ConvArgs ca{};
      ca.n_init = j.n_init;
      ca.kf = kf;
      ca.kf_sol_stride = kf_sol;
      ca.S = S;
      ca.A = A;
      ca.gk = j.gk;
      ca.Q = Q;
      if ((e = run_conv(true, t, (long)nw, ca, st)) != cudaSuccess) return e;
    } else {
      const int last = t.nd == 3 ? 2 : 1;
      if ((e = run_pass(false, last, t, (long)nw * KC, A, nullptr, nullptr, false, 1.f, st)) != cudaSuccess) return e;
      nd_adj_spectral_kernel<<<grid_for((long)nw * cells), kNT, 0, st>>>(t, nw, j.n_init, A, S, kf, kf_sol, j.gk, Q);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      if ((e = run_pass(true, last, t, (long)nw * m.C, Q, nullptr, nullptr, false, 1.f, st)) != cudaSuccess) return e;
    }
    if ((e = inverse_real_tail(t, (long)nw * m.C, Q, lam_out, true, 1.f, st)) != cudaSuccess) return e;
    lam_in = lam_out;
  }
  nd_param_reduce_kernel<<<grid_for((long)j.n_sols * (2 * m.K + m.C * m.K)), kNT, 0, st>>>(
      j.n_sols, j.n_init, m.K, m.C, pb, pacc, j.grad_gf, j.grad_weights);
  return cudaGetLastError();
}

size_t nd_kernel_grad_workspace_bytes(const Model& m, int n_sols) {
  return al256((size_t)n_sols * m.K * m.cells * sizeof(float2));
}

cudaError_t launch_nd_kernel_grad(const Model& m, int n_sols, int n_init, const float2* gk, float* out, void* ws,
                                  cudaStream_t st) {
  const NdTab t = make_tab(m, 2);
  float2* gsum = static_cast<float2*>(ws);
  const long per = (long)m.K * m.cells;
  nd_sum_inits_kernel<<<grid_for((long)n_sols * per), kNT, 0, st>>>(per, n_sols, n_init, gk, gsum);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // dL/dk = Re(IFFT(sum_t A_t conj(S_t))) = unnormalised inverse / cells
  return inverse_real(t, (long)n_sols * m.K, gsum, out, false, 1.f / (float)m.cells, st);
}

size_t nd_spectrum_workspace_bytes(int nb_dims, const int* world, int planes) {
  long cells = 1;
  for (int i = 0; i < nb_dims; ++i) cells *= world[i];
  return al256((size_t)planes * cells * sizeof(float2));
}

cudaError_t launch_nd_spectrum(int nb_dims, const int* world, int planes, const float* k_real, float2* k_half,
                               void* ws, cudaStream_t st) {
  Model m;
  m.nb_dims = nb_dims;
  m.D = nb_dims == 3 ? world[0] : 1;
  m.H = world[nb_dims - 2];
  m.W = world[nb_dims - 1];
  m.cells = (long)m.D * m.H * m.W;
  m.C = m.K = m.max_k = 1;
  m.mean = 1;
  m.state_fn = 0;
  m.cin[0] = m.slot[0] = m.gf[0] = 0;
  const NdTab t = make_tab(m, 0);
  float2* full = static_cast<float2*>(ws);
  cudaError_t e = forward_real(t, planes, k_real, full, st);
  if (e != cudaSuccess) return e;
  const long total = (long)planes * m.D * m.H * (m.W / 2 + 1);
  nd_half_kernel<<<grid_for(total), kNT, 0, st>>>(planes, m.D, m.H, m.W, full, k_half);
  return cudaGetLastError();
}

}  // namespace lgx
