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
// Two slice barriers per step.  The moments of step t are reduced across warps
// by the slice's last warp during the column pass of step t+1, which also
// advances the carried torus shift before the row inverse of step t+1 reads it.
//
// This is leniax core.update (core.py:13-49) with get_potential_fft
// (core.py:52-102), get_field (core.py:163-199) and get_state (core.py:245-319)
// iterated as in runner._scan_fn (runner.py:295-334); the statistics moments
// follow statistics.py:36-126 on the world rolled by the carried shift.
#include "resident.cuh"

namespace lgx {

namespace {

template <int N, int G, int GF, bool STATS>
__global__ void __launch_bounds__(512, 1) resident_kernel(ResidentArgs a) {
  using CF = RCfg<N, G>;
  extern __shared__ __align__(16) float2 sm[];
  init_twiddles<typename CF::GE>(sm, sm + N, sm + 2 * N, threadIdx.x, blockDim.x);
  __syncthreads();
  int loaded_sol = -1;
  const int n_items = (a.n_worlds + CF::WPC - 1) / CF::WPC;
  for (int item = blockIdx.x; item < n_items; item += gridDim.x)
    resident_item<N, G, GF, STATS>(a, item, sm, sm + 3 * N, loaded_sol);
}

template <int N>
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

template <int N, int G, int GF, bool STATS>
cudaError_t launch_one(const ResidentArgs& a, int grid, cudaStream_t st) {
  using CF = RCfg<N, G>;
  cudaError_t e = cudaFuncSetAttribute(resident_kernel<N, G, GF, STATS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)CF::SMEM);
  if (e != cudaSuccess) return e;
  resident_kernel<N, G, GF, STATS><<<grid, 512, CF::SMEM, st>>>(a);
  return cudaGetLastError();
}

// The statistics-free variant exists for 128 x 128 (the differentiation
// workload's checkpointed forward and trajectory recompute); smaller worlds
// compute the moments and ignore them.
template <int N, int G, bool STATS>
cudaError_t launch_gf(const ResidentArgs& a, int grid, cudaStream_t st) {
  if (a.gf_id == LGX_GF_GAUSSIAN) return launch_one<N, G, GF_FAST_GAUSSIAN, STATS>(a, grid, st);
  if (a.gf_id == LGX_GF_POLY_QUAD4) return launch_one<N, G, GF_FAST_POLY4, STATS>(a, grid, st);
  return launch_one<N, G, GF_GENERIC, STATS>(a, grid, st);
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
    case 32: return launch_gf<32, 4, true>(a, grid, st);
    case 64: return launch_gf<64, 4, true>(a, grid, st);
    case 128: return a.no_stats ? launch_gf<128, 8, false>(a, grid, st) : launch_gf<128, 8, true>(a, grid, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_prepare_resident_spectrum(int N, int n_sols, const float2* k_half, float2* kp, cudaStream_t st) {
  const int threads = 256;
  const long total = (long)n_sols * N * (N / 2 + 2);
  const int blocks = (int)((total + threads - 1) / threads > 4096 ? 4096 : (total + threads - 1) / threads);
  switch (N) {
    case 32: prepare_resident_kernel<32><<<blocks, threads, 0, st>>>(n_sols, k_half, kp); break;
    case 64: prepare_resident_kernel<64><<<blocks, threads, 0, st>>>(n_sols, k_half, kp); break;
    case 128: prepare_resident_kernel<128><<<blocks, threads, 0, st>>>(n_sols, k_half, kp); break;
    case 256: prepare_resident_kernel<256><<<blocks, threads, 0, st>>>(n_sols, k_half, kp); break;  // big 2D items
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace lgx
