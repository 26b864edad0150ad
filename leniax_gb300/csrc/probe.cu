// FP32-pipe peak probe: a pure FMA kernel with independent chains, used by
// the benchmark to measure the FP32 roofline of the GPU it runs on.
#include "../../include/lenia_gb300.h"
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) fma_probe_kernel(float* sink, int iters, float seed) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      a0 = fmaf(a0, m, c);
      a1 = fmaf(a1, m, c);
      a2 = fmaf(a2, m, c);
      a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c);
      a5 = fmaf(a5, m, c);
      a6 = fmaf(a6, m, c);
      a7 = fmaf(a7, m, c);
    }
  }
  const float r = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (r == 12345.678f) sink[blockIdx.x] = r;  // keeps the chains alive
}

}  // namespace

extern "C" LGX_API long long lgx_fp32_probe(float* sink, int blocks, int iters, void* stream) {
  if (!sink || blocks < 1 || iters < 1) return -1;
  fma_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(sink, iters, 0.5f);
  if (cudaGetLastError() != cudaSuccess) return -1;
  return 2LL * 8 * 16 * 256 * (long long)blocks * iters;  // flops launched
}
