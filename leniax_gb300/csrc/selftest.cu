// Failure-detection self test: the bounded mbarrier wait of the streamed and
// batch kernels, driven to its limit on purpose.  The mbarrier expects two
// arrivals and gets one (a flag nothing sets), so the wait gives up after
// `max_polls` polls; the kernel then records the timeout status exactly as
// the engines do and leaves.  No copy is in flight, nothing faults.
#include <cuda_runtime.h>

#include "../../include/lenia_gb300.h"
#include "tma.cuh"

namespace {

__global__ void __launch_bounds__(32) wait_timeout_kernel(int max_polls, int* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    lgx::mbar_init(&bar, 2);
    lgx::fence_proxy_async();
    lgx::mbar_arrive(&bar);  // one of the two arrivals the phase needs
  }
  __syncwarp();
  const bool landed = lgx::mbar_wait(&bar, 0, max_polls);
  if (__any_sync(0xffffffffu, !landed) && threadIdx.x == 0) atomicExch(status, lgx::kStatusCopyTimeout);
  __syncwarp();
  if (threadIdx.x == 0) lgx::mbar_inval(&bar);
}

}  // namespace

extern "C" LGX_API int lgx_selftest_wait_timeout(int max_polls, int* status, void* stream) {
  if (!status || max_polls < 1) return LGX_ERR_INVALID;
  wait_timeout_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(max_polls, status);
  return cudaGetLastError() == cudaSuccess ? LGX_OK : LGX_ERR_CUDA;
}
