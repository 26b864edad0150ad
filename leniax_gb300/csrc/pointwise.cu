// The step's pointwise stages as separate entry points, for callers that use
// leniax's building blocks directly instead of core.update:
//   lgx_growth    growth_functions.* on the potentials   [n, K, cells] -> [n, K, cells]
//   lgx_weighted  core.weighted_sum / weighted_mean      [n, K, cells] -> [n, C, cells]
//   lgx_field     core.get_field (growth + merge fused)  [n, K, cells] -> [n, C, cells]
//   lgx_state     core.get_state / _v2 / _simple         [n, C, cells] -> [n, C, cells]
// Grid-stride kernels over the cells; the arithmetic is the engines' own
// (common.cuh growth_fn / state_fn, the merge in kernel order with the
// mean's divisor summed over every kernel, core.py:202-242).
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "engine.h"

namespace lgx {
namespace {

constexpr int kPT = 256;

struct GrowthTab {
  int K;
  int id[kMaxKernels];
};

inline int pw_grid(long total) {
  return (int)std::max(1L, std::min<long>((total + kPT - 1) / kPT, 152L * 16));
}

__global__ void growth_kernel(GrowthTab g, long n_cells, long cells, const float* __restrict__ pot,
                              const float* __restrict__ gf, float* __restrict__ out) {
  // n_cells = n * K * cells; plane (world, kernel) = i / cells
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n_cells; i += (long)gridDim.x * blockDim.x) {
    const int k = (int)((i / cells) % g.K);
    out[i] = growth_fn(g.id[k], __ldg(pot + i), __ldg(gf + 2 * k), __ldg(gf + 2 * k + 1));
  }
}

// out[w, c] = sum_k w_ck f[w, k] (/ sum_k w_ck); with `growth`, f = growth_k(in)
template <bool GROWTH>
__global__ void merge_kernel(GrowthTab g, int C, int mean, long n_cells, long cells, const float* __restrict__ in,
                             const float* __restrict__ gf, const float* __restrict__ wt, float* __restrict__ out) {
  const int K = g.K;
  // n_cells = n * cells
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n_cells; i += (long)gridDim.x * blockDim.x) {
    const long w = i / cells, cell = i - w * cells;
    for (int c = 0; c < C; ++c) {
      float f = 0.f, wsum = 0.f;
      for (int k = 0; k < K; ++k) {
        const float wk = __ldg(wt + c * K + k);
        wsum += wk;
        if (wk == 0.f) continue;
        float v = __ldg(in + (w * K + k) * cells + cell);
        if (GROWTH) v = growth_fn(g.id[k], v, __ldg(gf + 2 * k), __ldg(gf + 2 * k + 1));
        f = fmaf(wk, v, f);
      }
      out[(w * C + c) * cells + cell] = mean ? f / wsum : f;
    }
  }
}

__global__ void state_kernel(int sfid, long n_cells, long per_world, const float* __restrict__ s,
                             const float* __restrict__ f, const float* __restrict__ dt, int dt_per_world,
                             float* __restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n_cells; i += (long)gridDim.x * blockDim.x) {
    const float d = __ldg(dt + (dt_per_world ? i / per_world : 0));
    out[i] = state_fn(sfid, __ldg(s + i), __ldg(f + i), d);
  }
}

bool tab_of(int K, const int* gf_ids, GrowthTab* g) {
  if (K < 1 || K > kMaxKernels || !gf_ids) return false;
  g->K = K;
  for (int k = 0; k < kMaxKernels; ++k) {
    const int id = k < K ? gf_ids[k] : 0;
    if (id < 0 || id > LGX_GF_IDENTITY) return false;
    g->id[k] = id;
  }
  return true;
}

int launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return LGX_OK;
  return api_error(LGX_ERR_CUDA, what);
}

}  // namespace
}  // namespace lgx

using namespace lgx;

extern "C" LGX_API int lgx_growth(int n, int K, long cells, const int* gf_ids, const float* potential,
                                  const float* gf_params, float* out, void* stream) {
  GrowthTab g;
  if (n < 0 || cells < 1 || !tab_of(K, gf_ids, &g)) return api_error(LGX_ERR_INVALID, "lgx_growth: bad sizes or ids");
  if (n == 0) return LGX_OK;
  if (!potential || !gf_params || !out) return api_error(LGX_ERR_INVALID, "lgx_growth: null pointer");
  const long total = (long)n * K * cells;
  growth_kernel<<<pw_grid(total), kPT, 0, static_cast<cudaStream_t>(stream)>>>(g, total, cells, potential, gf_params,
                                                                                out);
  return launched("lgx_growth: launch failed");
}

extern "C" LGX_API int lgx_weighted(int n, int K, int C, long cells, const float* fields, const float* weights,
                                    int mean, float* out, void* stream) {
  GrowthTab g;
  int ids[kMaxKernels] = {0};
  if (n < 0 || cells < 1 || C < 1 || C > kMaxChannels || !tab_of(K, ids, &g))
    return api_error(LGX_ERR_INVALID, "lgx_weighted: bad sizes");
  if (n == 0) return LGX_OK;
  if (!fields || !weights || !out) return api_error(LGX_ERR_INVALID, "lgx_weighted: null pointer");
  const long total = (long)n * cells;
  merge_kernel<false><<<pw_grid(total), kPT, 0, static_cast<cudaStream_t>(stream)>>>(g, C, mean ? 1 : 0, total, cells,
                                                                                    fields, nullptr, weights, out);
  return launched("lgx_weighted: launch failed");
}

extern "C" LGX_API int lgx_field(int n, int K, int C, long cells, const int* gf_ids, const float* potential,
                                 const float* gf_params, const float* weights, int mean, float* field, void* stream) {
  GrowthTab g;
  if (n < 0 || cells < 1 || C < 1 || C > kMaxChannels || !tab_of(K, gf_ids, &g))
    return api_error(LGX_ERR_INVALID, "lgx_field: bad sizes or ids");
  if (n == 0) return LGX_OK;
  if (!potential || !gf_params || !weights || !field) return api_error(LGX_ERR_INVALID, "lgx_field: null pointer");
  const long total = (long)n * cells;
  merge_kernel<true><<<pw_grid(total), kPT, 0, static_cast<cudaStream_t>(stream)>>>(g, C, mean ? 1 : 0, total, cells,
                                                                                   potential, gf_params, weights, field);
  return launched("lgx_field: launch failed");
}

extern "C" LGX_API int lgx_state(int n, int C, long cells, int state_fn_id, const float* state, const float* field,
                                 const float* dt, int dt_per_world, float* out, void* stream) {
  if (n < 0 || C < 1 || cells < 1 || state_fn_id < LGX_STATE_V1 || state_fn_id > LGX_STATE_SIMPLE)
    return api_error(LGX_ERR_INVALID, "lgx_state: bad sizes or state function");
  if (n == 0) return LGX_OK;
  if (!state || !field || !dt || !out) return api_error(LGX_ERR_INVALID, "lgx_state: null pointer");
  const long total = (long)n * C * cells;
  state_kernel<<<pw_grid(total), kPT, 0, static_cast<cudaStream_t>(stream)>>>(state_fn_id, total, (long)C * cells,
                                                                              state, field, dt, dt_per_world, out);
  return launched("lgx_state: launch failed");
}
