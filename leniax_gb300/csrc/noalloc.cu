// lgx_run_noalloc: the resident rollout with its scratch in a fixed device
// array instead of a caller-provided workspace.
//
// Who needs it: callers that cannot allocate device memory at call time.  The
// usual case is a host runtime that reserves (almost) all device memory for
// its own pool at start-up -- for example a JAX/XLA process calling this
// engine from a custom call -- where a cudaMalloc fails or competes with that
// pool, and latency-sensitive callers that must not pay for the implicit
// device synchronisation of cudaMalloc/cudaFree.  Those callers pass inputs
// and outputs only; the engine's scratch lives in the array below.
//
// Cost: every GPU that loads this library reserves LGX_NOALLOC_SCRATCH_BYTES of
// device memory for the array until the process exits.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"
#include "engine.h"

using namespace lgx;

namespace {

// The scratch of every lgx_run_noalloc call on a device: prepared spectra
// followed by the raw per-step moments.
static __device__ __align__(256) unsigned char g_noalloc_scratch[LGX_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Per device: the scratch address and the unique id of the CUDA context it was
// resolved in.  A device reset, or a caller running in another (non-primary)
// context, gives a new context id, and the address is resolved again there.
void* g_scratch_ptr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};

thread_local std::string g_na_err;

int na_fail(int code, const char* msg) {
  g_na_err = msg;
  return code;
}

// Device address of the scratch array in the current device's current
// context.  Resolved with that device current the first time a device (or a
// new context on it) is seen; in host code g_noalloc_scratch names a host-side
// shadow, never the device memory, so only this address is passed on.
int scratch_for_current_device(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return na_fail(LGX_ERR_CUDA, "lgx_run_noalloc: no current CUDA device");
  std::lock_guard<std::mutex> lk(g_mu);
  unsigned long long ctx = 0;
  if (!current_context_id(&ctx) || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    // first call on this device or in this context (cudaGetSymbolAddress also
    // binds the runtime's context when no context was current yet)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      g_na_err = std::string("lgx_run_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
      return LGX_ERR_CUDA;
    }
    if (!current_context_id(&ctx))
      return na_fail(LGX_ERR_CUDA, "lgx_run_noalloc: cannot identify the current CUDA context");
    g_scratch_ptr[dev] = p;
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return LGX_OK;
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" LGX_API size_t lgx_noalloc_scratch_bytes(const lgx_plan* plan, int n_sols, int n_init, int steps) {
  const Model* m = plan_model(plan);
  if (!m || n_sols < 1 || n_init < 1 || steps < 1) return 0;
  return al256((size_t)n_sols * m->H * resident_kpitch(m->H) * sizeof(float2)) +
         al256((size_t)n_sols * steps * n_init * raw_stride(m->C) * sizeof(float));
}

extern "C" LGX_API const char* lgx_noalloc_last_error(void) { return g_na_err.c_str(); }

extern "C" LGX_API int lgx_run_noalloc(const lgx_plan* plan, const lgx_rollout* j, void* stream) {
  const Model* mp = plan_model(plan);
  if (!mp || !j) return na_fail(LGX_ERR_INVALID, "lgx_run_noalloc: null plan or job");
  const Model& m = *mp;
  if (!resident_supported(m))
    return na_fail(LGX_ERR_UNSUPPORTED,
                   "lgx_run_noalloc: resident models only (2D, C=1, K=1, square 32/64/128 worlds)");
  if (j->n_sols < 1 || j->n_init < 1 || j->steps < 0)
    return na_fail(LGX_ERR_INVALID, "lgx_run_noalloc: need n_sols >= 1, n_init >= 1, steps >= 0");
  if (!j->cells0 || !j->k_half || !j->gf_params || !j->weights || !j->T)
    return na_fail(LGX_ERR_INVALID, "lgx_run_noalloc: null input tensor");
  if (!(j->stats_R > 0.f) || !(j->stats_T > 0.f))
    return na_fail(LGX_ERR_INVALID, "lgx_run_noalloc: stats_R and stats_T must be > 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (j->steps == 0) {  // as lgx_run: the initial cells come back, both stop counts are 0; no scratch used
    const size_t bytes = (size_t)j->n_sols * j->n_init * m.C * m.cells * sizeof(float);
    cudaError_t ce = cudaSuccess;
    if (j->final_cells) ce = cudaMemcpyAsync(j->final_cells, j->cells0, bytes, cudaMemcpyDeviceToDevice, st);
    if (ce == cudaSuccess && j->n_continue)
      ce = cudaMemsetAsync(j->n_continue, 0, (size_t)j->n_sols * j->n_init * sizeof(float), st);
    if (ce == cudaSuccess && j->n_box) ce = cudaMemsetAsync(j->n_box, 0, (size_t)j->n_sols * j->n_init * sizeof(float), st);
    if (ce != cudaSuccess) return na_fail(LGX_ERR_CUDA, cudaGetErrorString(ce));
    g_na_err.clear();
    return LGX_OK;
  }
  const size_t kp_bytes = al256((size_t)j->n_sols * m.H * resident_kpitch(m.H) * sizeof(float2));
  const size_t raw_bytes = (size_t)j->n_sols * j->steps * j->n_init * raw_stride(m.C) * sizeof(float);
  if (kp_bytes + raw_bytes > (size_t)LGX_NOALLOC_SCRATCH_BYTES) {
    char buf[256];
    snprintf(buf, sizeof(buf),
             "lgx_run_noalloc: batch needs %zu scratch bytes, more than the fixed %zu-byte array; "
             "split the batch or use lgx_run with a workspace",
             kp_bytes + raw_bytes, (size_t)LGX_NOALLOC_SCRATCH_BYTES);
    return na_fail(LGX_ERR_WORKSPACE, buf);
  }
  void* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc != LGX_OK) return rc;
  float2* kp = reinterpret_cast<float2*>(base);
  float* raw = reinterpret_cast<float*>(static_cast<char*>(base) + kp_bytes);
  // The array keeps the previous call's contents: clear the moments region so
  // no slot of this batch can read a stale value.
  cudaError_t ce = cudaMemsetAsync(raw, 0, raw_bytes, st);
  if (ce == cudaSuccess)
    ce = launch_prepare_resident_spectrum(m.H, j->n_sols, reinterpret_cast<const float2*>(j->k_half), kp, st);
  if (ce != cudaSuccess) return na_fail(LGX_ERR_CUDA, cudaGetErrorString(ce));
  ResidentArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n_worlds = j->n_sols * j->n_init;
  a.n_init = j->n_init;
  a.steps = j->steps;
  a.gf_id = m.gf[0];
  a.state_fn = m.state_fn;
  a.mean = m.mean;
  a.cells0 = j->cells0;
  a.kp = kp;
  a.gf = j->gf_params;
  a.w = j->weights;
  a.T = j->T;
  a.final_cells = j->final_cells;
  a.raw = raw;
  a.traj_cells = j->traj_cells;
  a.traj_field = j->traj_field;
  a.traj_pot = j->traj_potential;
  const int wpc = 512 / ((m.H / 2) * (m.H == 128 ? 8 : 4));
  const int items = (a.n_worlds + wpc - 1) / wpc;
  const int grid = items < resident_max_grid(m.H) ? items : resident_max_grid(m.H);
  ce = launch_resident(m.H, a, grid > 0 ? grid : 1, st);
  if (ce != cudaSuccess) return na_fail(LGX_ERR_CUDA, cudaGetErrorString(ce));
  StatsArgs sa;
  std::memset(&sa, 0, sizeof(sa));
  sa.n_sols = j->n_sols;
  sa.n_init = j->n_init;
  sa.steps = j->steps;
  sa.C = m.C;
  sa.nb_dims = m.nb_dims;
  for (int i = 0; i < 3; ++i) sa.world[i] = m.world[i];
  sa.R = j->stats_R;
  sa.T = j->stats_T;
  sa.R_arr = j->stats_R_sol;
  sa.T_arr = j->stats_T_sol;
  sa.raw = raw;
  sa.stats = j->stats;
  sa.n_continue = j->n_continue;
  sa.n_box = j->n_box;
  sa.centroid = j->centroid;
  ce = launch_stats(sa, st);
  if (ce != cudaSuccess) return na_fail(LGX_ERR_CUDA, cudaGetErrorString(ce));
  g_na_err.clear();
  return LGX_OK;
}
