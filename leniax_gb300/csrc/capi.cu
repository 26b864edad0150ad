// C ABI of the GB300 Lenia engine: plan validation, workspace layout and
// dispatch to the resident / streamed / plain engines.  See
// include/lenia_gb300.h for the contract.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "common.cuh"
#include "engine.h"

using namespace lgx;

struct lgx_plan {
  Model m;
  int adjoint_engine;  // LGX_ENGINE_AUTO or LGX_ENGINE_ND (lgx_plan_set_adjoint_engine)
};

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(LGX_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

}  // namespace

int lgx::api_error(int code, const char* msg) {
  g_err = msg;
  return code;
}

// Unique id of the current driver context (cuCtxGetCurrent + cuCtxGetId,
// fetched through the runtime's driver entry points, so the library does not
// link the driver library itself).  Returns false when it cannot be read.
bool lgx::current_context_id(unsigned long long* id) {
  typedef int (*GetCurrent)(void**);
  typedef int (*GetId)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag looked_up;
  std::call_once(looked_up, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  void* ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx) return false;
  return get_id(ctx, id) == 0;
}

namespace {

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// Bump allocator over a caller-owned workspace.  `fits()` tells whether the
// layout carved so far stays inside the caller's bytes; every entry point
// checks it before launching anything.
struct Carve {
  char* base;
  size_t off = 0, cap;
  Carve(void* b, size_t c) : base(static_cast<char*>(b)), cap(c) {}
  template <class T>
  T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base + off);
    off = al256(off + count * sizeof(T));
    return p;
  }
  bool fits() const { return off <= cap; }
};

// 3D worlds of side 32 / 64 with one channel and one kernel: one world per CTA
// (the plane-fused items of the mixed kernel).
bool cta_supported(const Model& m) {
  return m.nb_dims == 3 && m.C == 1 && m.K == 1 && m.D == m.H && m.H == m.W && (m.H == 32 || m.H == 64);
}

int select_engine(const Model& m, int requested) {
  if (requested == LGX_ENGINE_RESIDENT) return resident_supported(m) ? LGX_ENGINE_RESIDENT : -1;
  if (requested == LGX_ENGINE_STREAMED) return streamed_supported(m) ? LGX_ENGINE_STREAMED : -1;
  if (requested == LGX_ENGINE_PLAIN)
    return resident_supported(m) ? LGX_ENGINE_PLAIN : (streamed_supported(m) ? LGX_ENGINE_PLAIN_STREAMED : -1);
  if (requested == LGX_ENGINE_PLAIN_STREAMED) return streamed_supported(m) ? LGX_ENGINE_PLAIN_STREAMED : -1;
  if (requested == LGX_ENGINE_CTA) return cta_supported(m) ? LGX_ENGINE_CTA : -1;
  if (requested == LGX_ENGINE_ND) return nd_supported(m) ? LGX_ENGINE_ND : -1;
  if (requested != LGX_ENGINE_AUTO) return -1;
  if (resident_supported(m)) return LGX_ENGINE_RESIDENT;
  // even sides that are not powers of two: the N-D engine measured 1.1-1.7x
  // the mixed-radix streamed step at C = K = 1 (48^2, 72^2, 112^2) and the
  // same at C = 3, K = 15 (96^2); the streamed step stays available on request
  if (streamed_supported(m) && !(generic_size(m.H) && nd_supported(m))) return LGX_ENGINE_STREAMED;
  if (cta_supported(m)) return LGX_ENGINE_CTA;
  if (nd_supported(m)) return LGX_ENGINE_ND;
  return -1;
}

int sm_count_now() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// Every lgx_run / lgx_update workspace starts with a 256-byte status block
// (first int: device status word, see lgx_workspace_status).
constexpr size_t kStatusBytes = 256;

size_t resident_ws(const Model& m, int n_sols, int n_init, int steps) {
  size_t b = kStatusBytes;
  b += al256((size_t)n_sols * m.H * resident_kpitch(m.H) * sizeof(float2));
  b += al256((size_t)n_sols * std::max(steps, 1) * n_init * raw_stride(m.C) * sizeof(float));
  return b;
}

// CTA engine layout: status, prepared spectra [Ns, N, N, N/2+1], raw moments,
// class table + queue, state [nw, N^3] (when the caller wants no final cells),
// per-CTA spectrum scratch.
struct CtaLayout {
  size_t kp, raw, setup, state, scratch, end;
  int grid;
};

CtaLayout cta_layout(const Model& m, int n_sols, int n_init, int steps) {
  CtaLayout L;
  const int nw = n_sols * n_init;
  const size_t N = (size_t)m.H;
  size_t off = kStatusBytes;
  L.kp = off;
  off += al256((size_t)n_sols * N * N * (N / 2 + 1) * sizeof(float2));
  L.raw = off;
  off += al256((size_t)n_sols * std::max(steps, 1) * n_init * raw_stride(m.C) * sizeof(float));
  L.setup = off;
  off += al256(big_rollout_setup_bytes(nw));
  L.state = off;
  off += al256((size_t)nw * m.cells * sizeof(float));
  L.grid = std::max(1, std::min(nw, sm_count_now()));
  L.scratch = off;
  off += al256((size_t)L.grid * big_kind_scratch(m.nb_dims, m.H) * sizeof(float2));
  L.end = off;
  return L;
}

// One world and one Euler step per launch through the resident kernel: the
// resident layout plus a state ping-pong and the carried shifts.
size_t plain_ws(const Model& m, int n_sols, int n_init, int steps) {
  const size_t nw = (size_t)n_sols * n_init;
  return resident_ws(m, n_sols, n_init, steps) + 2 * al256(nw * m.C * m.cells * sizeof(float)) +
         al256(nw * 2 * sizeof(int));
}

size_t streamed_ws(const Model& m, int n_sols, int n_init, int steps, bool with_raw) {
  const int nw = n_sols * n_init;
  size_t b = kStatusBytes + streamed_workspace_bytes(m, nw, n_sols);
  b += 2 * al256((size_t)nw * m.C * m.cells * sizeof(float));  // state ping-pong
  if (with_raw) b += al256((size_t)n_sols * std::max(steps, 1) * n_init * raw_stride(m.C) * sizeof(float));
  return b;
}

// General N-D engine: status, prepared spectra, raw moments, state ping-pong,
// carried shifts, the step's own buffers.
struct NdLayout {
  size_t kf, raw, sa, sb, shift, step, end;
};

NdLayout nd_layout(const Model& m, int n_sols, int n_init, int steps) {
  NdLayout L;
  const size_t nw = (size_t)n_sols * n_init;
  size_t off = kStatusBytes;
  L.kf = off;
  off += nd_prepared_bytes(m, n_sols);
  L.raw = off;
  off += al256((size_t)n_sols * std::max(steps, 1) * n_init * raw_stride(m.C) * sizeof(float));
  L.sa = off;
  off += al256(nw * m.C * m.cells * sizeof(float));
  L.sb = off;
  off += al256(nw * m.C * m.cells * sizeof(float));
  L.shift = off;  // [nw, 3] carried shifts, then [nw] block counters of the N-D epilogue
  off += al256(nw * 4 * sizeof(int));
  L.step = off;
  off += nd_step_workspace_bytes(m, (int)nw);
  L.end = off;
  return L;
}

struct StreamedBufs {
  float2 *spec, *prod, *kp;
  float* partial;
  int *shift, *status;
  float *sa, *sb, *raw;
  size_t used;  // bytes of the layout
};

StreamedBufs carve_streamed(const Model& m, int n_sols, int n_init, int steps, void* ws, size_t ws_bytes,
                            bool with_raw) {
  Carve cv(ws, ws_bytes);
  const int nw = n_sols * n_init;
  StreamedBufs b;
  b.status = cv.take<int>(kStatusBytes / sizeof(int));
  b.spec = cv.take<float2>((size_t)nw * m.C * m.cells / 2);
  b.prod = cv.take<float2>((size_t)nw * m.K * m.cells / 2);
  b.kp = cv.take<float2>((size_t)n_sols * m.C * m.max_k * m.H * (m.W / 2 + 2));
  b.partial = cv.take<float>((size_t)nw * streamed_blocks_per_world(m) * raw_stride(m.C));
  b.shift = cv.take<int>((size_t)nw * 3);
  b.sa = cv.take<float>((size_t)nw * m.C * m.cells);
  b.sb = cv.take<float>((size_t)nw * m.C * m.cells);
  b.raw = with_raw ? cv.take<float>((size_t)n_sols * std::max(steps, 1) * n_init * raw_stride(m.C)) : nullptr;
  b.used = cv.off;
  return b;
}

}  // namespace

extern "C" {

int lgx_version(void) { return LGX_ABI_VERSION; }

const char* lgx_last_error(void) { return g_err.c_str(); }

int lgx_plan_create(const lgx_model_desc* d, lgx_plan** out) {
  if (!d || !out) return fail(LGX_ERR_INVALID, "lgx_plan_create: null argument");
  *out = nullptr;
  if (d->nb_dims != 2 && d->nb_dims != 3) return fail(LGX_ERR_INVALID, "nb_dims must be 2 or 3 (got %d)", d->nb_dims);
  if (d->nb_channels < 1 || d->nb_channels > kMaxChannels)
    return fail(LGX_ERR_INVALID, "nb_channels must be in [1, %d] (got %d)", kMaxChannels, d->nb_channels);
  if (d->nb_kernels < 1 || d->nb_kernels > kMaxKernels)
    return fail(LGX_ERR_INVALID, "nb_kernels must be in [1, %d] (got %d)", kMaxKernels, d->nb_kernels);
  if (d->max_k < 1) return fail(LGX_ERR_INVALID, "max_k must be >= 1");
  if (!d->kernel_cin || !d->kernel_slot || !d->growth_fn) return fail(LGX_ERR_INVALID, "null kernel table");
  if (d->state_fn < LGX_STATE_V1 || d->state_fn > LGX_STATE_SIMPLE)
    return fail(LGX_ERR_INVALID, "unknown state function id %d", d->state_fn);
  Model m;
  std::memset(&m, 0, sizeof(m));
  m.nb_dims = d->nb_dims;
  for (int i = 0; i < d->nb_dims; ++i) {
    if (!nd_side_ok(d->world[i]))
      return fail(LGX_ERR_UNSUPPORTED,
                  "world axis %d has size %d: sides from 2 to %d whose prime factors are 2, 3, 5 and 7", i,
                  d->world[i], nd_max_side());
    m.world[i] = d->world[i];
  }
  m.C = d->nb_channels;
  m.K = d->nb_kernels;
  m.max_k = d->max_k;
  int per_ch[kMaxChannels] = {0};
  for (int k = 0; k < m.K; ++k) {
    const int c = d->kernel_cin[k], s = d->kernel_slot[k], g = d->growth_fn[k];
    if (c < 0 || c >= m.C) return fail(LGX_ERR_INVALID, "kernel %d reads channel %d of %d", k, c, m.C);
    if (s < 0 || s >= m.max_k) return fail(LGX_ERR_INVALID, "kernel %d slot %d >= max_k %d", k, s, m.max_k);
    if (g < LGX_GF_POLY_QUAD4 || g > LGX_GF_IDENTITY)
      return fail(LGX_ERR_UNSUPPORTED, "kernel %d: unknown growth function id %d", k, g);
    m.cin[k] = c;
    m.slot[k] = s;
    m.gf[k] = g;
    per_ch[c]++;
  }
  for (int c = 0; c < m.C; ++c)
    if (per_ch[c] > m.max_k) return fail(LGX_ERR_INVALID, "channel %d has more kernels than max_k", c);
  m.state_fn = d->state_fn;
  m.mean = d->weighted_average ? 1 : 0;
  if (m.nb_dims == 2) {
    m.D = 1;
    m.H = m.world[0];
    m.W = m.world[1];
  } else {
    m.D = m.world[0];
    m.H = m.world[1];
    m.W = m.world[2];
  }
  m.cells = (long)m.D * m.H * m.W;
  lgx_plan* p = new (std::nothrow) lgx_plan;
  if (!p) return fail(LGX_ERR_INVALID, "out of host memory");
  p->m = m;
  p->adjoint_engine = LGX_ENGINE_AUTO;
  *out = p;
  g_err.clear();
  return LGX_OK;
}

void lgx_plan_destroy(lgx_plan* plan) { delete plan; }

int lgx_select_engine(const lgx_plan* plan, int n_sols, int n_init, int requested) {
  if (!plan || n_sols < 1 || n_init < 1) return -1;
  return select_engine(plan->m, requested);
}

size_t lgx_run_workspace_bytes(const lgx_plan* plan, int n_sols, int n_init, int steps, int engine) {
  if (!plan || n_sols < 1 || n_init < 1 || steps < 0) return 0;
  const int e = select_engine(plan->m, engine);
  if (e == LGX_ENGINE_RESIDENT) return resident_ws(plan->m, n_sols, n_init, steps);
  if (e == LGX_ENGINE_STREAMED || e == LGX_ENGINE_PLAIN_STREAMED)
    return streamed_ws(plan->m, n_sols, n_init, steps, true);
  if (e == LGX_ENGINE_PLAIN) return plain_ws(plan->m, n_sols, n_init, steps);
  if (e == LGX_ENGINE_ND) return nd_layout(plan->m, n_sols, n_init, steps).end;
  if (e == LGX_ENGINE_CTA) return cta_layout(plan->m, n_sols, n_init, steps).end;
  return 0;
}

int lgx_run(const lgx_plan* plan, const lgx_rollout* j, void* ws, size_t ws_bytes, void* stream) {
  if (!plan || !j) return fail(LGX_ERR_INVALID, "lgx_run: null plan or job");
  const Model& m = plan->m;
  if (j->n_sols < 1 || j->n_init < 1 || j->steps < 0)
    return fail(LGX_ERR_INVALID, "lgx_run: bad batch (n_sols=%d n_init=%d steps=%d)", j->n_sols, j->n_init, j->steps);
  if (!j->cells0 || !j->k_half || !j->gf_params || !j->weights || !j->T)
    return fail(LGX_ERR_INVALID, "lgx_run: null input tensor");
  if (!(j->stats_R > 0.f) || !(j->stats_T > 0.f)) return fail(LGX_ERR_INVALID, "lgx_run: stats_R and stats_T must be > 0");
  const int e = select_engine(m, j->engine);
  if (e < 0) return fail(LGX_ERR_UNSUPPORTED, "lgx_run: no engine for this model (engine=%d, C=%d, K=%d, size=%d)",
                         j->engine, m.C, m.K, m.H);
  const size_t need = lgx_run_workspace_bytes(plan, j->n_sols, j->n_init, j->steps, e);
  if (!ws || ws_bytes < need) return fail(LGX_ERR_WORKSPACE, "lgx_run: workspace %zu < %zu bytes", ws_bytes, need);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nw = j->n_sols * j->n_init;
  const size_t plane = (size_t)m.C * m.cells;
  cudaError_t ce;
  if (j->steps == 0) {
    if (j->final_cells) {
      ce = cudaMemcpyAsync(j->final_cells, j->cells0, (size_t)nw * plane * sizeof(float), cudaMemcpyDeviceToDevice, st);
      if (ce != cudaSuccess) return cuda_fail(ce, "lgx_run copy");
    }
    if (j->n_continue) cudaMemsetAsync(j->n_continue, 0, (size_t)nw * sizeof(float), st);
    if (j->n_box) cudaMemsetAsync(j->n_box, 0, (size_t)nw * sizeof(float), st);
    return LGX_OK;
  }
  ce = cudaMemsetAsync(ws, 0, sizeof(int), st);  // status word
  if (ce != cudaSuccess) return cuda_fail(ce, "memset");
  float* raw = nullptr;
  if (e == LGX_ENGINE_CTA) {
    const CtaLayout L = cta_layout(m, j->n_sols, j->n_init, j->steps);
    char* base = static_cast<char*>(ws);
    float2* kp = reinterpret_cast<float2*>(base + L.kp);
    raw = reinterpret_cast<float*>(base + L.raw);
    ce = launch_prepare_3d_spectrum(m.H, j->n_sols, reinterpret_cast<const float2*>(j->k_half), kp, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    BigArgs b;
    std::memset(&b, 0, sizeof(b));
    b.n_worlds = nw;
    b.n_init = j->n_init;
    b.steps = j->steps;
    b.gf_id = m.gf[0];
    b.state_fn = m.state_fn;
    b.mean = m.mean;
    b.cells0 = j->cells0;
    b.kp = kp;
    b.gf = j->gf_params;
    b.w = j->weights;
    b.T = j->T;
    b.state = j->final_cells ? j->final_cells : reinterpret_cast<float*>(base + L.state);
    b.raw = raw;
    b.scratch = reinterpret_cast<float2*>(base + L.scratch);
    b.scratch_per_cta = big_kind_scratch(m.nb_dims, m.H);
    b.status = static_cast<int*>(ws);
    b.traj_cells = j->traj_cells;
    b.traj_field = j->traj_field;
    b.traj_pot = j->traj_potential;
    if (j->main_events[0]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[0]), st);
    ce = launch_big_rollout(m.nb_dims, m.H, b, m.gf[0], L.grid, base + L.setup, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "one-world-per-CTA rollout");
    if (j->main_events[1]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[1]), st);
  } else if (e == LGX_ENGINE_ND) {
    const NdLayout L = nd_layout(m, j->n_sols, j->n_init, j->steps);
    char* base = static_cast<char*>(ws);
    float2* kf = reinterpret_cast<float2*>(base + L.kf);
    raw = reinterpret_cast<float*>(base + L.raw);
    float* sa = reinterpret_cast<float*>(base + L.sa);
    float* sb = reinterpret_cast<float*>(base + L.sb);
    int* shift = reinterpret_cast<int*>(base + L.shift);
    ce = launch_nd_prepare(m, j->n_sols, reinterpret_cast<const float2*>(j->k_half), kf, st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(shift, 0, (size_t)nw * 4 * sizeof(int), st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    const long raws = raw_stride(m.C);
    const float* cur = j->cells0;
    if (j->main_events[0]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[0]), st);
    for (int s = 0; s < j->steps; ++s) {
      float* out = (s == j->steps - 1 && j->final_cells) ? j->final_cells : ((s & 1) ? sb : sa);
      NdStep ns;
      ns.state_copy = j->traj_cells ? j->traj_cells + (size_t)s * nw * plane : nullptr;
      ns.m = &m;
      ns.n_worlds = nw;
      ns.n_init = j->n_init;
      ns.state = cur;
      ns.state_out = out;
      ns.kf = kf;
      ns.kf_sol_stride = (long)m.C * m.max_k * m.cells;
      ns.gf = j->gf_params;
      ns.gf_sol_stride = 2L * m.K;
      ns.w = j->weights;
      ns.w_sol_stride = (long)m.C * m.K;
      ns.dt = j->T;
      ns.dt_mode = 2;
      ns.field_out = j->traj_field ? j->traj_field + (size_t)s * nw * plane : nullptr;
      ns.pot_out = j->traj_potential ? j->traj_potential + (size_t)s * nw * m.K * m.cells : nullptr;
      ns.raw = raw + (size_t)s * j->n_init * raws;
      ns.raw_world_stride = raws;
      ns.raw_sol_stride = (long)j->steps * j->n_init * raws;
      ns.shift = shift;
      ns.done = shift + 3 * nw;
      ns.ws = base + L.step;
      ce = launch_nd_step(ns, st);
      if (ce != cudaSuccess) return cuda_fail(ce, "N-D step");
      cur = out;
    }
    if (j->main_events[1]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[1]), st);
    if (j->final_cells && cur != j->final_cells) {
      ce = cudaMemcpyAsync(j->final_cells, cur, (size_t)nw * plane * sizeof(float), cudaMemcpyDeviceToDevice, st);
      if (ce != cudaSuccess) return cuda_fail(ce, "final copy");
    }
  } else if (e == LGX_ENGINE_PLAIN) {
    // the reference one-world-per-launch step: the resident kernel launched for
    // one world and one Euler step at a time, the carried shift chained
    // through global memory between launches
    Carve cv(ws, ws_bytes);
    cv.take<int>(kStatusBytes / sizeof(int));
    float2* kp = cv.take<float2>((size_t)j->n_sols * m.H * resident_kpitch(m.H));
    raw = cv.take<float>((size_t)j->n_sols * j->steps * j->n_init * raw_stride(m.C));
    float* sa = cv.take<float>((size_t)nw * plane);
    float* sb = cv.take<float>((size_t)nw * plane);
    int* shift = cv.take<int>((size_t)nw * 2);
    if (!cv.fits()) return fail(LGX_ERR_WORKSPACE, "lgx_run: internal workspace layout exceeds its size query");
    ce = launch_prepare_resident_spectrum(m.H, j->n_sols, reinterpret_cast<const float2*>(j->k_half), kp, st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(shift, 0, (size_t)nw * 2 * sizeof(int), st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    const long kps = (long)m.H * resident_kpitch(m.H);
    const int raws = raw_stride(m.C);
    const float* cur = j->cells0;
    if (j->main_events[0]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[0]), st);
    for (int s = 0; s < j->steps; ++s) {
      float* out = (s == j->steps - 1 && j->final_cells) ? j->final_cells : ((s & 1) ? sb : sa);
      for (int wdx = 0; wdx < nw; ++wdx) {
        const int sol = wdx / j->n_init, init = wdx % j->n_init;
        ResidentArgs a;
        std::memset(&a, 0, sizeof(a));
        a.n_worlds = 1;
        a.n_init = 1;
        a.steps = 1;
        a.gf_id = m.gf[0];
        a.state_fn = m.state_fn;
        a.mean = m.mean;
        a.cells0 = cur + (size_t)wdx * plane;
        a.kp = kp + sol * kps;
        a.gf = j->gf_params + 2 * sol;
        a.w = j->weights + sol;
        a.T = j->T + sol;
        a.final_cells = out + (size_t)wdx * plane;
        a.raw = raw + (((size_t)sol * j->steps + s) * j->n_init + init) * raws;
        const size_t tr = ((size_t)s * nw + wdx) * plane;
        a.traj_cells = j->traj_cells ? j->traj_cells + tr : nullptr;
        a.traj_field = j->traj_field ? j->traj_field + tr : nullptr;
        a.traj_pot = j->traj_potential ? j->traj_potential + tr : nullptr;
        a.shift_in = shift + 2 * wdx;
        a.shift_out = shift + 2 * wdx;
        ce = launch_resident(m.H, a, 1, st);
        if (ce != cudaSuccess) return cuda_fail(ce, "plain step");
      }
      cur = out;
    }
    if (j->main_events[1]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[1]), st);
    if (j->final_cells && cur != j->final_cells) {
      ce = cudaMemcpyAsync(j->final_cells, cur, (size_t)nw * plane * sizeof(float), cudaMemcpyDeviceToDevice, st);
      if (ce != cudaSuccess) return cuda_fail(ce, "final copy");
    }
  } else if (e == LGX_ENGINE_RESIDENT) {
    Carve cv(ws, ws_bytes);
    cv.take<int>(kStatusBytes / sizeof(int));
    float2* kp = cv.take<float2>((size_t)j->n_sols * m.H * resident_kpitch(m.H));
    raw = cv.take<float>((size_t)j->n_sols * j->steps * j->n_init * raw_stride(m.C));
    if (!cv.fits()) return fail(LGX_ERR_WORKSPACE, "lgx_run: internal workspace layout exceeds its size query");
    ce = launch_prepare_resident_spectrum(m.H, j->n_sols, reinterpret_cast<const float2*>(j->k_half), kp, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    ResidentArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n_worlds = nw;
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
    a.no_stats = (j->stats || j->n_continue || j->n_box || j->centroid) ? 0 : 1;
    const int wpc = 512 / ((m.H / 2) * (m.H == 128 ? 8 : 4));
    const int items = (nw + wpc - 1) / wpc;
    const int grid = std::max(1, std::min(items, resident_max_grid(m.H)));
    if (j->main_events[0]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[0]), st);
    ce = launch_resident(m.H, a, grid, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "resident kernel");
    if (j->main_events[1]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[1]), st);
  } else {
    StreamedBufs b = carve_streamed(m, j->n_sols, j->n_init, j->steps, ws, ws_bytes, true);
    if (b.used > ws_bytes) return fail(LGX_ERR_WORKSPACE, "lgx_run: internal workspace layout exceeds its size query");
    raw = b.raw;
    ce = launch_prepare_streamed_spectrum(m, j->n_sols, reinterpret_cast<const float2*>(j->k_half), b.kp, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    ce = cudaMemsetAsync(b.shift, 0, (size_t)nw * 3 * sizeof(int), st);
    if (ce != cudaSuccess) return cuda_fail(ce, "memset");
    const long kp_sol = (long)m.C * m.max_k * m.H * (m.W / 2 + 2);
    const long raws = raw_stride(m.C);
    const bool plain = (e == LGX_ENGINE_PLAIN_STREAMED);
    const float* cur = j->cells0;
    if (j->main_events[0]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[0]), st);
    for (int s = 0; s < j->steps; ++s) {
      float* out = (s == j->steps - 1 && j->final_cells) ? j->final_cells : ((s & 1) ? b.sb : b.sa);
      if (j->traj_cells) {
        ce = cudaMemcpyAsync(j->traj_cells + (size_t)s * nw * plane, cur, (size_t)nw * plane * sizeof(float),
                             cudaMemcpyDeviceToDevice, st);
        if (ce != cudaSuccess) return cuda_fail(ce, "trajectory copy");
      }
      StreamedStep ss;
      ss.m = &m;
      ss.kp_sol_stride = kp_sol;
      ss.gf_sol_stride = 2L * m.K;
      ss.w_sol_stride = (long)m.C * m.K;
      ss.dt_mode = 2;
      ss.raw_sol_stride = (long)j->steps * j->n_init * raws;
      ss.raw_world_stride = raws;
      if (!plain) {
        ss.n_worlds = nw;
        ss.n_init = j->n_init;
        ss.state = cur;
        ss.state_out = out;
        ss.kp = b.kp;
        ss.gf = j->gf_params;
        ss.w = j->weights;
        ss.dt = j->T;
        ss.field_out = j->traj_field ? j->traj_field + (size_t)s * nw * plane : nullptr;
        ss.pot_out = j->traj_potential ? j->traj_potential + (size_t)s * nw * m.K * m.cells : nullptr;
        ss.raw = raw + (size_t)s * j->n_init * raws;
        ss.shift = b.shift;
        ss.spec = b.spec;
        ss.prod = b.prod;
        ss.partial = b.partial;
        ss.status = b.status;
        // the row inverse of step s writes the row spectra step s + 1 starts from
        ss.spec_ready = s > 0;
        ss.emit_spec = s + 1 < j->steps;
        ce = launch_streamed_step(ss, st);
        if (ce != cudaSuccess) return cuda_fail(ce, "streamed step");
      } else {
        // one world per launch: the reference one-world-per-launch kernel sequence
        for (int wdx = 0; wdx < nw; ++wdx) {
          const int sol = wdx / j->n_init, init = wdx % j->n_init;
          ss.n_worlds = 1;
          ss.n_init = 1;
          ss.state = cur + (size_t)wdx * plane;
          ss.state_out = out + (size_t)wdx * plane;
          ss.kp = b.kp + sol * kp_sol;
          ss.gf = j->gf_params + (size_t)sol * 2 * m.K;
          ss.w = j->weights + (size_t)sol * m.C * m.K;
          ss.dt = j->T + sol;
          ss.field_out = j->traj_field ? j->traj_field + ((size_t)s * nw + wdx) * plane : nullptr;
          ss.pot_out = j->traj_potential ? j->traj_potential + ((size_t)s * nw + wdx) * m.K * m.cells : nullptr;
          ss.raw = raw + (((size_t)sol * j->steps + s) * j->n_init + init) * raws;
          ss.shift = b.shift + 3 * wdx;
          ss.spec = b.spec;
          ss.prod = b.prod;
          ss.partial = b.partial;
          ss.status = b.status;
          ss.spec_ready = false;  // one world per launch: the spectrum buffer is shared by all worlds
          ss.emit_spec = false;
          ce = launch_streamed_step(ss, st);
          if (ce != cudaSuccess) return cuda_fail(ce, "plain step");
        }
      }
      cur = out;
    }
    if (j->main_events[1]) cudaEventRecord(static_cast<cudaEvent_t>(j->main_events[1]), st);
    if (j->final_cells && cur != j->final_cells) {
      ce = cudaMemcpyAsync(j->final_cells, cur, (size_t)nw * plane * sizeof(float), cudaMemcpyDeviceToDevice, st);
      if (ce != cudaSuccess) return cuda_fail(ce, "final copy");
    }
  }
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
  if (ce != cudaSuccess) return cuda_fail(ce, "stats kernels");
  g_err.clear();
  return LGX_OK;
}

size_t lgx_update_workspace_bytes(const lgx_plan* plan, int n) {
  if (!plan || n < 1) return 0;
  const Model& m = plan->m;
  // lgx_update runs one streamed step for every 2D model (resident sizes
  // included) and a one-step one-world-per-CTA rollout for 3D models
  if (streamed_supported(m)) return streamed_ws(m, 1, n, 1, false);
  if (cta_supported(m)) return cta_layout(m, 1, n, 1).end;
  if (nd_supported(m)) return nd_layout(m, 1, n, 1).end;
  return 0;
}

int lgx_update(const lgx_plan* plan, int n, const float* state, const float* k_half, const float* gf_params,
               const float* weights, const float* dt, int dt_per_world, float* state_out, float* field_out,
               float* potential_out, void* ws, size_t ws_bytes, void* stream) {
  if (!plan) return fail(LGX_ERR_INVALID, "lgx_update: null plan");
  const Model& m = plan->m;
  if (n < 1) return fail(LGX_ERR_INVALID, "lgx_update: n must be >= 1");
  if (!state || !k_half || !gf_params || !weights || !dt || !state_out)
    return fail(LGX_ERR_INVALID, "lgx_update: null tensor");
  const size_t need = lgx_update_workspace_bytes(plan, n);
  if (need == 0) return fail(LGX_ERR_UNSUPPORTED, "lgx_update: no engine for this model");
  if (!ws || ws_bytes < need) return fail(LGX_ERR_WORKSPACE, "lgx_update: workspace %zu < %zu bytes", ws_bytes, need);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t ce;
  if (cta_supported(m)) {
    // 3D: one step of the plane-fused item, field and potential as its step-0 trajectory
    const CtaLayout L = cta_layout(m, 1, n, 1);
    char* base = static_cast<char*>(ws);
    ce = cudaMemsetAsync(ws, 0, sizeof(int), st);  // status word
    if (ce != cudaSuccess) return cuda_fail(ce, "memset");
    float2* kp = reinterpret_cast<float2*>(base + L.kp);
    ce = launch_prepare_3d_spectrum(m.H, 1, reinterpret_cast<const float2*>(k_half), kp, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    BigArgs b;
    std::memset(&b, 0, sizeof(b));
    b.n_worlds = n;
    b.n_init = n;  // every world belongs to the one solution
    b.steps = 1;
    b.gf_id = m.gf[0];
    b.state_fn = m.state_fn;
    b.mean = m.mean;
    b.cells0 = state;
    b.kp = kp;
    b.gf = gf_params;
    b.w = weights;
    b.dt = dt;
    b.dt_mode = dt_per_world ? 2 : 1;
    b.state = state_out;
    b.raw = reinterpret_cast<float*>(base + L.raw);
    b.scratch = reinterpret_cast<float2*>(base + L.scratch);
    b.scratch_per_cta = big_kind_scratch(m.nb_dims, m.H);
    b.status = static_cast<int*>(ws);
    b.traj_field = field_out;
    b.traj_pot = potential_out;
    ce = launch_big_rollout(m.nb_dims, m.H, b, m.gf[0], L.grid, base + L.setup, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "3D update");
    g_err.clear();
    return LGX_OK;
  }
  if (!streamed_supported(m) && nd_supported(m)) {
    // one step of the general N-D engine, scalar or per-world dt
    const NdLayout L = nd_layout(m, 1, n, 1);
    char* base = static_cast<char*>(ws);
    float2* kf = reinterpret_cast<float2*>(base + L.kf);
    int* shift = reinterpret_cast<int*>(base + L.shift);
    ce = cudaMemsetAsync(ws, 0, sizeof(int), st);
    if (ce == cudaSuccess) ce = launch_nd_prepare(m, 1, reinterpret_cast<const float2*>(k_half), kf, st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(shift, 0, (size_t)n * 4 * sizeof(int), st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    NdStep ns;
    ns.state_copy = nullptr;
    ns.done = shift + 3 * n;
    ns.m = &m;
    ns.n_worlds = n;
    ns.n_init = n;
    ns.state = state;
    ns.state_out = state_out;
    ns.kf = kf;
    ns.kf_sol_stride = 0;
    ns.gf = gf_params;
    ns.gf_sol_stride = 0;
    ns.w = weights;
    ns.w_sol_stride = 0;
    ns.dt = dt;
    ns.dt_mode = dt_per_world ? 1 : 0;
    ns.field_out = field_out;
    ns.pot_out = potential_out;
    ns.raw = nullptr;
    ns.raw_world_stride = 0;
    ns.raw_sol_stride = 0;
    ns.shift = shift;
    ns.ws = base + L.step;
    ce = launch_nd_step(ns, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "N-D update");
    g_err.clear();
    return LGX_OK;
  }
  if (!streamed_supported(m) && !resident_supported(m)) return fail(LGX_ERR_UNSUPPORTED, "lgx_update: unsupported");
  if (streamed_supported(m)) {
    StreamedBufs b = carve_streamed(m, 1, n, 1, ws, ws_bytes, false);
    if (b.used > ws_bytes) return fail(LGX_ERR_WORKSPACE, "lgx_update: internal workspace layout exceeds its size query");
    ce = cudaMemsetAsync(b.status, 0, sizeof(int), st);
    if (ce != cudaSuccess) return cuda_fail(ce, "memset");
    ce = launch_prepare_streamed_spectrum(m, 1, reinterpret_cast<const float2*>(k_half), b.kp, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
    ce = cudaMemsetAsync(b.shift, 0, (size_t)n * 3 * sizeof(int), st);
    if (ce != cudaSuccess) return cuda_fail(ce, "memset");
    StreamedStep ss;
    ss.m = &m;
    ss.n_worlds = n;
    ss.n_init = n;
    ss.state = state;
    ss.state_out = state_out;
    ss.kp = b.kp;
    ss.kp_sol_stride = 0;
    ss.gf = gf_params;
    ss.gf_sol_stride = 0;
    ss.w = weights;
    ss.w_sol_stride = 0;
    ss.dt = dt;
    ss.dt_mode = dt_per_world ? 1 : 0;
    ss.field_out = field_out;
    ss.pot_out = potential_out;
    ss.raw = nullptr;
    ss.raw_world_stride = 0;
    ss.raw_sol_stride = 0;
    ss.shift = b.shift;
    ss.spec = b.spec;
    ss.prod = b.prod;
    ss.partial = b.partial;
    ss.status = b.status;
    ss.spec_ready = false;
    ss.emit_spec = false;
    ce = launch_streamed_step(ss, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "update step");
    g_err.clear();
    return LGX_OK;
  }
  return fail(LGX_ERR_UNSUPPORTED, "lgx_update: unsupported world size");
}

int lgx_workspace_status(const void* ws, void* stream, int* status) {
  if (!ws || !status) return fail(LGX_ERR_INVALID, "lgx_workspace_status: null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t ce = cudaMemcpyAsync(status, ws, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) return cuda_fail(ce, "lgx_workspace_status");
  return LGX_OK;
}

}  // extern "C"

// Read-only view of a plan's model for other translation units of the engine.
namespace lgx {
const Model* plan_model(const lgx_plan* plan) { return plan ? &plan->m : nullptr; }
}  // namespace lgx

// ------------------------------------------------------------------ adjoint
namespace {

// The general N-D adjoint runs every model the one-kernel adjoint does not,
// and every model when the plan asks for it.
bool adjoint_is_nd(const lgx_plan& p) { return p.adjoint_engine == LGX_ENGINE_ND || !adjoint_supported(p.m); }

size_t adjoint_ws(const Model& m, int n_sols, int n_init) {
  const size_t nw = (size_t)n_sols * n_init, cells = (size_t)m.H * m.W;
  size_t b = 0;
  b += al256((size_t)n_sols * m.H * (m.W / 2 + 2) * sizeof(float2));  // kp
  b += 2 * al256(nw * cells * sizeof(float));                         // lam_a, lam_b
  b += al256(nw * cells * sizeof(float2));                            // spec (2 planes x N/2 x N)
  b += al256(nw * cells / 2 * sizeof(float2));                        // prod
  b += al256(nw * 64 * 3 * sizeof(float));                            // partial
  return b;
}

}  // namespace

extern "C" {

int lgx_plan_set_adjoint_engine(lgx_plan* plan, int engine) {
  if (!plan) return fail(LGX_ERR_INVALID, "lgx_plan_set_adjoint_engine: null plan");
  if (engine != LGX_ENGINE_AUTO && engine != LGX_ENGINE_ND)
    return fail(LGX_ERR_INVALID, "lgx_plan_set_adjoint_engine: LGX_ENGINE_AUTO or LGX_ENGINE_ND");
  if (engine == LGX_ENGINE_ND && !nd_supported(plan->m))
    return fail(LGX_ERR_UNSUPPORTED, "lgx_plan_set_adjoint_engine: no N-D adjoint for this model");
  plan->adjoint_engine = engine;
  g_err.clear();
  return LGX_OK;
}

size_t lgx_adjoint_workspace_bytes(const lgx_plan* plan, int n_sols, int n_init) {
  if (!plan || n_sols < 1 || n_init < 1) return 0;
  if (!adjoint_is_nd(*plan)) return adjoint_supported(plan->m) ? adjoint_ws(plan->m, n_sols, n_init) : 0;
  return nd_supported(plan->m) ? nd_adjoint_workspace_bytes(plan->m, n_sols, n_init) : 0;
}

size_t lgx_adjoint_kernel_grad_acc_bytes(const lgx_plan* plan, int n_sols, int n_init) {
  if (!plan || n_sols < 1 || n_init < 1) return 0;
  const Model& m = plan->m;
  if (!adjoint_is_nd(*plan))
    return adjoint_supported(m) ? (size_t)n_sols * n_init * (m.H / 2) * m.W * sizeof(float2) : 0;
  return nd_supported(m) ? nd_kernel_grad_acc_bytes(m, n_sols, n_init) : 0;
}

int lgx_adjoint(const lgx_plan* plan, const lgx_adjoint_job* j, void* ws, size_t ws_bytes, void* stream) {
  if (!plan || !j) return fail(LGX_ERR_INVALID, "lgx_adjoint: null plan or job");
  const Model& m = plan->m;
  if (!(adjoint_is_nd(*plan) ? nd_supported(m) : adjoint_supported(m)))
    return fail(LGX_ERR_UNSUPPORTED, "lgx_adjoint: no adjoint for this model");
  if (j->n_sols < 1 || j->n_init < 1 || j->steps < 1) return fail(LGX_ERR_INVALID, "lgx_adjoint: bad batch");
  if (!j->k_half || !j->gf_params || !j->weights || !j->T || !j->traj_cells || !j->traj_potential ||
      !j->lambda_in || !j->lambda_out || !j->kernel_grad_acc || !j->grad_gf || !j->grad_weights)
    return fail(LGX_ERR_INVALID, "lgx_adjoint: null tensor");
  if (j->lambda_in == j->lambda_out) return fail(LGX_ERR_INVALID, "lgx_adjoint: lambda_out aliases lambda_in");
  if (j->clip_grad != LGX_CLIP_GRAD_STE && j->clip_grad != LGX_CLIP_GRAD_MASK)
    return fail(LGX_ERR_INVALID, "lgx_adjoint: unknown clip_grad %d", j->clip_grad);
  const bool use_nd = adjoint_is_nd(*plan);
  const size_t need = lgx_adjoint_workspace_bytes(plan, j->n_sols, j->n_init);
  if (!ws || ws_bytes < need) return fail(LGX_ERR_WORKSPACE, "lgx_adjoint: workspace %zu < %zu bytes", ws_bytes, need);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (use_nd) {
    // the general N-D adjoint: any channels and kernels, 2D and 3D worlds
    NdAdjoint a;
    a.n_sols = j->n_sols;
    a.n_init = j->n_init;
    a.steps = j->steps;
    a.clip_mask = j->clip_grad == LGX_CLIP_GRAD_MASK;
    a.k_half = reinterpret_cast<const float2*>(j->k_half);
    a.gf_params = j->gf_params;
    a.weights = j->weights;
    a.T = j->T;
    a.traj_cells = j->traj_cells;
    a.traj_potential = j->traj_potential;
    a.lambda_in = j->lambda_in;
    a.lambda_out = j->lambda_out;
    a.gk = reinterpret_cast<float2*>(j->kernel_grad_acc);
    a.grad_gf = j->grad_gf;
    a.grad_weights = j->grad_weights;
    a.cells_after = j->cells_after;
    cudaError_t ce = launch_nd_adjoint(m, a, ws, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "N-D adjoint segment");
    g_err.clear();
    return LGX_OK;
  }
  const size_t nw = (size_t)j->n_sols * j->n_init, cells = (size_t)m.H * m.W;
  Carve cv(ws, ws_bytes);
  AdjointSegment a;
  std::memset(&a, 0, sizeof(a));
  float2* kp = cv.take<float2>((size_t)j->n_sols * m.H * (m.W / 2 + 2));
  a.lam_a = cv.take<float>(nw * cells);
  a.lam_b = cv.take<float>(nw * cells);
  a.spec = cv.take<float2>(nw * cells);
  a.prod = cv.take<float2>(nw * cells / 2);
  a.partial = cv.take<float>(nw * 64 * 3);
  if (!cv.fits()) return fail(LGX_ERR_WORKSPACE, "lgx_adjoint: internal workspace layout exceeds its size query");
  // the resident adjoint reads the row-major prepared planes, the streamed one
  // the column-major planes
  const bool resident = adjoint_resident_supported(m);
  cudaError_t ce =
      resident ? launch_prepare_resident_spectrum(m.H, j->n_sols, reinterpret_cast<const float2*>(j->k_half), kp, st)
               : launch_prepare_streamed_spectrum(m, j->n_sols, reinterpret_cast<const float2*>(j->k_half), kp, st);
  if (ce != cudaSuccess) return cuda_fail(ce, "prepare spectrum");
  a.n_sols = j->n_sols;
  a.n_init = j->n_init;
  a.steps = j->steps;
  a.gf_id = m.gf[0];
  a.state_fn = m.state_fn;
  a.mean = m.mean;
  a.clip_mask = j->clip_grad == LGX_CLIP_GRAD_MASK;
  a.gf_params = j->gf_params;
  a.weights = j->weights;
  a.T = j->T;
  a.kp = kp;
  a.traj_cells = j->traj_cells;
  a.traj_potential = j->traj_potential;
  a.lambda_in = j->lambda_in;
  a.lambda_out = j->lambda_out;
  a.gk = reinterpret_cast<float2*>(j->kernel_grad_acc);
  a.grad_gf = j->grad_gf;
  a.grad_w = j->grad_weights;
  a.cells_after = j->cells_after;
  if (resident) {
    // resident sizes: one persistent launch for the whole segment
    AdjResArgs r;
    r.n_worlds = (int)nw;
    r.n_init = j->n_init;
    r.steps = j->steps;
    r.gf_id = a.gf_id;
    r.state_fn = a.state_fn;
    r.mean = a.mean;
    r.clip_mask = a.clip_mask;
    r.gf = j->gf_params;
    r.w = j->weights;
    r.T = j->T;
    r.kp = kp;
    r.traj_cells = j->traj_cells;
    r.traj_pot = j->traj_potential;
    r.lambda_in = j->lambda_in;
    r.lambda_out = j->lambda_out;
    r.gk = reinterpret_cast<float2*>(j->kernel_grad_acc);
    r.pacc = a.partial;
    r.cells_after = j->cells_after;
    ce = cudaMemsetAsync(a.partial, 0, nw * 3 * sizeof(float), st);
    if (ce == cudaSuccess) ce = launch_adjoint_resident(m.H, r, st);
    if (ce == cudaSuccess) ce = launch_param_reduce(j->n_sols, j->n_init, 1, a.partial, j->grad_gf, j->grad_weights, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "resident adjoint segment");
  } else {
    ce = launch_adjoint_segment(m.H, a, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "adjoint segment");
  }
  g_err.clear();
  return LGX_OK;
}

int lgx_adjoint_kernel_grad(const lgx_plan* plan, int n_sols, int n_init, const float* acc, float* grad_kernel,
                            void* ws, size_t ws_bytes, void* stream) {
  if (!plan || !acc || !grad_kernel) return fail(LGX_ERR_INVALID, "lgx_adjoint_kernel_grad: null argument");
  const Model& m = plan->m;
  if (lgx_adjoint_workspace_bytes(plan, 1, 1) == 0)
    return fail(LGX_ERR_UNSUPPORTED, "lgx_adjoint_kernel_grad: unsupported model");
  if (n_sols < 1 || n_init < 1) return fail(LGX_ERR_INVALID, "lgx_adjoint_kernel_grad: bad batch");
  const size_t need = lgx_adjoint_workspace_bytes(plan, n_sols, n_init);
  if (!ws || ws_bytes < need)
    return fail(LGX_ERR_WORKSPACE, "lgx_adjoint_kernel_grad: workspace %zu < %zu bytes", ws_bytes, need);
  if (adjoint_is_nd(*plan)) {
    cudaError_t ce = launch_nd_kernel_grad(m, n_sols, n_init, reinterpret_cast<const float2*>(acc), grad_kernel, ws,
                                           static_cast<cudaStream_t>(stream));
    if (ce != cudaSuccess) return cuda_fail(ce, "kernel gradient");
    g_err.clear();
    return LGX_OK;
  }
  float2* prod = reinterpret_cast<float2*>(ws);
  cudaError_t ce = launch_gk_finish(m.H, n_sols, n_init, reinterpret_cast<const float2*>(acc), prod, grad_kernel,
                                    static_cast<cudaStream_t>(stream));
  if (ce != cudaSuccess) return cuda_fail(ce, "kernel gradient");
  g_err.clear();
  return LGX_OK;
}

size_t lgx_kernel_spectrum_nd_workspace_bytes(int nb_dims, const int* world, int planes) {
  if ((nb_dims != 2 && nb_dims != 3) || !world || planes < 1) return 0;
  for (int i = 0; i < nb_dims; ++i)
    if (!nd_side_ok(world[i])) return 0;
  return nd_spectrum_workspace_bytes(nb_dims, world, planes);
}

int lgx_kernel_spectrum_nd(int nb_dims, const int* world, int planes, const float* k_real, float* k_half, void* ws,
                           size_t ws_bytes, void* stream) {
  if (!k_real || !k_half || !world || planes < 1) return fail(LGX_ERR_INVALID, "lgx_kernel_spectrum_nd: bad argument");
  const size_t need = lgx_kernel_spectrum_nd_workspace_bytes(nb_dims, world, planes);
  if (need == 0)
    return fail(LGX_ERR_UNSUPPORTED, "lgx_kernel_spectrum_nd: 2D / 3D worlds with sides of factors 2, 3, 5, 7 only");
  if (!ws || ws_bytes < need)
    return fail(LGX_ERR_WORKSPACE, "lgx_kernel_spectrum_nd: workspace %zu < %zu", ws_bytes, need);
  cudaError_t ce = launch_nd_spectrum(nb_dims, world, planes, k_real, reinterpret_cast<float2*>(k_half), ws,
                                      static_cast<cudaStream_t>(stream));
  if (ce != cudaSuccess) return cuda_fail(ce, "kernel spectrum");
  g_err.clear();
  return LGX_OK;
}

int lgx_kernel_spectrum(int H, int W, int planes, const float* k_real, float* k_half, void* ws, size_t ws_bytes,
                        void* stream) {
  if (!k_real || !k_half || planes < 1) return fail(LGX_ERR_INVALID, "lgx_kernel_spectrum: bad argument");
  if (!spectrum_supported(H, W)) return fail(LGX_ERR_UNSUPPORTED, "lgx_kernel_spectrum: square 32..256 only");
  const size_t need = (size_t)planes * H * W * sizeof(float);
  if (!ws || ws_bytes < need) return fail(LGX_ERR_WORKSPACE, "lgx_kernel_spectrum: workspace %zu < %zu", ws_bytes, need);
  cudaError_t ce = launch_spectrum(H, planes, k_real, reinterpret_cast<float2*>(ws), reinterpret_cast<float2*>(k_half),
                                   static_cast<cudaStream_t>(stream));
  if (ce != cudaSuccess) return cuda_fail(ce, "kernel spectrum");
  g_err.clear();
  return LGX_OK;
}

}  // extern "C"
