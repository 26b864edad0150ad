// C ABI of the uneven-batch engine (lgx_batch_*): job validation, workspace
// layout, spectrum preparation, the device work queue, the mixed persistent
// launch and the statistics of every class.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"
#include "engine.h"

using namespace lgx;

namespace {

int bfail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int bfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return api_error(code, buf);
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

int kind_of(int nb_dims, int size) {
  if (nb_dims == 2) {
    switch (size) {
      case 32: return BK_R32;
      case 64: return BK_R64;
      case 128: return BK_R128;
      case 256: return BK_B2D256;
    }
  } else if (nb_dims == 3) {
    switch (size) {
      case 32: return BK_B3D32;
      case 64: return BK_B3D64;
    }
  }
  return -1;
}

bool is_big(int kind) { return kind >= BK_B2D256; }

long cells_of(const lgx_batch_class& c) {
  long n = 1;
  for (int i = 0; i < c.nb_dims; ++i) n *= c.size;
  return n;
}

// Prepared spectrum elements (float2) of one world.
long kp_elems(int kind, int N) {
  if (kind == BK_B3D32 || kind == BK_B3D64) return (long)N * N * (N / 2 + 1);
  return (long)N * (N / 2 + 2);
}

// Estimated time of one work item, in units of one 128^2 resident item; used
// by LGX_ORDER_LARGEST_FIRST only (the autotuner measures real costs).
double item_cost(int kind) {
  switch (kind) {
    case BK_R32: return 0.45;
    case BK_R64: return 0.9;
    case BK_R128: return 1.0;
    case BK_B2D256: return 5.0;
    case BK_B3D32: return 3.0;
    case BK_B3D64: return 30.0;
  }
  return 1.0;
}

int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

int validate(const lgx_batch_job* j) {
  if (!j) return bfail(LGX_ERR_INVALID, "lgx_batch: null job");
  if (j->n_classes < 1 || j->n_classes > LGX_BATCH_MAX_CLASSES || !j->classes)
    return bfail(LGX_ERR_INVALID, "lgx_batch: n_classes must be in [1, %d] with a classes array", LGX_BATCH_MAX_CLASSES);
  if (j->steps < 0) return bfail(LGX_ERR_INVALID, "lgx_batch: steps must be >= 0 (got %d)", j->steps);
  if (j->order != LGX_ORDER_LARGEST_FIRST && j->order != LGX_ORDER_AS_GIVEN && j->order != LGX_ORDER_EXPLICIT)
    return bfail(LGX_ERR_INVALID, "lgx_batch: unknown order %d", j->order);
  if (j->order == LGX_ORDER_EXPLICIT) {
    if (!j->class_order) return bfail(LGX_ERR_INVALID, "lgx_batch: LGX_ORDER_EXPLICIT needs class_order");
    bool seen[LGX_BATCH_MAX_CLASSES] = {false};
    for (int r = 0; r < j->n_classes; ++r) {
      const int c = j->class_order[r];
      if (c < 0 || c >= j->n_classes || seen[c])
        return bfail(LGX_ERR_INVALID, "lgx_batch: class_order is not a permutation of 0..%d", j->n_classes - 1);
      seen[c] = true;
    }
  }
  if (j->grid < 0) return bfail(LGX_ERR_INVALID, "lgx_batch: grid must be >= 0");
  if (j->line_group != 0 && j->line_group != 2 && j->line_group != 4)
    return bfail(LGX_ERR_INVALID, "lgx_batch: line_group must be 0, 2 or 4 (got %d)", j->line_group);
  for (int i = 0; i < j->n_classes; ++i) {
    const lgx_batch_class& c = j->classes[i];
    if (kind_of(c.nb_dims, c.size) < 0)
      return bfail(LGX_ERR_UNSUPPORTED, "lgx_batch: class %d: no engine for %dD worlds of side %d "
                                        "(2D 32/64/128/256, 3D 32/64)", i, c.nb_dims, c.size);
    if (c.n_worlds < 0) return bfail(LGX_ERR_INVALID, "lgx_batch: class %d: n_worlds < 0", i);
    if (c.gf_id < LGX_GF_POLY_QUAD4 || c.gf_id > LGX_GF_IDENTITY)
      return bfail(LGX_ERR_UNSUPPORTED, "lgx_batch: class %d: unknown growth function id %d", i, c.gf_id);
    if (c.state_fn < LGX_STATE_V1 || c.state_fn > LGX_STATE_SIMPLE)
      return bfail(LGX_ERR_INVALID, "lgx_batch: class %d: unknown state function id %d", i, c.state_fn);
    if (c.n_worlds == 0) continue;
    if (!c.cells0 || !c.k_half || !c.gf_params || !c.weights || !c.T || !c.final_cells)
      return bfail(LGX_ERR_INVALID, "lgx_batch: class %d: null input or output tensor", i);
    const bool want_stats = c.stats || c.n_continue || c.n_box || c.centroid;
    if (want_stats && (!c.stats_R || !c.stats_T))
      return bfail(LGX_ERR_INVALID, "lgx_batch: class %d: statistics need stats_R and stats_T", i);
  }
  return LGX_OK;
}

struct Layout {
  int grid;
  long scratch_per_cta;
  size_t status_off, cls_off, items_off, head_off, scratch_off, end;
  size_t kp_off[LGX_BATCH_MAX_CLASSES], raw_off[LGX_BATCH_MAX_CLASSES];
  int n_items[LGX_BATCH_MAX_CLASSES];
  int total_items;
};

Layout layout_of(const lgx_batch_job* j) {
  Layout L;
  std::memset(&L, 0, sizeof(L));
  size_t off = 0;
  L.status_off = off;  // first int: device status word (lgx_workspace_status)
  off = al256(off + sizeof(int));
  L.cls_off = off;
  off = al256(off + sizeof(BatchClassArgs) * kMaxBatchClasses);
  for (int i = 0; i < j->n_classes; ++i) {
    const lgx_batch_class& c = j->classes[i];
    const int kind = kind_of(c.nb_dims, c.size);
    const int wpi = batch_worlds_per_item(kind);
    L.n_items[i] = (c.n_worlds + wpi - 1) / wpi;
    L.total_items += L.n_items[i];
    if (is_big(kind) && c.n_worlds > 0) L.scratch_per_cta = std::max(L.scratch_per_cta, batch_scratch_per_cta(kind));
  }
  L.items_off = off;
  off = al256(off + sizeof(int2) * std::max(L.total_items, 1));
  L.head_off = off;
  off = al256(off + 64);
  for (int i = 0; i < j->n_classes; ++i) {
    const lgx_batch_class& c = j->classes[i];
    const int kind = kind_of(c.nb_dims, c.size);
    L.kp_off[i] = off;
    off = al256(off + sizeof(float2) * (size_t)c.n_worlds * kp_elems(kind, c.size));
    L.raw_off[i] = off;
    off = al256(off + sizeof(float) * (size_t)c.n_worlds * std::max(j->steps, 1) * raw_stride(1));
  }
  const int sms = sm_count();
  L.grid = j->grid > 0 ? j->grid : sms;
  L.grid = std::max(1, std::min(L.grid, std::max(L.total_items, 1)));
  L.scratch_off = off;
  off = al256(off + sizeof(float2) * (size_t)L.grid * L.scratch_per_cta);
  L.end = off;
  return L;
}

}  // namespace

namespace lgx {

size_t big_rollout_setup_bytes(int n_worlds) {
  return al256(sizeof(BatchClassArgs) * kMaxBatchClasses) + al256(sizeof(int2) * std::max(n_worlds, 1)) + 256;
}

long big_kind_scratch(int nb_dims, int size) {
  const int kind = kind_of(nb_dims, size);
  return kind >= 0 && is_big(kind) ? batch_scratch_per_cta(kind) : 0;
}

cudaError_t launch_big_rollout(int nb_dims, int size, const BigArgs& b, int gf_id, int grid, void* setup_ws,
                               cudaStream_t st) {
  const int kind = kind_of(nb_dims, size);
  if (kind < 0 || !is_big(kind)) return cudaErrorInvalidValue;
  BatchSetup su;
  std::memset(&su, 0, sizeof(su));
  su.cls[0].kind = kind;
  su.cls[0].gf_variant = batch_kind_gf_variant(gf_id);
  su.cls[0].line_group = 4;
  su.cls[0].b = b;
  su.n_cls = 1;
  su.n_items = b.n_worlds;
  su.cls_of_rank[0] = 0;
  su.first_item[0] = 0;
  for (int r = 1; r <= kMaxBatchClasses; ++r) su.first_item[r] = b.n_worlds;
  char* base = static_cast<char*>(setup_ws);
  su.cls_out = reinterpret_cast<BatchClassArgs*>(base);
  su.items = reinterpret_cast<int2*>(base + al256(sizeof(BatchClassArgs) * kMaxBatchClasses));
  su.head = reinterpret_cast<int*>(base + al256(sizeof(BatchClassArgs) * kMaxBatchClasses) +
                                   al256(sizeof(int2) * std::max(b.n_worlds, 1)));
  cudaError_t e = launch_batch_setup(su, st);
  if (e != cudaSuccess) return e;
  MixedArgs ma;
  ma.n_items = b.n_worlds;
  ma.n_cls = 1;
  ma.items = su.items;
  ma.head = su.head;
  ma.cls = su.cls_out;
  return launch_mixed(ma, grid, st);
}

}  // namespace lgx

extern "C" {

int lgx_batch_workspace_bytes(const lgx_batch_job* j, size_t* bytes) {
  if (!bytes) return bfail(LGX_ERR_INVALID, "lgx_batch_workspace_bytes: null output");
  *bytes = 0;
  const int v = validate(j);
  if (v != LGX_OK) return v;
  *bytes = layout_of(j).end;
  return LGX_OK;
}

int lgx_batch_run(const lgx_batch_job* j, void* ws, size_t ws_bytes, void* stream) {
  const int v = validate(j);
  if (v != LGX_OK) return v;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (j->steps == 0) {  // the final cells are the initial cells; no statistics rows
    for (int i = 0; i < j->n_classes; ++i) {
      const lgx_batch_class& c = j->classes[i];
      if (c.n_worlds == 0) continue;
      cudaError_t e = cudaMemcpyAsync(c.final_cells, c.cells0, sizeof(float) * c.n_worlds * cells_of(c),
                                      cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return bfail(LGX_ERR_CUDA, "lgx_batch_run copy: %s", cudaGetErrorString(e));
    }
    return LGX_OK;
  }
  const Layout L = layout_of(j);
  if (!ws || ws_bytes < L.end)
    return bfail(LGX_ERR_WORKSPACE, "lgx_batch_run: workspace %zu < %zu bytes", ws_bytes, L.end);
  char* base = static_cast<char*>(ws);
  cudaError_t e = cudaMemsetAsync(base + L.status_off, 0, sizeof(int), st);  // status word
  if (e != cudaSuccess) return bfail(LGX_ERR_CUDA, "lgx_batch_run memset: %s", cudaGetErrorString(e));

  BatchSetup su;
  std::memset(&su, 0, sizeof(su));
  const int lg = j->line_group == 0 ? 4 : j->line_group;
  int n_active = 0;
  int rank_cls[LGX_BATCH_MAX_CLASSES];
  for (int q = 0; q < j->n_classes; ++q) {
    const int i = j->order == LGX_ORDER_EXPLICIT ? j->class_order[q] : q;
    const lgx_batch_class& c = j->classes[i];
    const int kind = kind_of(c.nb_dims, c.size);
    BatchClassArgs& a = su.cls[i];
    a.kind = kind;
    a.gf_variant = batch_kind_gf_variant(c.gf_id);
    a.line_group = lg;
    if (c.n_worlds == 0) continue;
    float2* kp = reinterpret_cast<float2*>(base + L.kp_off[i]);
    float* raw = reinterpret_cast<float*>(base + L.raw_off[i]);
    const float2* kh = reinterpret_cast<const float2*>(c.k_half);
    if (kind == BK_B3D32 || kind == BK_B3D64) e = launch_prepare_3d_spectrum(c.size, c.n_worlds, kh, kp, st);
    else e = launch_prepare_resident_spectrum(c.size, c.n_worlds, kh, kp, st);
    if (e != cudaSuccess) return bfail(LGX_ERR_CUDA, "lgx_batch_run prepare: %s", cudaGetErrorString(e));
    if (is_big(kind)) {
      BigArgs& b = a.b;
      b.n_worlds = c.n_worlds;
      b.n_init = 1;
      b.steps = j->steps;
      b.gf_id = c.gf_id;
      b.state_fn = c.state_fn;
      b.mean = c.mean;
      b.cells0 = c.cells0;
      b.kp = kp;
      b.gf = c.gf_params;
      b.w = c.weights;
      b.T = c.T;
      b.state = c.final_cells;
      b.raw = raw;
      b.scratch = reinterpret_cast<float2*>(base + L.scratch_off);
      b.scratch_per_cta = L.scratch_per_cta;
      b.status = reinterpret_cast<int*>(base + L.status_off);
    } else {
      ResidentArgs& r = a.r;
      r.n_worlds = c.n_worlds;
      r.n_init = 1;
      r.steps = j->steps;
      r.gf_id = c.gf_id;
      r.state_fn = c.state_fn;
      r.mean = c.mean;
      r.cells0 = c.cells0;
      r.kp = kp;
      r.gf = c.gf_params;
      r.w = c.weights;
      r.T = c.T;
      r.final_cells = c.final_cells;
      r.raw = raw;
    }
    rank_cls[n_active++] = i;
  }
  if (n_active == 0) return LGX_OK;
  if (j->order == LGX_ORDER_LARGEST_FIRST)
    std::stable_sort(rank_cls, rank_cls + n_active,
                     [&](int x, int y) { return item_cost(su.cls[x].kind) > item_cost(su.cls[y].kind); });
  su.n_cls = j->n_classes;
  su.n_items = L.total_items;
  int pos = 0;
  for (int r = 0; r < n_active; ++r) {
    su.cls_of_rank[r] = rank_cls[r];
    su.first_item[r] = pos;
    pos += L.n_items[rank_cls[r]];
  }
  // ranks past n_active start at n_items, so the setup kernel never selects them
  for (int r = n_active; r <= kMaxBatchClasses; ++r) su.first_item[r] = pos;
  su.cls_out = reinterpret_cast<BatchClassArgs*>(base + L.cls_off);
  su.items = reinterpret_cast<int2*>(base + L.items_off);
  su.head = reinterpret_cast<int*>(base + L.head_off);
  e = launch_batch_setup(su, st);
  if (e != cudaSuccess) return bfail(LGX_ERR_CUDA, "lgx_batch_run setup: %s", cudaGetErrorString(e));

  MixedArgs ma;
  ma.n_items = L.total_items;
  ma.n_cls = j->n_classes;
  ma.items = su.items;
  ma.head = su.head;
  ma.cls = su.cls_out;
  e = launch_mixed(ma, L.grid, st);
  if (e != cudaSuccess) return bfail(LGX_ERR_CUDA, "lgx_batch_run mixed kernel: %s", cudaGetErrorString(e));

  for (int i = 0; i < j->n_classes; ++i) {
    const lgx_batch_class& c = j->classes[i];
    if (c.n_worlds == 0 || !(c.stats || c.n_continue || c.n_box || c.centroid)) continue;
    StatsArgs sa;
    std::memset(&sa, 0, sizeof(sa));
    sa.n_sols = c.n_worlds;
    sa.n_init = 1;
    sa.steps = j->steps;
    sa.C = 1;
    sa.nb_dims = c.nb_dims;
    for (int d = 0; d < 3; ++d) sa.world[d] = d < c.nb_dims ? c.size : 1;
    sa.R = 1.f;
    sa.T = 1.f;
    sa.R_arr = c.stats_R;
    sa.T_arr = c.stats_T;
    sa.raw = reinterpret_cast<const float*>(base + L.raw_off[i]);
    sa.stats = c.stats;
    sa.n_continue = c.n_continue;
    sa.n_box = c.n_box;
    sa.centroid = c.centroid;
    e = launch_stats(sa, st);
    if (e != cudaSuccess) return bfail(LGX_ERR_CUDA, "lgx_batch_run stats: %s", cudaGetErrorString(e));
  }
  return LGX_OK;
}

}  // extern "C"
