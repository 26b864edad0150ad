// Statistics and stop heuristics from the raw per-step moments.
//
//  stats_kernel      : one thread per (sol, step, init): leniax compute_stats
//                      (statistics.py:36-126).  The carried centroid / angle of
//                      step t only depend on the moments of steps t-1 and t-2,
//                      so every step is evaluated independently.
//  heuristics_kernel : one thread per (sol, init): the sequential scan of
//                      check_heuristics (statistics.py:134-205) -> N, and the
//                      box stop set (mass < 1e-3, mass > 0.9 * area, a live
//                      cell on the outer layer) -> N_box.
#include "common.cuh"
#include "engine.h"

namespace lgx {

namespace {

constexpr float kRad2Deg = 57.295779513082320876798f;  // 180/pi

struct Ctx {
  int nd, C, steps, n_init;
  float R, dt;
};

__device__ __forceinline__ const float* raw_at(const float* raw, const Ctx& c, int sol, int step, int init) {
  return raw + (((size_t)sol * c.steps + step) * c.n_init + init) * raw_stride(c.C);
}

__device__ __forceinline__ void centroid(const float* r, int nd, float* out) {
  const float m00 = r[RAW_M00];
  for (int a = 0; a < nd; ++a) out[a] = r[RAW_MX + a] / (m00 + kEps);
}

// carried (fractional) centroid entering step t
__device__ __forceinline__ void prev_frac(const float* raw, const Ctx& c, int sol, int step, int init, float* out) {
  if (step == 0) {
    for (int a = 0; a < 3; ++a) out[a] = 0.f;
    return;
  }
  float cc[3] = {0.f, 0.f, 0.f};
  centroid(raw_at(raw, c, sol, step - 1, init), c.nd, cc);
  for (int a = 0; a < 3; ++a) out[a] = cc[a] - truncf(cc[a]);
}

__device__ __forceinline__ float angle_of(const float* delta, float dist, const Ctx& c) {
  const float ang = atan2f(delta[1], delta[0]) * kRad2Deg;  // jnp.degrees(arctan2(d1, d0))
  return ang * ((dist / c.R > 0.001f) ? 1.f : 0.f);
}

__global__ void stats_kernel(Ctx c, int n_sols, const float* __restrict__ raw, float* __restrict__ stats) {
  const long total = (long)n_sols * c.steps * c.n_init;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int init = (int)(i % c.n_init);
  const int step = (int)((i / c.n_init) % c.steps);
  const int sol = (int)(i / ((long)c.n_init * c.steps));
  const float* r = raw_at(raw, c, sol, step, init);
  const float R2 = c.R * c.R;
  const float m00 = r[RAW_M00], g00 = r[RAW_G00];
  float cen[3] = {0.f, 0.f, 0.f}, pc[3];
  centroid(r, c.nd, cen);
  prev_frac(raw, c, sol, step, init, pc);
  float delta[3] = {0.f, 0.f, 0.f}, d2 = 0.f;
  for (int a = 0; a < c.nd; ++a) {
    delta[a] = cen[a] - pc[a];
    d2 += delta[a] * delta[a];
  }
  const float dist_m = sqrtf(d2);
  const float mass_angle = angle_of(delta, dist_m, c);
  float prev_angle = 0.f;
  if (step > 0) {
    float c1[3] = {0.f, 0.f, 0.f}, p1[3], dl[3] = {0.f, 0.f, 0.f}, e2 = 0.f;
    centroid(raw_at(raw, c, sol, step - 1, init), c.nd, c1);
    prev_frac(raw, c, sol, step - 1, init, p1);
    for (int a = 0; a < c.nd; ++a) {
      dl[a] = c1[a] - p1[a];
      e2 += dl[a] * dl[a];
    }
    prev_angle = angle_of(dl, sqrtf(e2), c);
  }
  float gcd2 = 0.f, inertia = 0.f;
  for (int a = 0; a < c.nd; ++a) {
    const float gc = r[RAW_GX + a] / (g00 + kEps);
    gcd2 += (gc - cen[a]) * (gc - cen[a]);
    const float mux2 = r[RAW_MX2 + a] - cen[a] * r[RAW_MX + a];
    inertia += mux2 / (m00 * m00 + kEps);
  }
  float ang = mass_angle - prev_angle + 540.f;  // python-style modulo (jnp %)
  float md = fmodf(ang, 360.f);
  if (md != 0.f && md < 0.f) md += 360.f;
  const float mass = m00 / R2;
  const float mass_volume = r[RAW_CNT_MASS] / R2;
  const float growth = g00 / R2;
  const float growth_volume = r[RAW_CNT_GROW] / R2;
  float* o = stats + i * (size_t)(c.C + LGX_NSTAT_SCALAR);
  for (int ch = 0; ch < c.C; ++ch) o[ch] = r[RAW_CM + ch] / R2;
  float* s = o + c.C;
  s[0] = mass;
  s[1] = mass_volume;
  s[2] = mass / (mass_volume + kEps);
  s[3] = growth;
  s[4] = growth_volume;
  s[5] = growth / (growth_volume + kEps);
  s[6] = dist_m / c.R / c.dt;
  s[7] = (md - 180.f) / c.dt;
  s[8] = sqrtf(gcd2) / c.R;
  s[9] = inertia;
  s[10] = r[RAW_CNT_POT] / R2;
}

__global__ void heuristics_kernel(Ctx c, int n_sols, float area, const float* __restrict__ raw,
                                  float* __restrict__ n_cont, float* __restrict__ n_box) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_sols * c.n_init) return;
  const int sol = i / c.n_init, init = i % c.n_init;
  const float R2 = c.R * c.R;
  float init_cm[kMaxChannels];
  const float* r0 = raw_at(raw, c, sol, 0, init);
  for (int ch = 0; ch < c.C && ch < kMaxChannels; ++ch) init_cm[ch] = r0[RAW_CM + ch] / R2;
  float should = 1.f, N = 0.f, prev_mass = r0[RAW_M00] / R2, prev_sign = 0.f;
  int c_mono = 0, c_vol = 0;
  float box = 1.f, NB = 0.f;
  for (int t = 0; t < c.steps; ++t) {
    const float* r = raw_at(raw, c, sol, t, init);
    bool cond = true;
    for (int ch = 0; ch < c.C && ch < kMaxChannels; ++ch) {
      const float cm = r[RAW_CM + ch] / R2;
      cond = cond && (cm >= kEps) && (cm <= 3.f * init_cm[ch]);  // statistics.py:224-251
    }
    const float mass = r[RAW_M00] / R2;
    const float d = mass - prev_mass;
    const float sign = d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);
    c_mono = c_mono * (sign == prev_sign ? 1 : 0) + 1;  // statistics.py:287-306
    cond = cond && (c_mono <= 128);
    const float mv = r[RAW_CNT_MASS] / R2;
    c_vol = c_vol * (mv > 10.f ? 1 : 0) + 1;  // statistics.py:317-333
    cond = cond && (c_vol <= 128);
    should = should * (cond ? 1.f : 0.f);
    N += should;
    prev_mass = mass;
    prev_sign = sign;
    const float raw_mass = r[RAW_M00];
    const bool bc = raw_mass >= 1e-3f && raw_mass <= 0.9f * area && r[RAW_BORDER] == 0.f;
    box = box * (bc ? 1.f : 0.f);
    NB += box;
  }
  if (n_cont) n_cont[i] = N;
  if (n_box) n_box[i] = NB;
}

}  // namespace

cudaError_t launch_stats(const StatsArgs& a, cudaStream_t st) {
  Ctx c;
  c.nd = a.nb_dims;
  c.C = a.C;
  c.steps = a.steps;
  c.n_init = a.n_init;
  c.R = a.R;
  c.dt = 1.f / a.T;
  if (a.steps <= 0) return cudaSuccess;
  if (a.stats) {
    const long total = (long)a.n_sols * a.steps * a.n_init;
    stats_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c, a.n_sols, a.raw, a.stats);
  }
  if (a.n_continue || a.n_box) {
    float area = (float)a.C;
    for (int d = 0; d < a.nb_dims; ++d) area *= (float)a.world[d];
    const int n = a.n_sols * a.n_init;
    heuristics_kernel<<<(n + 127) / 128, 128, 0, st>>>(c, a.n_sols, area, a.raw, a.n_continue, a.n_box);
  }
  return cudaGetLastError();
}

}  // namespace lgx
