// Statistics and stop heuristics from the raw per-step moments.
//
//  stats_kernel      : one thread per (sol, step, init): leniax compute_stats
//                      (statistics.py:36-126).  The carried centroid / angle of
//                      step t only depend on the moments of steps t-1 and t-2,
//                      so every step is evaluated independently.
//  heuristics_kernel : one warp per (sol, init): check_heuristics
//                      (statistics.py:134-205) -> N, and the box stop set
//                      (mass < 1e-3, mass > 0.9 * area, a live cell on the
//                      outer layer) -> N_box, 32 steps per round.
#include "common.cuh"
#include "engine.h"

namespace lgx {

namespace {

constexpr float kRad2Deg = 57.295779513082320876798f;  // 180/pi

struct Ctx {
  int nd, C, steps, n_init;
  float R, dt;
  int world[3];
  const float* R_arr;  // per-solution R (or null: R)
  const float* T_arr;  // per-solution static T (or null: 1/dt)
};

// Per-axis triples are kept as named scalars and returned by value (no
// partially written local arrays): an earlier array-based form of this kernel
// was mis-optimised by nvcc 13.0 at -O3 (correct only at -G).
struct Tri {
  float a0, a1, a2;
};

__device__ __forceinline__ const float* raw_at(const float* raw, const Ctx c, int sol, int step, int init) {
  return raw + (((size_t)sol * c.steps + step) * c.n_init + init) * raw_stride(c.C);
}

// mass centroid of a step's moments (statistics.py:83)
__device__ __forceinline__ Tri centroid(const float* r, int nd) {
  const float den = r[RAW_M00] + kEps;
  Tri o;
  o.a0 = r[RAW_MX + 0] / den;
  o.a1 = nd > 1 ? r[RAW_MX + 1] / den : 0.f;
  o.a2 = nd > 2 ? r[RAW_MX + 2] / den : 0.f;
  return o;
}

__device__ __forceinline__ Tri frac(Tri c) {  // x - trunc(x): the carried centroid (statistics.py:124)
  Tri o;
  o.a0 = c.a0 - truncf(c.a0);
  o.a1 = c.a1 - truncf(c.a1);
  o.a2 = c.a2 - truncf(c.a2);
  return o;
}

__device__ __forceinline__ Tri sub(Tri a, Tri b) {
  Tri o;
  o.a0 = a.a0 - b.a0;
  o.a1 = a.a1 - b.a1;
  o.a2 = a.a2 - b.a2;
  return o;
}

__device__ __forceinline__ float norm(Tri d, int nd) {
  float s = d.a0 * d.a0;
  if (nd > 1) s += d.a1 * d.a1;
  if (nd > 2) s += d.a2 * d.a2;
  return sqrtf(s);
}

// jnp.degrees(arctan2(delta[1], delta[0])) * (dist / R > 0.001)   (statistics.py:89)
__device__ __forceinline__ float angle_of(Tri d, float dist, float R) {
  const float ang = atan2f(d.a1, d.a0) * kRad2Deg;
  return ang * ((dist / R > 0.001f) ? 1.f : 0.f);
}

// Absolute torus position of the centroid: centred-frame centroid + N/2 +
// carried shift, wrapped to [0, N).
__device__ __forceinline__ float wrap_pos(float cen, float shift, int n) {
  float p = fmodf(cen + (float)(n / 2) + shift, (float)n);
  return p < 0.f ? p + (float)n : p;
}

__global__ void stats_kernel(Ctx c, int n_sols, const float* __restrict__ raw, float* __restrict__ stats,
                             float* __restrict__ centroid_out) {
  const long total = (long)n_sols * c.steps * c.n_init;
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int init = (int)(i % c.n_init);
  const int step = (int)((i / c.n_init) % c.steps);
  const int sol = (int)(i / ((long)c.n_init * c.steps));
  const int nd = c.nd;
  const float* r = raw_at(raw, c, sol, step, init);
  const float Rs = c.R_arr ? __ldg(c.R_arr + sol) : c.R;
  const float dts = c.T_arr ? 1.f / __ldg(c.T_arr + sol) : c.dt;
  const float R2 = Rs * Rs;
  const float m00 = r[RAW_M00], g00 = r[RAW_G00];
  const Tri zero = {0.f, 0.f, 0.f};
  const Tri cen = centroid(r, nd);
  // carried centroid entering this step, and the angle carried from the previous step
  Tri pc = zero;
  float prev_angle = 0.f;
  if (step > 0) {
    const Tri c1 = centroid(raw_at(raw, c, sol, step - 1, init), nd);
    pc = frac(c1);
    const Tri p1 = (step > 1) ? frac(centroid(raw_at(raw, c, sol, step - 2, init), nd)) : zero;
    const Tri d1 = sub(c1, p1);
    prev_angle = angle_of(d1, norm(d1, nd), Rs);
  }
  const Tri delta = sub(cen, pc);
  const float dist_m = norm(delta, nd);
  const float mass_angle = angle_of(delta, dist_m, Rs);
  // growth centroid distance and inertia (statistics.py:93-100)
  const float gden = g00 + kEps, mden = m00 * m00 + kEps;
  float gcd2, inertia;
  {
    const float g0 = r[RAW_GX + 0] / gden - cen.a0;
    gcd2 = g0 * g0;
    inertia = (r[RAW_MX2 + 0] - cen.a0 * r[RAW_MX + 0]) / mden;
    if (nd > 1) {
      const float g1 = r[RAW_GX + 1] / gden - cen.a1;
      gcd2 += g1 * g1;
      inertia += (r[RAW_MX2 + 1] - cen.a1 * r[RAW_MX + 1]) / mden;
    }
    if (nd > 2) {
      const float g2 = r[RAW_GX + 2] / gden - cen.a2;
      gcd2 += g2 * g2;
      inertia += (r[RAW_MX2 + 2] - cen.a2 * r[RAW_MX + 2]) / mden;
    }
  }
  const float ang = mass_angle - prev_angle + 540.f;  // python-style modulo (jnp %)
  float md = fmodf(ang, 360.f);
  if (md < 0.f) md += 360.f;
  const float mass = m00 / R2;
  const float mass_volume = r[RAW_CNT_MASS] / R2;
  const float growth = g00 / R2;
  const float growth_volume = r[RAW_CNT_GROW] / R2;
  if (centroid_out) {
    float* co = centroid_out + i * (size_t)nd;
    co[0] = wrap_pos(cen.a0, r[RAW_SHIFT + 0], c.world[0]);
    if (nd > 1) co[1] = wrap_pos(cen.a1, r[RAW_SHIFT + 1], c.world[1]);
    if (nd > 2) co[2] = wrap_pos(cen.a2, r[RAW_SHIFT + 2], c.world[2]);
  }
  if (!stats) return;
  float* o = stats + i * (size_t)(c.C + LGX_NSTAT_SCALAR);
  for (int ch = 0; ch < c.C; ++ch) o[ch] = r[RAW_CM + ch] / R2;
  float* s = o + c.C;
  s[0] = mass;
  s[1] = mass_volume;
  s[2] = mass / (mass_volume + kEps);
  s[3] = growth;
  s[4] = growth_volume;
  s[5] = growth / (growth_volume + kEps);
  s[6] = dist_m / Rs / dts;
  s[7] = (md - 180.f) / dts;
  s[8] = sqrtf(gcd2) / Rs;
  s[9] = inertia;
  s[10] = r[RAW_CNT_POT] / R2;
}

// One warp per (sol, init), 32 steps per round.  The scan of
// statistics.py:134-205 is rewritten in closed form so the lanes of a round
// work independently: the monotone and mass-volume counters at step t equal
// t - b + 1 with b the last reset step at or before t (a sign change, resp.
// mass_volume <= 10; step 0 counts as a reset), found with a warp max-scan
// carried across rounds; should_continue is the product of the conditions,
// so N is the first step whose condition fails (steps if none), found with a
// ballot.  The box stop set is the same first-failure search.  Results equal
// the sequential scan's (same per-step arithmetic).
__device__ __forceinline__ int warp_max_scan(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = max(v, u);
  }
  return v;
}

__global__ void heuristics_kernel(Ctx c, int n_sols, float area, const float* __restrict__ raw,
                                  float* __restrict__ n_cont, float* __restrict__ n_box) {
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n_sols * c.n_init) return;  // whole warps
  const int sol = i / c.n_init, init = i % c.n_init;
  const float Rs = c.R_arr ? __ldg(c.R_arr + sol) : c.R;
  const float R2 = Rs * Rs;
  const float* r0 = raw_at(raw, c, sol, 0, init);
  const int T = c.steps;
  int N = T, NB = T;
  bool foundN = false, foundB = false;
  float prev_mass = r0[RAW_M00] / R2, prev_sign = 0.f;  // carried into each round's lane 0
  int carry_bm = 0, carry_bv = 0;                        // last reset steps so far
  for (int t0 = 0; t0 < T && !(foundN && foundB); t0 += 32) {
    const int t = t0 + lane;
    const bool valid = t < T;
    const float* r = raw_at(raw, c, sol, valid ? t : T - 1, init);
    bool cond = true;
    for (int ch = 0; ch < c.C && ch < kMaxChannels; ++ch) {
      const float cm = r[RAW_CM + ch] / R2;
      const float cm0 = r0[RAW_CM + ch] / R2;
      cond = cond && (cm >= kEps) && (cm <= 3.f * cm0);  // statistics.py:224-251
    }
    const float mass = r[RAW_M00] / R2;
    float pm = __shfl_up_sync(0xffffffffu, mass, 1);
    if (lane == 0) pm = prev_mass;
    const float d = mass - pm;
    const float sign = d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);
    float ps = __shfl_up_sync(0xffffffffu, sign, 1);
    if (lane == 0) ps = prev_sign;
    // monotone counter (statistics.py:287-306): resets where the sign changes
    const int bm = max(warp_max_scan((t == 0 || sign != ps) ? t : -1, lane), carry_bm);
    const int c_mono = t - bm + 1;
    // mass-volume counter (statistics.py:317-333): resets where mass_volume <= 10
    const float mv = r[RAW_CNT_MASS] / R2;
    const int bv = max(warp_max_scan((t == 0 || !(mv > 10.f)) ? t : -1, lane), carry_bv);
    const int c_vol = t - bv + 1;
    cond = cond && (c_mono <= 128) && (c_vol <= 128);
    const unsigned failN = __ballot_sync(0xffffffffu, valid && !cond);
    if (!foundN && failN) {
      N = t0 + __ffs(failN) - 1;
      foundN = true;
    }
    const float raw_mass = r[RAW_M00];
    const bool bc = raw_mass >= 1e-3f && raw_mass <= 0.9f * area && r[RAW_BORDER] == 0.f;
    const unsigned failB = __ballot_sync(0xffffffffu, valid && !bc);
    if (!foundB && failB) {
      NB = t0 + __ffs(failB) - 1;
      foundB = true;
    }
    prev_mass = __shfl_sync(0xffffffffu, mass, 31);
    prev_sign = __shfl_sync(0xffffffffu, sign, 31);
    carry_bm = __shfl_sync(0xffffffffu, bm, 31);
    carry_bv = __shfl_sync(0xffffffffu, bv, 31);
  }
  if (lane == 0) {
    if (n_cont) n_cont[i] = (float)N;
    if (n_box) n_box[i] = (float)NB;
  }
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
  c.R_arr = a.R_arr;
  c.T_arr = a.T_arr;
  for (int d = 0; d < 3; ++d) c.world[d] = a.world[d];
  if (a.steps <= 0) return cudaSuccess;
  if (a.stats || a.centroid) {
    const long total = (long)a.n_sols * a.steps * a.n_init;
    stats_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c, a.n_sols, a.raw, a.stats, a.centroid);
  }
  if (a.n_continue || a.n_box) {
    float area = (float)a.C;
    for (int d = 0; d < a.nb_dims; ++d) area *= (float)a.world[d];
    const int n = a.n_sols * a.n_init;  // one warp each
    heuristics_kernel<<<(n + 7) / 8, 256, 0, st>>>(c, a.n_sols, area, a.raw, a.n_continue, a.n_box);
  }
  return cudaGetLastError();
}

}  // namespace lgx
