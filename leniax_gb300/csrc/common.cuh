// Shared device helpers of the Lenia engine: growth functions, state updates,
// raw-moment layout and small reductions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lenia_gb300.h"

namespace lgx {

constexpr float kEps = 1e-7f;  // leniax/constant.py:7

// Raw per-(world, step) moments written by the step kernels and turned into
// leniax's statistics by the stats kernel.  Coordinates are the centred ones
// of statistics.py:28-33 on the world rolled by the carried shift
// (utils.py:269-293); axis a is world axis a (outermost first).
enum RawSlot : int {
  RAW_M00 = 0,      // sum of cells
  RAW_G00 = 1,      // sum of max(field, 0)
  RAW_CNT_POT = 2,  // #(potential > eps) over all kernels
  RAW_CNT_MASS = 3, // #(cells > eps)
  RAW_CNT_GROW = 4, // #(max(field,0) > eps)
  RAW_MX = 5,       // 3 slots: sum cells * c_a
  RAW_GX = 8,       // 3 slots: sum max(field,0) * c_a
  RAW_MX2 = 11,     // 3 slots: sum cells * c_a^2
  RAW_BORDER = 14,  // 1 if a live cell (> eps) lies on the outer layer of the un-centred world
  RAW_SHIFT = 15,   // 3 slots: carried torus shift used to centre this step (per axis)
  RAW_CM = 18,      // C slots: per-channel sum of cells
};
__host__ __device__ constexpr int raw_stride(int C) { return RAW_CM + C; }

// Growth functions, leniax/growth_functions.py (same operation order).
__device__ __forceinline__ float growth_fn(int id, float x, float m, float s) {
  switch (id) {
    case LGX_GF_POLY_QUAD4: {  // growth_functions.py:38-45
      float d = x - m;
      float o = 1.f - (d * d) / (9.f * (s * s));
      o = fmaxf(0.f, o);
      o = o * o;
      o = o * o;
      return 2.f * o - 1.f;
    }
    case LGX_GF_GAUSSIAN: {  // growth_functions.py:76-82
      float d = (x - m) / s;
      float o = expf(-(d * d) / 2.f);
      return 2.f * o - 1.f;
    }
    case LGX_GF_GAUSSIAN_TARGET: {  // growth_functions.py:113-119
      float d = (x - m) / s;
      return expf(-(d * d) / 2.f);
    }
    case LGX_GF_STEP: {  // growth_functions.py:154-160
      return fabsf(x - m) <= s ? 1.f : -1.f;
    }
    case LGX_GF_STAIRCASE: {  // growth_functions.py:194-201
      float o = 0.f;
      if (x >= m - s && x < m - s / 2.f) o += 0.5f;
      if (x >= m - s / 2.f && x <= m + s / 2.f) o += 1.f;
      if (x > m + s / 2.f && x <= m + s) o += 0.5f;
      return 2.f * o - 1.f;
    }
    case LGX_GF_TRIANGLE: {  // growth_functions.py:234-243
      float left = m - s, right = m + s, o = 0.f;
      if (x >= left && x < m) o += (x - left) / (m - left);
      if (x >= m && x <= right) o += (x - right) / (m - right);
      return 2.f * o - 1.f;
    }
    default:  // LGX_GF_IDENTITY, growth_functions.py:246-253
      return x;
  }
}

// State updates, leniax/core.py:245-319.
__device__ __forceinline__ float state_fn(int id, float s, float f, float dt) {
  if (id == LGX_STATE_V1) {
    float n = s + dt * f;
    return fminf(fmaxf(n, 0.f), 1.f);
  } else if (id == LGX_STATE_V2) {
    return s * (1.f - dt) + dt * f;
  }
  return s + dt * f;
}

// Growth-function specialisations of the per-cell epilogue.
constexpr int GF_GENERIC = 0, GF_FAST_GAUSSIAN = 1, GF_FAST_POLY4 = 2;

__device__ __forceinline__ float fast_exp2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Per-world growth parameters.  The gaussian family uses
// exp(-d^2/2) = 2^(-(d*sqrt(log2(e)/2))^2): the scale folds 1/s and that
// constant, so a cell costs one subtract, two multiplies and one ex2.
struct GrowthP {
  float m, s, a;  // a: gaussian scale or 1/(9 s^2)
  int id;
};

// The fast growth forms are 2 e(x) - 1; growth_core returns e(x), so a
// weighted sum of growths can accumulate 2 w e(x) and subtract sum(w) once.
template <int GF>
__device__ __forceinline__ float growth_core(const GrowthP& g, float x) {
  static_assert(GF == GF_FAST_GAUSSIAN || GF == GF_FAST_POLY4, "2 e(x) - 1 forms only");
  if constexpr (GF == GF_FAST_GAUSSIAN) {
    const float d = (x - g.m) * g.a;
    return fast_exp2(-(d * d));
  } else {
    const float d = x - g.m;
    float o = fmaxf(0.f, fmaf(-(d * d), g.a, 1.f));
    o = o * o;
    return o * o;
  }
}

template <int GF>
__device__ __forceinline__ float growth_cell(const GrowthP& g, float x) {
  if constexpr (GF == GF_FAST_GAUSSIAN) {
    const float d = (x - g.m) * g.a;
    return fmaf(2.f, fast_exp2(-(d * d)), -1.f);
  } else if constexpr (GF == GF_FAST_POLY4) {
    const float d = x - g.m;
    float o = fmaxf(0.f, fmaf(-(d * d), g.a, 1.f));
    o = o * o;
    return fmaf(2.f, o * o, -1.f);
  } else {
    return growth_fn(g.id, x, g.m, g.s);
  }
}

// w * growth(x): the 2 e - 1 forms fold w into one fma (bit-identical to
// growth(x) * w when w == 1, the weighted_mean case of a single kernel)
template <int GF>
__device__ __forceinline__ float weighted_growth(const GrowthP& g, float x, float w) {
  if constexpr (GF == GF_GENERIC) return growth_cell<GF>(g, x) * w;
  else return fmaf(2.f * w, growth_core<GF>(g, x), -w);
}

// growth_core of a cell pair on the packed FP32x2 pipe (gaussian form:
// -(u a)^2 evaluated as u^2 (-a^2)).
template <int GF>
__device__ __forceinline__ float2 growth_core2(const GrowthP& g, float2 p) {
  static_assert(GF == GF_FAST_GAUSSIAN || GF == GF_FAST_POLY4, "2 e(x) - 1 forms only");
  const float2 u = __fadd2_rn(p, make_float2(-g.m, -g.m));
  const float2 u2 = __fmul2_rn(u, u);
  if constexpr (GF == GF_FAST_GAUSSIAN) {
    const float na2 = -(g.a * g.a);
    const float2 q = __fmul2_rn(u2, make_float2(na2, na2));
    return make_float2(fast_exp2(q.x), fast_exp2(q.y));
  } else {
    const float2 t = __ffma2_rn(u2, make_float2(-g.a, -g.a), make_float2(1.f, 1.f));
    float2 o = make_float2(fmaxf(0.f, t.x), fmaxf(0.f, t.y));
    o = __fmul2_rn(o, o);
    return __fmul2_rn(o, o);
  }
}

// weighted_growth of a cell pair.
template <int GF>
__device__ __forceinline__ float2 weighted_growth2(const GrowthP& g, float2 p, float w) {
  if constexpr (GF == GF_FAST_GAUSSIAN || GF == GF_FAST_POLY4) {
    return __ffma2_rn(make_float2(2.f * w, 2.f * w), growth_core2<GF>(g, p), make_float2(-w, -w));
  } else {
    return make_float2(weighted_growth<GF>(g, p.x, w), weighted_growth<GF>(g, p.y, w));
  }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums of 16 values across the warp in 16 shuffles (one per value would take
// 80): at each butterfly level a lane keeps half of its values and sends the
// other half to its partner.  Returns, in lane L, the warp total of value
// L >> 1 (lanes L and L ^ 1 hold the same total).
__device__ __forceinline__ float warp_sum16(float (&v)[16]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int lvl = 0; lvl < 4; ++lvl) {
    const int mask = 16 >> lvl, half = 8 >> lvl;
    const bool hi = (lane & mask) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = hi ? v[i] : v[half + i];
      const float keep = hi ? v[half + i] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, mask);
    }
  }
  return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// Named barrier over `count` threads (count a multiple of 32).
__device__ __forceinline__ void named_bar(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Non-negative modulo for the carried torus shift (jnp `%`, statistics.py:119).
__device__ __forceinline__ int pmod(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}

}  // namespace lgx
