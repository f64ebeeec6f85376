// Device-side helpers: nonuniform point generation and kernel taps.
#pragma once

#include "cov3d_internal.cuh"

namespace cov3d {

__device__ __forceinline__ int pmod(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}

// torch.remainder(x + pi, 2 pi) - pi in float32 (poses.py:259-261, nufft_plan.py:327).
__device__ __forceinline__ float wrap_pi(float x) {
  const float two_pi = 6.28318530717958647692f;
  float a = __fadd_rn(x, kPiF);
  float q = floorf(__fdiv_rn(a, two_pi));
  float r = __fsub_rn(a, __fmul_rn(q, two_pi));
  return __fsub_rn(r, kPiF);
}

// Normalised plane coordinate ceil(i - Lp/2) / (Lp/2) in float32 (ASPIRE grid definition used
// by poses.py:197-213), times float32(pi).
__device__ __forceinline__ float plane_coord(int i, const PointGeom &g) {
  float k = ceilf((float)i - 0.5f * (float)g.Lp);
  return __fmul_rn(kPiF, __fdiv_rn(k, g.plane_half));
}

// Frequency (radians) of point `id` along volume axes 0, 1, 2.
__device__ __forceinline__ void point_freq(const PointGeom &g, int64_t id, float w[3]) {
  const int64_t b = id / g.P;
  const int p = (int)(id - b * g.P);
  if (g.kind == kPointsExplicit) {
    const float *base = g.pts + b * 3 * (int64_t)g.P + p;
    w[0] = __ldg(base);
    w[1] = __ldg(base + g.P);
    w[2] = __ldg(base + 2 * (int64_t)g.P);
    if (g.wrap) {
      w[0] = wrap_pi(w[0]);
      w[1] = wrap_pi(w[1]);
      w[2] = wrap_pi(w[2]);
    }
  } else {
    const float *R = g.rot + b * 9;
    const int row = p / g.Lp;
    const int col = p - row * g.Lp;
    const float x = plane_coord(col, g);
    const float y = plane_coord(row, g);
    // pts = flip_axis0(R @ [x, y, 0]): axis 0 <- row 2 of R, axis 2 <- row 0 of R
    w[0] = wrap_pi(__fadd_rn(__fmul_rn(__ldg(R + 6), x), __fmul_rn(__ldg(R + 7), y)));
    w[1] = wrap_pi(__fadd_rn(__fmul_rn(__ldg(R + 3), x), __fmul_rn(__ldg(R + 4), y)));
    w[2] = wrap_pi(__fadd_rn(__fmul_rn(__ldg(R + 0), x), __fmul_rn(__ldg(R + 1), y)));
  }
}

// Fractional centered-grid index of a frequency.
__device__ __forceinline__ float freq_to_index(const PointGeom &g, float w) {
  if (g.mapping == kMapES) {
    return __fadd_rn(__fmul_rn(w, g.s_es), g.half_n);
  }
  // NufftPlanDiscretized.setpts scaling (nufft_plan.py:113-116), then grid_sample's
  // align_corners unnormalisation ((x + 1) / 2) * (n - 1).
  float x = __fadd_rn(__fmul_rn(w, g.gs_scale), g.gs_off);
  return __fmul_rn(__fmul_rn(__fadd_rn(x, 1.0f), 0.5f), (float)(g.n - 1));
}

__device__ __forceinline__ void point_index(const PointGeom &g, int64_t id, float t[3]) {
  float w[3];
  point_freq(g, id, w);
  t[0] = freq_to_index(g, w[0]);
  t[1] = freq_to_index(g, w[1]);
  t[2] = freq_to_index(g, w[2]);
}

// First cell of a point's window along one axis.
template <int KT, int W>
__device__ __forceinline__ int first_cell(float t) {
  if (KT == COV3D_KERNEL_NEAREST) return (int)rintf(t);
  if (KT == COV3D_KERNEL_LINEAR) return (int)floorf(t);
  return (int)ceilf(t - 0.5f * (float)W);
}

// Kernel taps along one axis: window cells c0 .. c0+W-1 and their weights.
template <int KT, int W>
__device__ __forceinline__ int taps(float t, float beta, float *wt) {
  if (KT == COV3D_KERNEL_NEAREST) {
    wt[0] = 1.0f;
    return (int)rintf(t);
  } else if (KT == COV3D_KERNEL_LINEAR) {
    const float f0 = floorf(t);
    wt[0] = (f0 + 1.0f) - t;
    wt[1] = t - f0;
    return (int)f0;
  } else {
    const int c0 = (int)ceilf(t - 0.5f * (float)W);
    const float inv_half = 2.0f / (float)W;
#pragma unroll
    for (int j = 0; j < W; ++j) {
      const float x = (t - (float)(c0 + j)) * inv_half;
      const float u = 1.0f - x * x;
      wt[j] = u > 0.0f ? expf(beta * (sqrtf(u) - 1.0f)) : 0.0f;
    }
    return c0;
  }
}

}  // namespace cov3d
