// Device-side helpers: nonuniform point generation and kernel taps.
#pragma once

#include "cov3d_internal.cuh"

namespace cov3d {

__device__ __forceinline__ int pmod(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}

// a mod n for a in [-n, 2n): the window corners of wrapped points.
__device__ __forceinline__ int wrap1(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

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

// ES kernel value exp(beta * (sqrt(1 - (2x/W)^2) - 1)) for |x| < W/2, else 0, with the fast
// hardware exponential and reciprocal square root (relative error ~1e-6, far below the ES
// approximation error of the NUFFT).
template <int W>
__device__ __forceinline__ float es_weight(float x, float beta) {
  const float y = x * (2.0f / (float)W);
  const float u = 1.0f - y * y;
  return u > 0.0f ? __expf(beta * (u * rsqrtf(u) - 1.0f)) : 0.0f;
}

// Sorted point record written by the sort: fractional grid indices along axes 0..2 and the
// point id, with kNyquistBit set when the point lies on the Nyquist row / column of an
// even-sized image (vol_forward zeroes those pixels, projection_funcs.py:355-358).
struct SortedPoint {
  float t0, t1, t2;
  int idf;
};
constexpr int kNyquistBit = 1 << 30;
__device__ __forceinline__ int sp_id(int idf) { return idf & (kNyquistBit - 1); }
__device__ __forceinline__ bool sp_nyquist(int idf) { return (idf & kNyquistBit) != 0; }

__device__ __forceinline__ bool on_nyquist(const PointGeom &g, int64_t id) {
  if (g.Lp % 2 != 0) return false;
  const int p = (int)(id % g.P);
  return p < g.Lp || (p % g.Lp) == 0;
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
#pragma unroll
    for (int j = 0; j < W; ++j) wt[j] = es_weight<W>(t - (float)(c0 + j), beta);
    return c0;
  }
}

// Weight of tap q (0 <= q < W) of the window of a point at fractional index t.
template <int KT, int W>
__device__ __forceinline__ float tap_weight(float t, int q, float beta) {
  if (KT == COV3D_KERNEL_NEAREST) return 1.0f;
  if (KT == COV3D_KERNEL_LINEAR) {
    const float f0 = floorf(t);
    return q == 0 ? (f0 + 1.0f) - t : t - f0;
  }
  const int c0 = (int)ceilf(t - 0.5f * (float)W);
  return es_weight<W>(t - (float)(c0 + q), beta);
}

// CTF at pixel offsets (ka, kb) (row, column) from the image centre: sqrt(1 - w^2) sin(gamma) -
// w cos(gamma) with gamma = c0 K + c1 D + c2 X + d K^2 - ps (see CtfCoef).  gamma reaches a few
// hundred radians at high frequency, so its large terms are formed in double-float arithmetic
// (exact products by fmaf, TwoSum), reduced modulo 2 pi by Cody-Waite with a 2 pi split into a
// 12-bit head (n * head exact for |n| < 2^12) and a float tail, and only the reduced angle goes
// to sincosf: the absolute phase error stays near float rounding of the reduced angle.
__device__ __forceinline__ float ctf_eval(const CtfCoef &c, int ka, int kb) {
  const float K = (float)(ka * ka + kb * kb), D = (float)(ka * ka - kb * kb), X = (float)(2 * ka * kb);
  const float p0 = c.c0h * K, e0 = fmaf(c.c0h, K, -p0);
  const float p1 = c.c1h * D, e1 = fmaf(c.c1h, D, -p1);
  const float p2 = c.c2h * X, e2 = fmaf(c.c2h, X, -p2);
  float s = p0 + p1;
  float bb = s - p0;
  float err = (p0 - (s - bb)) + (p1 - bb);
  const float t = s + p2;
  bb = t - s;
  err += (s - (t - bb)) + (p2 - bb);
  const float lo = err + e0 + e1 + e2 + fmaf(c.c0l, K, fmaf(c.c1l, D, c.c2l * X)) + c.d * K * K - c.ps;
  constexpr float kTwoPiHead = 6.283203125f;          // 3217 / 512
  constexpr float kTwoPiTail = -1.7817820413e-05f;    // 2 pi - head
  constexpr float kInvTwoPi = 0.15915494309189535f;
  const float nq = rintf((t + lo) * kInvTwoPi);
  float r = fmaf(-nq, kTwoPiHead, t);
  r = fmaf(-nq, kTwoPiTail, r) + lo;
  float sn, cs;
  sincosf(r, &sn, &cs);
  return c.sw * sn - c.w * cs;
}

// The CTF factor of point id: the per-pixel array, or the per-image coefficients, or 1.
__device__ __forceinline__ float ctf_factor(const float *ctf, const CtfCoef *ctfc, const PointGeom &g, int64_t id) {
  if (ctf) return __ldg(ctf + id);
  if (!ctfc) return 1.0f;
  const int64_t b = id / g.P;
  const int p = (int)(id - b * g.P);
  const int row = p / g.Lp, col = p - (p / g.Lp) * g.Lp;
  return ctf_eval(ctfc[b], row - g.Lp / 2, col - g.Lp / 2);
}

// Index maps of the fine grid (FFT-native storage: frequency / voxel offset k at k mod n).
// centered index of storage index s on a grid of size m (fftshift)
__device__ __forceinline__ int native_to_centered(int s, int m) {
  const int c = s + m / 2;
  return c >= m ? c - m : c;
}
// voxel index (0 .. L-1) of storage index s on a zero-padded axis, or -1 for padding
__device__ __forceinline__ int pad_voxel(int s, int L, int n) {
  const int h = L / 2;
  return s < L - h ? s + h : (s >= n - h ? s - n + h : -1);
}
// storage index of voxel j
__device__ __forceinline__ int voxel_store(int j, int L, int n) {
  const int k = j - L / 2;
  return k < 0 ? k + n : k;
}

}  // namespace cov3d
