// Hand-written line DFTs of the fine grid: register radix-4 DFTs combined by a four-step
// decomposition, one shared-memory exchange per transform.  They carry the pruned 3D
// transforms of the mean CG's padding operator and of the covariance step (pack, forward
// transform and regulariser; inverse transform and unpack), each fused with the elementwise
// work around it, for fine grids of n = 128, 256, 512 (and the axis-0 CG kernel also for 64).
// Twiddles exp(-2 pi i j / n) are computed on the host in double precision.

#include <cmath>
#include <vector>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

// DFT of N values held in registers (natural order in, natural order out), recursive
// decimation in time, radix 4 (radix 2 for the last factor when N is not a power of 4);
// w[j] = exp(-2 pi i j / n) is the n-point twiddle table and STRIDE = n / N picks the N-point
// twiddles from it; INV uses exp(+2 pi i j / n) (unnormalised, as cuFFT).
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <int STRIDE, bool INV>
__device__ __forceinline__ float2 twiddle(const float2 *w, int j) {
  float2 t = w[j * STRIDE];
  if (INV) t.y = -t.y;
  return t;
}

template <int N, int STRIDE, bool INV>
__device__ __forceinline__ void reg_dft(float2 *a, const float2 *w) {
  if constexpr (N == 2) {
    const float2 x = a[0], y = a[1];
    a[0] = make_float2(x.x + y.x, x.y + y.y);
    a[1] = make_float2(x.x - y.x, x.y - y.y);
  } else if constexpr (N >= 4) {
    constexpr int Q = N / 4;
    float2 s0[Q], s1[Q], s2[Q], s3[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      s0[i] = a[4 * i];
      s1[i] = a[4 * i + 1];
      s2[i] = a[4 * i + 2];
      s3[i] = a[4 * i + 3];
    }
    if constexpr (Q > 1) {
      reg_dft<Q, 4 * STRIDE, INV>(s0, w);
      reg_dft<Q, 4 * STRIDE, INV>(s1, w);
      reg_dft<Q, 4 * STRIDE, INV>(s2, w);
      reg_dft<Q, 4 * STRIDE, INV>(s3, w);
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      const float2 t0 = s0[k];
      const float2 t1 = k == 0 ? s1[k] : cmulf(s1[k], twiddle<STRIDE, INV>(w, k));
      const float2 t2 = k == 0 ? s2[k] : cmulf(s2[k], twiddle<STRIDE, INV>(w, 2 * k));
      const float2 t3 = k == 0 ? s3[k] : cmulf(s3[k], twiddle<STRIDE, INV>(w, 3 * k));
      const float2 a0 = make_float2(t0.x + t2.x, t0.y + t2.y), a1 = make_float2(t0.x - t2.x, t0.y - t2.y);
      const float2 b0 = make_float2(t1.x + t3.x, t1.y + t3.y), b1 = make_float2(t1.x - t3.x, t1.y - t3.y);
      // forward: X[k + Q] = a1 - i b1, X[k + 3Q] = a1 + i b1; the inverse swaps them
      const float2 mib = INV ? make_float2(-b1.y, b1.x) : make_float2(b1.y, -b1.x);
      a[k] = make_float2(a0.x + b0.x, a0.y + b0.y);
      a[k + Q] = make_float2(a1.x + mib.x, a1.y + mib.y);
      a[k + 2 * Q] = make_float2(a0.x - b0.x, a0.y - b0.y);
      a[k + 3 * Q] = make_float2(a1.x - mib.x, a1.y - mib.y);
    }
  }
}

// The axis-0 part of the CG operator, fused: for every line (s1, s2) of an n^3 FFT-native grid
// whose nonzero axis-0 entries are the support planes [0, L/2) and [n - L/2, n), the forward DFT
// along axis 0, the multiply by scale * diag (scale / diag with `divide`; diag centred like
// fine_diag_kernel's), the inverse DFT and the store of the support entries only, in place.
// L >= 2n makes every plane a support plane (a full transform, for the L^3 preconditioner).
// The twiddles are every tw_step-th entry of a larger table.
// It replaces a cuFFT axis-0 transform, fine_diag_kernel and the inverse transform (three
// passes over n^3 values) by one pass over the support half and the diagonal.
// n = N1 * N2 by the four-step decomposition: index i0 = n1 + N1 n2, frequency k = k2 + N2 k1;
// N2-point DFTs over n2 (thread n1), twiddle exp(-2 pi i n1 k2 / n), an exchange through shared
// memory, N1-point DFTs over n1 (thread k2); the inverse mirrors it.  A block takes 256 / TPL
// consecutive lines s2 of one s1, so every row of loads and stores is contiguous.
template <int N1, int N2>
__global__ void __launch_bounds__(256) axis0_diag_kernel(float2 *__restrict__ g, const float *__restrict__ diag,
                                                         const float2 *__restrict__ tw, int tw_step, int L,
                                                         int divide, float scale, const int *stop) {
  constexpr int n = N1 * N2;
  constexpr int TPL = N1 > N2 ? N1 : N2;  // threads per line
  constexpr int LPB = 256 / TPL;          // lines per block
  constexpr int RA = N1 + 1;              // exchange row of the forward transform (padded)
  constexpr int RB = N2 + 1;              // exchange row of the inverse transform (padded)
  // per-line exchange stride: a half warp (16 lanes of 8-byte accesses) spans H = min(LPB, 16)
  // lines and 16 / H roles, so lines must fall 16 / H banks-pairs apart: EX = 16 / H (mod 16)
  constexpr int EX0 = N2 * RA > N1 * RB ? N2 * RA : N1 * RB;
  constexpr int STEP = 16 / (LPB < 16 ? LPB : 16);
  constexpr int EX = EX0 + ((STEP - EX0 % 16) % 16 + 16) % 16;
  __shared__ float2 s_tw[n];
  __shared__ float2 s_ex[LPB * EX];
  if (stop && *stop) return;
  for (int j = threadIdx.x; j < n; j += blockDim.x) s_tw[j] = tw[j * tw_step];
  const int l = threadIdx.x % LPB, role = threadIdx.x / LPB;
  const int64_t line = (int64_t)blockIdx.x * LPB + l;  // s1 * n + s2
  const int s1 = (int)(line / n), s2 = (int)(line - (int64_t)s1 * n);
  const int64_t nn = (int64_t)n * n;
  float2 *col = g + line;  // entry i0 of the line at col[i0 * nn]
  const int h = L / 2;
  float2 *ex = s_ex + l * EX;
  __syncthreads();
  if (role < N1) {  // forward, thread n1: N2-point DFT over n2 of x[n1 + N1 n2], twiddle, exchange
    float2 v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) {
      const int i0 = role + N1 * n2;
      v[n2] = (i0 < h || i0 >= n - h) ? col[i0 * nn] : make_float2(0.f, 0.f);
    }
    reg_dft<N2, n / N2, false>(v, s_tw);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) ex[k2 * RA + role] = k2 == 0 ? v[0] : cmulf(v[k2], s_tw[role * k2]);
  }
  __syncthreads();
  float2 u[N1];
  if (role < N2) {
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) u[n1] = ex[role * RA + n1];
  }
  __syncthreads();
  if (role < N2) {  // thread k2: N1-point DFT over n1 gives X[k2 + N2 k1]; diagonal; inverse over k1
    const float *dcol = diag + (int64_t)native_to_centered(s1, n) * n + native_to_centered(s2, n);
    float d[N1];  // loaded before the transform, so their latency hides behind it
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) d[k1] = __ldg(dcol + (int64_t)native_to_centered(role + N2 * k1, n) * nn);
    reg_dft<N1, n / N1, false>(u, s_tw);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) {
      const float f = divide ? scale / d[k1] : scale * d[k1];
      u[k1] = make_float2(u[k1].x * f, u[k1].y * f);
    }
    reg_dft<N1, n / N1, true>(u, s_tw);  // u[m1] = sum_k1 X[k2 + N2 k1] exp(+2 pi i k1 m1 / N1)
#pragma unroll
    for (int m1 = 0; m1 < N1; ++m1) {
      float2 t = s_tw[role * m1];
      t.y = -t.y;
      ex[m1 * RB + role] = m1 == 0 ? u[0] : cmulf(u[m1], t);
    }
  }
  __syncthreads();
  if (role < N1) {  // thread m1: inverse N2-point DFT over k2 gives x[m1 + N1 m2]; support rows only
    float2 v[N2];
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) v[k2] = ex[role * RB + k2];
    reg_dft<N2, n / N2, true>(v, s_tw);
#pragma unroll
    for (int m2 = 0; m2 < N2; ++m2) {
      const int i0 = role + N1 * m2;
      if (i0 < h || i0 >= n - h) col[i0 * nn] = v[m2];
    }
  }
}

// One n-point DFT per line by the same four-step decomposition as axis0_diag_kernel: element
// i = n1 + N1 n2 comes from load(i) (thread n1), the result X[k], k = k2 + N2 k1, goes to
// store(k, X) (thread k2).  ex is the line's exchange area (N2 (N1 + 1) values); every thread
// of the block calls it (it synchronises the block).
template <int N1, int N2, bool INV, typename Load, typename Store>
__device__ __forceinline__ void line_dft(float2 *ex, const float2 *s_tw, int role, Load load, Store store) {
  constexpr int n = N1 * N2;
  constexpr int RA = N1 + 1;
  if (role < N1) {
    float2 v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = load(role + N1 * n2);
    reg_dft<N2, n / N2, INV>(v, s_tw);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) ex[k2 * RA + role] = k2 == 0 ? v[0] : cmulf(v[k2], twiddle<1, INV>(s_tw, role * k2));
  }
  __syncthreads();
  if (role < N2) {
    float2 u[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) u[n1] = ex[role * RA + n1];
    reg_dft<N1, n / N1, INV>(u, s_tw);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) store(role + N2 * k1, u[k1]);
  }
}

// support plane / row t in [0, L) of an axis of the fine grid (FFT-native storage)
__device__ __forceinline__ int support_index(int t, int L, int n) { return t < L / 2 ? t : n - L + t; }
__device__ __forceinline__ bool in_support(int s, int L, int n) { return s < L / 2 || s >= n - L / 2; }

// Block sums of two doubles added to a and b (either may be null); every thread calls it.
__device__ void block_add_pair(double x, double y, double *a, double *b) {
  __shared__ double sx[8], sy[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    x += __shfl_xor_sync(0xffffffffu, x, o);
    y += __shfl_xor_sync(0xffffffffu, y, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sx[w] = x;
    sy[w] = y;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tx = 0.0, ty = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      tx += sx[i];
      ty += sy[i];
    }
    if (a) atomicAdd(a, tx);
    if (b) atomicAdd(b, ty);
  }
}

// Line transforms of the fine grid (n = N1 N2, FFT-native storage, voxel j of an L^3 volume at
// storage index voxel_store(j)); channel blockIdx.y at g + c * cs.  Lines whose entries are
// adjacent (rows, axis 2) put a line's threads on adjacent lanes; lines of stride n (columns,
// axis 1) or n^2 (axis 0) put adjacent lines on adjacent lanes.  Pruning: only support planes
// and rows of the zero-padded volume are transformed, and each kernel writes exactly what the
// next one reads, so no grid is ever zeroed.
//   kRowFwd    CG: the volume row zero-padded (pad fused), forward along axis 2, whole row out
//   kPackRows  step: eigenvector row * exp(log_sqrt) / grid correction, zero-padded, forward
//   kColFwd    forward along axis 1 over the support entries of a support plane, whole column out
//   kColInv    inverse along axis 1, support entries out
//   kRowInv    CG: inverse along axis 2, the L support entries / n^3 to the volume (crop fused),
//              <p, out> accumulated
//   kUnpackRows step: inverse along axis 2, then d cost / d eigenvectors (2 Re(.) / grid
//              correction * exp(log_sqrt)) and the per-channel d cost / d log_sqrt sum
//   kAxisFwd   step: forward along axis 0 over the support rows; G written whole to gout, and the
//              gradient grid initialised in place: coef * fr * G (the Fourier regulariser's
//              derivative) with its value coef * sum fr |G|^2 accumulated, or zero without fr
//   kAxisInv   step: inverse along axis 0, support rows out
enum { kRowFwd, kPackRows, kColFwd, kColInv, kRowInv, kUnpackRows, kAxisFwd, kAxisInv };

struct LineArgs {
  int L;
  const float2 *tw;  // n twiddles
  const int *stop;   // the CG's done flag (every kernel returns once it is set) or null
  float2 *g;         // fine grid, channel stride cs
  int64_t cs;
  const float2 *vol;  // kRowFwd: L^3 input
  float2 *out;        // kRowInv: L^3 output
  const float2 *p;    // kRowInv: <p, out> operand or null
  double *dot;        // kRowInv: <p, out> (2 doubles)
  const float *vec;   // kPackRows, kUnpackRows: (r, L^3) eigenvectors
  const float *logs;  // (r) log sqrt eigenvalues or null
  const float *gc;    // (L) grid correction or null
  float *gvec;        // kUnpackRows: (r, L^3) gradient
  double *glog;       // kUnpackRows: (r) d cost / d log_sqrt accumulators
  float2 *gout;       // kAxisFwd: transformed grid (channel stride cs)
  const float *fr;    // kAxisFwd: regulariser weights (n^3, centred) or null
  int64_t frs;        // kAxisFwd: element stride between channels' weights (0: shared)
  double coef;        // kAxisFwd: regulariser coefficient
  double *cost;       // kAxisFwd: regulariser value accumulator
};

template <int N1, int N2, int KIND>
__global__ void __launch_bounds__(256) line_kernel(const LineArgs a) {
  constexpr int n = N1 * N2;
  constexpr int TPL = N1 > N2 ? N1 : N2;
  constexpr int LPB = 256 / TPL;
  constexpr bool ROWS = KIND == kRowFwd || KIND == kPackRows || KIND == kRowInv || KIND == kUnpackRows;
  constexpr int RA = N1 + 1;
  // exchange stride per line: with strided lines a half warp spans min(LPB, 16) lines (see
  // axis0_diag_kernel); with rows (TPL >= 16) it stays within one line
  constexpr int EX0 = N2 * RA;
  constexpr int STEP = 16 / (LPB < 16 ? LPB : 16);
  constexpr int EX = ROWS ? EX0 : EX0 + ((STEP - EX0 % 16) % 16 + 16) % 16;
  static_assert(!ROWS || TPL >= 16, "row lines need at least 16 threads per line");
  __shared__ float2 s_tw[n];
  __shared__ float2 s_ex[LPB * EX];
  if (a.stop && *a.stop) return;
  for (int j = threadIdx.x; j < n; j += blockDim.x) s_tw[j] = a.tw[j];
  const int l = ROWS ? threadIdx.x / TPL : threadIdx.x % LPB;
  const int role = ROWS ? threadIdx.x % TPL : threadIdx.x / LPB;
  const int64_t line = (int64_t)blockIdx.x * LPB + l;
  const int c = blockIdx.y;
  const int L = a.L;
  const int64_t L3 = (int64_t)L * L * L, nn = (int64_t)n * n;
  float2 *g = a.g + c * a.cs;
  float2 *ex = s_ex + l * EX;
  const float2 zero = make_float2(0.f, 0.f);
  __syncthreads();
  if (ROWS) {
    const int j0 = (int)(line / L), j1 = (int)(line - (int64_t)(line / L) * L);
    float2 *row = g + ((int64_t)voxel_store(j0, L, n) * n + voxel_store(j1, L, n)) * n;
    const int64_t vrow = ((int64_t)j0 * L + j1) * L;  // voxel row in the L^3 volume
    if (KIND == kRowFwd) {
      const float2 *src = a.vol + vrow;
      line_dft<N1, N2, false>(
          ex, s_tw, role, [&](int i) { const int j = pad_voxel(i, L, n); return j < 0 ? zero : src[j]; },
          [&](int k, float2 v) { row[k] = v; });
    } else if (KIND == kPackRows) {
      const float *src = a.vec + c * L3 + vrow;
      const float es = a.logs ? expf(__ldg(a.logs + c)) : 1.0f;
      const float g01 = a.gc ? __ldg(a.gc + j0) * __ldg(a.gc + j1) : 1.0f;
      line_dft<N1, N2, false>(
          ex, s_tw, role,
          [&](int i) {
            const int j = pad_voxel(i, L, n);
            if (j < 0) return zero;
            const float gi = a.gc ? 1.0f / (g01 * __ldg(a.gc + j)) : 1.0f;
            return make_float2(__ldg(src + j) * (gi * es), 0.f);
          },
          [&](int k, float2 v) { row[k] = v; });
    } else if (KIND == kRowInv) {
      float2 *dst = a.out + vrow;
      const float2 *pr = a.p ? a.p + vrow : nullptr;
      const float inv = 1.0f / ((float)n * (float)n * (float)n);
      double re = 0.0, im = 0.0;
      line_dft<N1, N2, true>(
          ex, s_tw, role, [&](int i) { return row[i]; },
          [&](int k, float2 v) {
            const int j = pad_voxel(k, L, n);
            if (j < 0) return;
            const float2 y = make_float2(v.x * inv, v.y * inv);
            dst[j] = y;
            if (pr) {  // conj(p) * y
              const float2 q = pr[j];
              re += (double)q.x * y.x + (double)q.y * y.y;
              im += (double)q.x * y.y - (double)q.y * y.x;
            }
          });
      if (a.p) block_add_pair(re, im, a.dot, a.dot + 1);
    } else {  // kUnpackRows
      const float es = a.logs ? expf(__ldg(a.logs + c)) : 1.0f;
      const float g01 = a.gc ? 1.0f / (__ldg(a.gc + j0) * __ldg(a.gc + j1)) : 1.0f;
      const float *vsrc = a.vec + c * L3 + vrow;
      float *gdst = a.gvec + c * L3 + vrow;
      float part = 0.0f;  // this thread's terms in FP32, then one FP64 block sum
      line_dft<N1, N2, true>(
          ex, s_tw, role, [&](int i) { return row[i]; },
          [&](int k, float2 v) {
            const int j = pad_voxel(k, L, n);
            if (j < 0) return;
            const float gj = a.gc ? g01 / __ldg(a.gc + j) : 1.0f;
            const float dV = 2.0f * v.x * gj;
            gdst[j] = dV * es;
            part = fmaf(dV, __ldg(vsrc + j) * es, part);
          });
      block_add_pair((double)part, 0.0, a.glog + c, nullptr);
    }
  } else if (KIND == kColFwd || KIND == kColInv) {
    const int t0 = (int)(line / n), s2 = (int)(line - (int64_t)(line / n) * n);
    float2 *col = g + (int64_t)support_index(t0, L, n) * nn + s2;  // entry s1 at col[s1 * n]
    if (KIND == kColFwd) {
      line_dft<N1, N2, false>(
          ex, s_tw, role, [&](int i) { return in_support(i, L, n) ? col[(int64_t)i * n] : zero; },
          [&](int k, float2 v) { col[(int64_t)k * n] = v; });
    } else {
      line_dft<N1, N2, true>(
          ex, s_tw, role, [&](int i) { return col[(int64_t)i * n]; },
          [&](int k, float2 v) { if (in_support(k, L, n)) col[(int64_t)k * n] = v; });
    }
  } else {  // axis 0: line (s1, s2), entry s0 at g[s0 * n^2 + line]
    float2 *ax = g + line;
    if (KIND == kAxisFwd) {
      const int s1 = (int)(line / n), s2 = (int)(line - (int64_t)(line / n) * n);
      float2 *gx = a.gout + c * a.cs + line;
      const float *frl =
          a.fr ? a.fr + c * a.frs + (int64_t)native_to_centered(s1, n) * n + native_to_centered(s2, n) : nullptr;
      float part = 0.0f;  // this thread's N1 terms in FP32, then one FP64 block sum (FP64 is slow)
      line_dft<N1, N2, false>(
          ex, s_tw, role, [&](int i) { return in_support(i, L, n) ? ax[(int64_t)i * nn] : zero; },
          [&](int k, float2 v) {
            gx[(int64_t)k * nn] = v;
            float2 y = zero;
            if (frl) {
              const float w = __ldg(frl + (int64_t)native_to_centered(k, n) * nn);
              const float cf = (float)a.coef * w;
              y = make_float2(cf * v.x, cf * v.y);
              part = fmaf(w, fmaf(v.x, v.x, v.y * v.y), part);
            }
            ax[(int64_t)k * nn] = y;
          });
      if (a.fr) block_add_pair((double)part * a.coef, 0.0, a.cost, nullptr);
    } else {  // kAxisInv
      line_dft<N1, N2, true>(
          ex, s_tw, role, [&](int i) { return ax[(int64_t)i * nn]; },
          [&](int k, float2 v) { if (in_support(k, L, n)) ax[(int64_t)k * nn] = v; });
    }
  }
}

}  // namespace

bool axis0_fused_size(int n) { return n == 64 || n == 128 || n == 256 || n == 512; }
bool line_transform_size(int n) { return n == 128 || n == 256 || n == 512; }

// One twiddle table exp(-2 pi i j / tn) of the plan's fine size tn serves every transform of
// the plan (size n reads every (tn / n)-th entry); built on the host in double precision.
int ensure_twiddles(cov3d_plan *p, int n) {
  const int tn = p->n % n == 0 ? p->n : n;
  if (p->fftw_n == tn) return COV3D_OK;
  std::vector<float2> h(tn);
  for (int j = 0; j < tn; ++j) {
    const double a = 2.0 * 3.14159265358979323846 * (double)j / (double)tn;
    h[j] = make_float2((float)std::cos(a), (float)-std::sin(a));
  }
  COV3D_TRY(grow(p->fftw, (int64_t)tn * sizeof(float2)));
  COV3D_CUDA(cudaMemcpyAsync(p->fftw.ptr, h.data(), tn * sizeof(float2), cudaMemcpyHostToDevice, p->stream));
  COV3D_CUDA(cudaStreamSynchronize(p->stream));  // h goes out of scope
  p->fftw_n = tn;
  return COV3D_OK;
}

int launch_axis0_diag(cov3d_plan *p, float2 *g, const float *diag, int L, int n, int divide, float scale,
                      const int *stop) {
  COV3D_TRY(ensure_twiddles(p, n));
  const float2 *tw = p->fftw.as<float2>();
  const int ts = p->fftw_n / n;
  const int64_t lines = (int64_t)n * n;
  cudaStream_t s = p->stream;
  switch (n) {
    case 64: axis0_diag_kernel<8, 8><<<(unsigned)(lines / 32), 256, 0, s>>>(g, diag, tw, ts, L, divide, scale, stop); break;
    case 128: axis0_diag_kernel<16, 8><<<(unsigned)(lines / 16), 256, 0, s>>>(g, diag, tw, ts, L, divide, scale, stop); break;
    case 256: axis0_diag_kernel<16, 16><<<(unsigned)(lines / 16), 256, 0, s>>>(g, diag, tw, ts, L, divide, scale, stop); break;
    case 512: axis0_diag_kernel<32, 16><<<(unsigned)(lines / 8), 256, 0, s>>>(g, diag, tw, ts, L, divide, scale, stop); break;
    default: set_error("no fused axis-0 transform for n = %d", n); return COV3D_EINVAL;
  }
  return launched("axis0_diag_kernel");
}

namespace {

template <int N1, int N2, int KIND>
int launch_lines(cov3d_plan *p, const LineArgs &a, int64_t lines, int nchan) {
  constexpr int TPL = N1 > N2 ? N1 : N2, LPB = 256 / TPL;
  line_kernel<N1, N2, KIND><<<dim3((unsigned)(lines / LPB), (unsigned)nchan), 256, 0, p->stream>>>(a);
  return launched("line_kernel");
}

template <int N1, int N2>
int cg_operator_n(cov3d_plan *p, LineArgs a, const float *diag, int divide, const int *stop_last) {
  constexpr int n = N1 * N2;
  const int L = a.L;
  COV3D_TRY((launch_lines<N1, N2, kRowFwd>(p, a, (int64_t)L * L, 1)));
  COV3D_TRY((launch_lines<N1, N2, kColFwd>(p, a, (int64_t)L * n, 1)));
  COV3D_TRY(launch_axis0_diag(p, a.g, diag, L, n, divide, 1.0f, a.stop));
  COV3D_TRY((launch_lines<N1, N2, kColInv>(p, a, (int64_t)L * n, 1)));
  a.stop = stop_last;
  return launch_lines<N1, N2, kRowInv>(p, a, (int64_t)L * L, 1);
}

template <int N1, int N2>
int step_forward_n(cov3d_plan *p, const LineArgs &a, int r) {
  constexpr int n = N1 * N2;
  COV3D_TRY((launch_lines<N1, N2, kPackRows>(p, a, (int64_t)a.L * a.L, r)));
  COV3D_TRY((launch_lines<N1, N2, kColFwd>(p, a, (int64_t)a.L * n, r)));
  return launch_lines<N1, N2, kAxisFwd>(p, a, (int64_t)n * n, r);
}

template <int N1, int N2>
int step_inverse_n(cov3d_plan *p, const LineArgs &a, int r) {
  constexpr int n = N1 * N2;
  COV3D_TRY((launch_lines<N1, N2, kAxisInv>(p, a, (int64_t)n * n, r)));
  COV3D_TRY((launch_lines<N1, N2, kColInv>(p, a, (int64_t)a.L * n, r)));
  return launch_lines<N1, N2, kUnpackRows>(p, a, (int64_t)a.L * a.L, r);
}

// The plan's twiddles for its fine size n; line transforms need the table of exactly n.
int line_args(cov3d_plan *p, LineArgs &a) {
  COV3D_TRY(ensure_twiddles(p, p->n));
  if (!line_transform_size(p->n) || p->fftw_n != p->n || p->L % 2 != 0 || p->n < p->L + 2) {
    set_error("no line transform for L = %d, n = %d", p->L, p->n);
    return COV3D_EINVAL;
  }
  a = LineArgs{};
  a.L = p->L;
  a.tw = p->fftw.as<float2>();
  return COV3D_OK;
}

}  // namespace

bool line_transforms_apply(const cov3d_plan *p) {
  return line_transform_size(p->n) && p->L % 2 == 0 && p->n >= p->L + 2;
}

int cg_operator_lines(cov3d_plan *p, const float2 *in, float2 *fine, float2 *out, const float2 *dotp,
                      const float *diag, int divide, const int *stop, const int *stop_last, double *dot) {
  LineArgs a;
  COV3D_TRY(line_args(p, a));
  a.stop = stop;
  a.g = fine;
  a.cs = 0;
  a.vol = in;
  a.out = out;
  a.p = dotp;
  a.dot = dot;
  switch (p->n) {
    case 128: return cg_operator_n<16, 8>(p, a, diag, divide, stop_last);
    case 256: return cg_operator_n<16, 16>(p, a, diag, divide, stop_last);
    default: return cg_operator_n<32, 16>(p, a, diag, divide, stop_last);
  }
}

int step_forward_lines(cov3d_plan *p, const float *vec, const float *logs, const float *gc, int r, float2 *stage,
                       float2 *grid, const float *fr, int64_t fr_stride, double coef, double *cost) {
  LineArgs a;
  COV3D_TRY(line_args(p, a));
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  a.g = stage;
  a.cs = n3;
  a.vec = vec;
  a.logs = logs;
  a.gc = gc;
  a.gout = grid;
  a.fr = fr;
  a.frs = fr_stride;
  a.coef = coef;
  a.cost = cost;
  switch (p->n) {
    case 128: return step_forward_n<16, 8>(p, a, r);
    case 256: return step_forward_n<16, 16>(p, a, r);
    default: return step_forward_n<32, 16>(p, a, r);
  }
}

int step_inverse_lines(cov3d_plan *p, float2 *grad_grid, const float *vec, const float *logs, const float *gc, int r,
                       float *gvec, double *glog) {
  LineArgs a;
  COV3D_TRY(line_args(p, a));
  a.g = grad_grid;
  a.cs = (int64_t)p->n * p->n * p->n;
  a.vec = vec;
  a.logs = logs;
  a.gc = gc;
  a.gvec = gvec;
  a.glog = glog;
  switch (p->n) {
    case 128: return step_inverse_n<16, 8>(p, a, r);
    case 256: return step_inverse_n<16, 16>(p, a, r);
    default: return step_inverse_n<32, 16>(p, a, r);
  }
}

}  // namespace cov3d
