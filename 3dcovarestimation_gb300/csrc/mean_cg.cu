// Mean-volume reconstruction on the device: backprojection of the images and of the squared
// CTFs into the centered fine grid (reference reconstruct_mean, mean.py:145-259), the
// shell-floor regularisation of the kernel (regularize_lhs, mean.py:135-142), the
// Fourier-diagonal first solve, and the conjugate-gradient correction for the zero padding
// (complex_conjugate_gradient + correct_upsampling_padding, mean.py:43-132):
//
//   A(x) = crop_L( ifft3( lhs * fft3( pad_n(x) ) ) )      (centered transforms, ifft / n^3)
//
// The operator is pad + cuFFT + diagonal multiply + inverse cuFFT + crop.  The vector updates
// are fused with their inner products, which accumulate in FP64.  The iteration scalars stay
// in device memory and a convergence flag turns every kernel of later iterations into a
// no-op, so the host polls the flag only every few iterations.  Preconditioners:
//   1: M r = crop(ifft3(fft3(pad r) / lhs))              (the Fourier-diagonal solve on the
//      fine grid, the operator the reference uses for its starting point, mean.py:238-239)
//   2: M r = ifft3_L(fft3_L(r) / s)                      (a Fourier diagonal on the L^3 grid:
//      the optimal circulant approximation of A from cov3d_circulant_symbol, or a learned s)
#include <cmath>
#include <vector>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

struct CgState {
  double rz;      // <r, z>  (z = r without a preconditioner)
  double rr;      // <r, r>
  double b2;      // <b, b>
  double pap[2];  // <p, A p>, complex
  double rz_new;
  double rr_new;
  int done;       // 1 converged, 2 reached maxiter
  int iters;      // loop index at which the loop stopped (the reference's num_iter)
  int running;    // current loop index
  int pad;
};

inline unsigned nb(int64_t n) { return (unsigned)((n + 255) / 256); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block reduction of two partial sums, added to global accumulators (either may be null).
__device__ void block_add2(double a, double b, double *ga, double *gb) {
  __shared__ double sa[32], sb[32];
  a = warp_sum(a);
  b = warp_sum(b);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sa[w] = a;
    sb[w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      ta += sa[i];
      tb += sb[i];
    }
    if (ga) atomicAdd(ga, ta);
    if (gb) atomicAdd(gb, tb);
  }
}

__device__ __forceinline__ bool stopped(const CgState *st) { return st != nullptr && st->done != 0; }

// centered index of FFT-native storage index s on a grid of size m (fftshift)
__device__ __forceinline__ int native_to_centered(int s, int m) {
  const int c = s + m / 2;
  return c >= m ? c - m : c;
}

// fine[s] = src[centered(s)] (/ div[centered(s)]); src complex or real
__global__ void load_centered_kernel(const float2 *__restrict__ src, const float *__restrict__ src_real,
                                     const float *__restrict__ div, int n, float2 *__restrict__ fine) {
  const int64_t n3 = (int64_t)n * n * n;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= n3) return;
  const int s2 = (int)(cell % n), s1 = (int)((cell / n) % n), s0 = (int)(cell / ((int64_t)n * n));
  const int64_t c = ((int64_t)native_to_centered(s0, n) * n + native_to_centered(s1, n)) * n + native_to_centered(s2, n);
  float2 v = src ? src[c] : make_float2(src_real[c], 0.0f);
  if (div) {
    const float d = div[c];
    v = make_float2(v.x / d, v.y / d);
  }
  fine[cell] = v;
}

// The grid kernels walk whole rows (one division per row, none per element) and the reductions
// run a capped grid of blocks in grid-stride loops, so each reduction costs one FP64 atomic per
// block rather than one per 256 elements.
constexpr int kRowBlocks = 1216;  // 8 blocks of 256 threads per SM

inline unsigned capped(int64_t n_items_per_block_unit) {
  return (unsigned)(n_items_per_block_unit < kRowBlocks ? (n_items_per_block_unit > 0 ? n_items_per_block_unit : 1)
                                                        : kRowBlocks);
}

// voxel index of FFT-native storage index s on the padded axis, or -1 for padding
__device__ __forceinline__ int pad_voxel(int s, int L, int n) {
  const int h = L / 2;
  return s < L - h ? s + h : (s >= n - h ? s - n + h : -1);
}
// FFT-native storage index of voxel j
__device__ __forceinline__ int voxel_store(int j, int L, int n) {
  const int k = j - L / 2;
  return k < 0 ? k + n : k;
}

// zero-pad x (L^3, voxel offset k = j - L/2) into FFT-native storage k mod n
__global__ void pad_kernel(const float2 *__restrict__ x, int L, int n, float2 *__restrict__ fine, const CgState *st) {
  if (stopped(st)) return;
  for (int64_t row = blockIdx.x; row < (int64_t)n * n; row += gridDim.x) {
    const int s0 = (int)(row / n), s1 = (int)(row - (int64_t)s0 * n);
    const int j0 = pad_voxel(s0, L, n), j1 = pad_voxel(s1, L, n);
    float2 *dst = fine + row * n;
    if (j0 < 0 || j1 < 0) {
      for (int s2 = threadIdx.x; s2 < n; s2 += blockDim.x) dst[s2] = make_float2(0.f, 0.f);
      continue;
    }
    const float2 *src = x + ((int64_t)j0 * L + j1) * L;
    for (int s2 = threadIdx.x; s2 < n; s2 += blockDim.x) {
      const int j2 = pad_voxel(s2, L, n);
      dst[s2] = j2 < 0 ? make_float2(0.f, 0.f) : src[j2];
    }
  }
}

// pad_kernel restricted to the L support planes (the other planes of `fine` stay zero)
__global__ void pad_support_kernel(const float2 *__restrict__ x, int L, int n, float2 *__restrict__ fine,
                                   const CgState *st) {
  if (stopped(st)) return;
  const int h = L / 2;
  for (int64_t row = blockIdx.x; row < (int64_t)L * n; row += gridDim.x) {
    const int sp = (int)(row / n), s1 = (int)(row - (int64_t)sp * n);
    const int s0 = sp < L - h ? sp : n - L + sp;
    const int j0 = pad_voxel(s0, L, n), j1 = pad_voxel(s1, L, n);
    float2 *dst = fine + ((int64_t)s0 * n + s1) * n;
    if (j1 < 0) {
      for (int s2 = threadIdx.x; s2 < n; s2 += blockDim.x) dst[s2] = make_float2(0.f, 0.f);
      continue;
    }
    const float2 *src = x + ((int64_t)j0 * L + j1) * L;
    for (int s2 = threadIdx.x; s2 < n; s2 += blockDim.x) {
      const int j2 = pad_voxel(s2, L, n);
      dst[s2] = j2 < 0 ? make_float2(0.f, 0.f) : src[j2];
    }
  }
}

// g[s] *= diag[centered(s)] * scale (divide instead when `divide`), g an m^3 FFT-native grid
__global__ void fine_diag_kernel(float2 *__restrict__ g, const float *__restrict__ diag, int m, int divide, float scale,
                                 const CgState *st) {
  if (stopped(st)) return;
  for (int64_t row = blockIdx.x; row < (int64_t)m * m; row += gridDim.x) {
    const int s0 = (int)(row / m), s1 = (int)(row - (int64_t)s0 * m);
    const float *drow = diag + ((int64_t)native_to_centered(s0, m) * m + native_to_centered(s1, m)) * m;
    float2 *grow = g + row * m;
    for (int s2 = threadIdx.x; s2 < m; s2 += blockDim.x) {
      const float d = __ldg(drow + native_to_centered(s2, m));
      const float f = divide ? scale / d : scale * d;
      const float2 v = grow[s2];
      grow[s2] = make_float2(v.x * f, v.y * f);
    }
  }
}

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
                                                         int divide, float scale, const CgState *st) {
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
  if (stopped(st)) return;
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

// The pruned transforms of the CG operator around axis0_diag_kernel, as line DFTs of the fine
// grid (n = N1 N2, FFT-native storage, a voxel j of the L^3 volume at index voxel_store(j)):
//   kRowFwd: rows (s0, s1) of support planes and rows: the volume row zero-padded, DFT along
//            axis 2, the whole row written (pad fused);
//   kColFwd: columns (s0, s2) of support planes: the support entries, DFT along axis 1, the whole
//            column written;
//   kColInv: the inverse along axis 1, support entries written;
//   kRowInv: the inverse along axis 2, the L support entries / n^3 written to the volume (crop
//            fused), with <p, out> into st->pap when p is given.
// Every kernel writes exactly what the next reads, so the grid needs no zeroing.  Rows are
// contiguous (a line's threads are adjacent lanes); columns are n apart (a block takes
// consecutive columns, adjacent lanes on adjacent columns).
enum { kRowFwd = 0, kColFwd = 1, kColInv = 2, kRowInv = 3 };

template <int N1, int N2, int KIND>
__global__ void __launch_bounds__(256) cg_line_kernel(const float2 *__restrict__ vol, float2 *__restrict__ g,
                                                      float2 *__restrict__ out, const float2 *__restrict__ p,
                                                      const float2 *__restrict__ tw, int L, CgState *st) {
  constexpr int n = N1 * N2;
  constexpr int TPL = N1 > N2 ? N1 : N2;
  constexpr int LPB = 256 / TPL;
  constexpr bool ROWS = KIND == kRowFwd || KIND == kRowInv;
  constexpr int RA = N1 + 1;
  // exchange stride per line: with columns a half warp spans min(LPB, 16) lines (see
  // axis0_diag_kernel); with rows (TPL >= 16) it stays within one line
  constexpr int EX0 = N2 * RA;
  constexpr int STEP = 16 / (LPB < 16 ? LPB : 16);
  constexpr int EX = ROWS ? EX0 : EX0 + ((STEP - EX0 % 16) % 16 + 16) % 16;
  static_assert(!ROWS || TPL >= 16, "row lines need at least 16 threads per line");
  __shared__ float2 s_tw[n];
  __shared__ float2 s_ex[LPB * EX];
  if (stopped(st)) return;
  for (int j = threadIdx.x; j < n; j += blockDim.x) s_tw[j] = tw[j];
  const int l = ROWS ? threadIdx.x / TPL : threadIdx.x % LPB;
  const int role = ROWS ? threadIdx.x % TPL : threadIdx.x / LPB;
  const int64_t line = (int64_t)blockIdx.x * LPB + l;
  float2 *ex = s_ex + l * EX;
  const float2 zero = make_float2(0.f, 0.f);
  __syncthreads();
  if (KIND == kRowFwd) {
    const int j0 = (int)(line / L), j1 = (int)(line - (int64_t)(line / L) * L);
    const float2 *src = vol + ((int64_t)j0 * L + j1) * L;
    float2 *dst = g + ((int64_t)voxel_store(j0, L, n) * n + voxel_store(j1, L, n)) * n;
    line_dft<N1, N2, false>(
        ex, s_tw, role, [&](int i) { const int j = pad_voxel(i, L, n); return j < 0 ? zero : src[j]; },
        [&](int k, float2 v) { dst[k] = v; });
  } else if (KIND == kColFwd || KIND == kColInv) {
    const int t0 = (int)(line / n), s2 = (int)(line - (int64_t)(line / n) * n);
    float2 *c = g + (int64_t)support_index(t0, L, n) * n * n + s2;  // entry s1 at c[s1 * n]
    if (KIND == kColFwd) {
      line_dft<N1, N2, false>(
          ex, s_tw, role, [&](int i) { return in_support(i, L, n) ? c[(int64_t)i * n] : zero; },
          [&](int k, float2 v) { c[(int64_t)k * n] = v; });
    } else {
      line_dft<N1, N2, true>(
          ex, s_tw, role, [&](int i) { return c[(int64_t)i * n]; },
          [&](int k, float2 v) { if (in_support(k, L, n)) c[(int64_t)k * n] = v; });
    }
  } else {  // kRowInv
    const int j0 = (int)(line / L), j1 = (int)(line - (int64_t)(line / L) * L);
    const float2 *src = g + ((int64_t)voxel_store(j0, L, n) * n + voxel_store(j1, L, n)) * n;
    float2 *dst = out + ((int64_t)j0 * L + j1) * L;
    const float2 *pr = p ? p + ((int64_t)j0 * L + j1) * L : nullptr;
    const float inv = 1.0f / ((float)n * (float)n * (float)n);
    double re = 0.0, im = 0.0;
    line_dft<N1, N2, true>(
        ex, s_tw, role, [&](int i) { return src[i]; },
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
    if (p) block_add2(re, im, &st->pap[0], &st->pap[1]);
  }
}

// The fused axis-0 transform for the grid sizes it is built for (n = 64 .. 512); returns false
// (nothing launched) for others, which take cuFFT and fine_diag_kernel.
bool axis0_fused_size(int n) { return n == 64 || n == 128 || n == 256 || n == 512; }

// One twiddle table exp(-2 pi i j / tn) of the plan's fine size tn serves the fine operator and
// the L^3 preconditioner (every (tn / n)-th entry); built on the host in double precision.
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
                      const CgState *gate) {
  COV3D_TRY(ensure_twiddles(p, n));
  const float2 *tw = p->fftw.as<float2>();
  const int ts = p->fftw_n / n;
  const int64_t lines = (int64_t)n * n;
  switch (n) {
    case 64: axis0_diag_kernel<8, 8><<<(unsigned)(lines / 32), 256, 0, p->stream>>>(g, diag, tw, ts, L, divide, scale, gate); break;
    case 128: axis0_diag_kernel<16, 8><<<(unsigned)(lines / 16), 256, 0, p->stream>>>(g, diag, tw, ts, L, divide, scale, gate); break;
    case 256: axis0_diag_kernel<16, 16><<<(unsigned)(lines / 16), 256, 0, p->stream>>>(g, diag, tw, ts, L, divide, scale, gate); break;
    case 512: axis0_diag_kernel<32, 16><<<(unsigned)(lines / 8), 256, 0, p->stream>>>(g, diag, tw, ts, L, divide, scale, gate); break;
    default: set_error("no fused axis-0 transform for n = %d", n); return COV3D_EINVAL;
  }
  return launched("axis0_diag_kernel");
}

// The whole CG operator on hand-written line DFTs (n = 128, 256, 512): pad + rows, columns,
// axis 0 with the diagonal, inverse columns, inverse rows + crop (+ <p, out> into acc).
bool pruned3_size(int n) { return n == 128 || n == 256 || n == 512; }

template <int N1, int N2>
int pruned3_launch(cov3d_plan *p, const float2 *in, float2 *fine, float2 *out, const float2 *dotp, const float *diag,
                   int divide, int L, const CgState *gate, CgState *acc) {
  constexpr int TPL = N1 > N2 ? N1 : N2, LPB = 256 / TPL;
  constexpr int n = N1 * N2;
  cudaStream_t s = p->stream;
  const float2 *tw = p->fftw.as<float2>();
  CgState *g = const_cast<CgState *>(gate);
  const unsigned rows = (unsigned)((int64_t)L * L / LPB), cols = (unsigned)((int64_t)L * n / LPB);
  cg_line_kernel<N1, N2, kRowFwd><<<rows, 256, 0, s>>>(in, fine, nullptr, nullptr, tw, L, g);
  COV3D_LAUNCHED("cg_line_kernel");
  cg_line_kernel<N1, N2, kColFwd><<<cols, 256, 0, s>>>(nullptr, fine, nullptr, nullptr, tw, L, g);
  COV3D_LAUNCHED("cg_line_kernel");
  COV3D_TRY(launch_axis0_diag(p, fine, diag, L, n, divide, 1.0f, gate));
  cg_line_kernel<N1, N2, kColInv><<<cols, 256, 0, s>>>(nullptr, fine, nullptr, nullptr, tw, L, g);
  COV3D_LAUNCHED("cg_line_kernel");
  cg_line_kernel<N1, N2, kRowInv><<<rows, 256, 0, s>>>(nullptr, fine, out, dotp, tw, L, dotp ? acc : g);
  return launched("cg_line_kernel");
}

int pruned3(cov3d_plan *p, const float2 *in, float2 *fine, float2 *out, const float2 *dotp, const float *diag,
            int divide, int L, int n, const CgState *gate, CgState *acc) {
  COV3D_TRY(ensure_twiddles(p, n));
  if (p->fftw_n != n) {
    set_error("pruned line transform: twiddle table of %d for n = %d", p->fftw_n, n);
    return COV3D_EINVAL;
  }
  switch (n) {
    case 128: return pruned3_launch<16, 8>(p, in, fine, out, dotp, diag, divide, L, gate, acc);
    case 256: return pruned3_launch<16, 16>(p, in, fine, out, dotp, diag, divide, L, gate, acc);
    case 512: return pruned3_launch<32, 16>(p, in, fine, out, dotp, diag, divide, L, gate, acc);
    default: set_error("no pruned line transform for n = %d", n); return COV3D_EINVAL;
  }
}

// out = crop(fine) / n^3; optionally keep only the real part; optionally accumulate <p, out>
__global__ void crop_kernel(const float2 *__restrict__ fine, int L, int n, float2 *__restrict__ out, int real_only,
                            const float2 *__restrict__ p, CgState *st) {
  if (stopped(st)) return;
  const float inv = 1.0f / ((float)n * (float)n * (float)n);
  double re = 0.0, im = 0.0;
  for (int64_t row = blockIdx.x; row < (int64_t)L * L; row += gridDim.x) {
    const int j0 = (int)(row / L), j1 = (int)(row - (int64_t)j0 * L);
    const float2 *src = fine + ((int64_t)voxel_store(j0, L, n) * n + voxel_store(j1, L, n)) * n;
    for (int j2 = threadIdx.x; j2 < L; j2 += blockDim.x) {
      const float2 a = src[voxel_store(j2, L, n)];
      const float2 y = make_float2(a.x * inv, real_only ? 0.0f : a.y * inv);
      out[row * L + j2] = y;
      if (p) {  // conj(p) * y
        const float2 q = p[row * L + j2];
        re += (double)q.x * y.x + (double)q.y * y.y;
        im += (double)q.x * y.y - (double)q.y * y.x;
      }
    }
  }
  if (p) block_add2(re, im, &st->pap[0], &st->pap[1]);
}

// r = b - r (r holds A x on entry); accumulate <r, r> and <b, b>
__global__ void residual_kernel(const float2 *__restrict__ b, float2 *__restrict__ r, int64_t N, CgState *st) {
  double rr = 0.0, bb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 bv = b[i], ax = r[i];
    const float2 rv = make_float2(bv.x - ax.x, bv.y - ax.y);
    r[i] = rv;
    rr += (double)rv.x * rv.x + (double)rv.y * rv.y;
    bb += (double)bv.x * bv.x + (double)bv.y * bv.y;
  }
  block_add2(rr, bb, &st->rr, &st->b2);
}

// Re <r, z> into st->rz_new
__global__ void dot_rz_kernel(const float2 *__restrict__ r, const float2 *__restrict__ z, int64_t N, CgState *st) {
  if (stopped(st)) return;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = r[i], c = z[i];
    acc += (double)a.x * c.x + (double)a.y * c.y;
  }
  block_add2(acc, 0.0, &st->rz_new, nullptr);
}

// alpha = rz / <p, Ap>;  x += alpha p;  r -= alpha Ap;  accumulate <r, r>
__global__ void update_kernel(float2 *__restrict__ x, float2 *__restrict__ r, const float2 *__restrict__ p,
                              const float2 *__restrict__ ap, int64_t N, CgState *st) {
  if (stopped(st)) return;
  const double pr = st->pap[0], pi = st->pap[1];
  const double den = pr * pr + pi * pi;
  const float ar = (float)(st->rz * pr / den), ai = (float)(-st->rz * pi / den);
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 pv = p[i], av = ap[i];
    float2 xv = x[i], rv = r[i];
    xv.x += ar * pv.x - ai * pv.y;
    xv.y += ar * pv.y + ai * pv.x;
    rv.x -= ar * av.x - ai * av.y;
    rv.y -= ar * av.y + ai * av.x;
    x[i] = xv;
    r[i] = rv;
    rr += (double)rv.x * rv.x + (double)rv.y * rv.y;
  }
  block_add2(rr, 0.0, &st->rr_new, nullptr);
}

// convergence test of loop index `running` (||r|| < rtol ||b||, mean.py:80-81)
__global__ void check_kernel(CgState *st, double rtol, int preconditioned, double *hist, int maxiter) {
  if (st->done) return;
  const int it = st->running;
  if (hist) hist[it + 1] = sqrt(st->rr_new / st->b2);
  if (!(st->rr_new == st->rr_new)) {  // NaN: stop, reported by the host
    st->done = 3;
    st->iters = it;
  } else if (sqrt(st->rr_new) < rtol * sqrt(st->b2)) {
    st->done = 1;
    st->iters = it;
  } else if (it + 1 >= maxiter) {
    st->done = 2;
    st->iters = it;
  } else if (!preconditioned) {
    st->rz_new = st->rr_new;
  }
}

// p = z + (rz_new / rz) p
__global__ void direction_kernel(float2 *__restrict__ p, const float2 *__restrict__ z, int64_t N, const CgState *st) {
  if (stopped(st)) return;
  const float beta = (float)(st->rz_new / st->rz);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 zv = z[i], pv = p[i];
    p[i] = make_float2(zv.x + beta * pv.x, zv.y + beta * pv.y);
  }
}

__global__ void roll_kernel(CgState *st) {
  if (st->done) return;
  st->rz = st->rz_new;
  st->rr = st->rr_new;
  st->rz_new = 0.0;
  st->rr_new = 0.0;
  st->pap[0] = 0.0;
  st->pap[1] = 0.0;
  st->running += 1;
}

__global__ void copy_kernel(const float2 *__restrict__ a, float2 *__restrict__ b, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) b[i] = a[i];
}

__global__ void init_kernel(CgState *st, int preconditioned, double *hist) {
  st->rz = preconditioned ? st->rz_new : st->rr;
  st->rz_new = 0.0;
  st->rr_new = 0.0;
  st->pap[0] = 0.0;
  st->pap[1] = 0.0;
  st->done = 0;
  st->iters = -1;
  st->running = 0;
  if (hist) hist[0] = sqrt(st->rr / st->b2);
}

// Optimal circulant (T. Chan 1988) of the L^3 block-Toeplitz operator A, whose convolution
// kernel is t = ifft_n(lhs): per axis c[tau] = ((L - tau) t[tau] + tau t[tau - L]) / L.  `t` is
// the unnormalised inverse FFT (FFT-native order); the 1/n^3 is applied here.
__global__ void circulant_gather_kernel(const float2 *__restrict__ t, int L, int n, float2 *__restrict__ c) {
  const int64_t L3 = (int64_t)L * L * L;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= L3) return;
  const int tau[3] = {(int)(v / ((int64_t)L * L)), (int)((v / L) % L), (int)(v % L)};
  int idx[3][2];
  float w[3][2];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    idx[a][0] = tau[a];
    w[a][0] = (float)(L - tau[a]) / (float)L;
    idx[a][1] = tau[a] - L < 0 ? tau[a] - L + n : tau[a] - L;
    w[a][1] = (float)tau[a] / (float)L;
  }
  double re = 0.0, im = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int a0 = q >> 2, a1 = (q >> 1) & 1, a2 = q & 1;
    const double wt = (double)w[0][a0] * w[1][a1] * w[2][a2];
    if (wt == 0.0) continue;
    const float2 tv = t[((int64_t)idx[0][a0] * n + idx[1][a1]) * n + idx[2][a2]];
    re += wt * tv.x;
    im += wt * tv.y;
  }
  const double inv = 1.0 / ((double)n * n * n);
  c[v] = make_float2((float)(re * inv), (float)(im * inv));
}

// symbol[centered] = Re(lambda[native]), floored at `floor_value`
__global__ void symbol_store_kernel(const float2 *__restrict__ lam, int L, float floor_value, float *__restrict__ sym) {
  const int64_t L3 = (int64_t)L * L * L;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= L3) return;
  const int s2 = (int)(v % L), s1 = (int)((v / L) % L), s0 = (int)(v / ((int64_t)L * L));
  const int64_t c = ((int64_t)native_to_centered(s0, L) * L + native_to_centered(s1, L)) * L + native_to_centered(s2, L);
  sym[c] = fmaxf(lam[v].x, floor_value);
}

// ---------------------------------------------------------------------------- regularize_lhs

// Shell of centered coordinates (k0, k1, k2): shell i holds radii in (i - 1/2, i + 1/2), the
// last shell (i - 1/2, i + 1) (fsc_utils.py FourierShell.radial_avg_interval); the radius is
// never a half integer, so the shell is round(radius) capped at nshell - 1.
__device__ __forceinline__ int shell_of(int k0, int k1, int k2, int nshell) {
  const double rad = sqrt((double)(k0 * k0 + k1 * k1 + k2 * k2));
  const int i = (int)floor(rad + 0.5);
  return i < nshell ? i : nshell - 1;
}

// one block per plane i0; each thread walks whole rows and flushes runs of equal shell
__global__ void shell_sum_kernel(const float2 *__restrict__ lhs, int n, int nshell, double *__restrict__ sums,
                                 double *__restrict__ counts) {
  extern __shared__ double sh[];  // sums[nshell], counts[nshell]
  for (int i = threadIdx.x; i < 2 * nshell; i += blockDim.x) sh[i] = 0.0;
  __syncthreads();
  const int h = n / 2;
  const int i0 = blockIdx.x;
  for (int i1 = threadIdx.x; i1 < n; i1 += blockDim.x) {
    const float2 *row = lhs + ((int64_t)i0 * n + i1) * n;
    int cur = -1;
    double acc = 0.0, cnt = 0.0;
    for (int i2 = 0; i2 < n; ++i2) {
      const int s = shell_of(i0 - h, i1 - h, i2 - h, nshell);
      if (s != cur) {
        if (cur >= 0) {
          atomicAdd(&sh[cur], acc);
          atomicAdd(&sh[nshell + cur], cnt);
        }
        cur = s;
        acc = 0.0;
        cnt = 0.0;
      }
      acc += (double)row[i2].x;
      cnt += 1.0;
    }
    if (cur >= 0) {
      atomicAdd(&sh[cur], acc);
      atomicAdd(&sh[nshell + cur], cnt);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nshell; i += blockDim.x) {
    if (sh[nshell + i] != 0.0) {
      atomicAdd(&sums[i], sh[i]);
      atomicAdd(&counts[i], sh[nshell + i]);
    }
  }
}

// reg = max(|lhs|, 1e-3 * shell mean of Re lhs), clamped at 1e-8 (mean.py:135-142)
__global__ void regularize_kernel(const float2 *__restrict__ lhs, int n, int nshell, const double *__restrict__ sums,
                                  const double *__restrict__ counts, float *__restrict__ out) {
  const int64_t n3 = (int64_t)n * n * n;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= n3) return;
  const int h = n / 2;
  const int i2 = (int)(cell % n), i1 = (int)((cell / n) % n), i0 = (int)(cell / ((int64_t)n * n));
  const int s = shell_of(i0 - h, i1 - h, i2 - h, nshell);
  const float floor_shell = (float)(sums[s] / counts[s]) * 1e-3f;
  const float2 v = lhs[cell];
  out[cell] = fmaxf(fmaxf(hypotf(v.x, v.y), floor_shell), 1e-8f);
}

// ---------------------------------------------------------------------------- backprojection

// Values spread for the mean: channel 0 = y * exp(-i (gx sx + gy sy)) * c * ctf (the image
// phase-shifted by -offset, mean.py:201-204), channel 1 = (c * ctf)^2 / L (the kernel, whose
// extra 1/L is mean.py:215); gx, gy = ceil(k - L/2) 2 pi / L (poses.py:70-89).
__global__ void mean_values_kernel(const float2 *__restrict__ images, const float *__restrict__ ctf,
                                   const float *__restrict__ offsets, const float *__restrict__ contrasts,
                                   int64_t n_images, int L, float2 *__restrict__ vals) {
  const int P = L * L;
  const int64_t M = n_images * P;
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= M) return;
  const int64_t b = id / P;
  const int p = (int)(id - b * P);
  float f = ctf ? __ldg(ctf + id) : 1.0f;
  if (contrasts) f *= __ldg(contrasts + b);
  float2 y = images[id];
  if (offsets) {
    const int row = p / L, col = p - row * L;
    const float half = 0.5f * (float)L;
    const float gx = __fdiv_rn(__fmul_rn(__fmul_rn(ceilf((float)col - half), 2.0f), kPiF), (float)L);
    const float gy = __fdiv_rn(__fmul_rn(__fmul_rn(ceilf((float)row - half), 2.0f), kPiF), (float)L);
    const float sx = -__ldg(offsets + 2 * b), sy = -__ldg(offsets + 2 * b + 1);
    const float arg = __fadd_rn(__fmul_rn(gx, sx), __fmul_rn(gy, sy));
    float sn, cs;
    sincosf(arg, &sn, &cs);
    y = make_float2(y.x * cs - y.y * sn, y.x * sn + y.y * cs);
  }
  vals[id] = make_float2(y.x * f, y.y * f);
  vals[M + id] = make_float2(f * f / (float)L, 0.0f);
}

}  // namespace

// cuFFT plan of one L^3 transform (kept in the plan's map under key -1)
static int get_fft_coarse(cov3d_plan *p, cufftHandle *out) {
  auto it = p->ffts->find(-1);
  if (it == p->ffts->end()) {
    cufftHandle h;
    COV3D_TRY(check_cufft(cufftPlan3d(&h, p->L, p->L, p->L, CUFFT_C2C), "cufftPlan3d"));
    it = p->ffts->emplace(-1, h).first;
  }
  *out = it->second;
  return check_cufft(cufftSetStream(it->second, p->stream), "cufftSetStream");
}

// 2D transforms of the L planes (axes 1, 2) of an L^3 volume
static int get_fft_coarse_planes(cov3d_plan *p, cufftHandle *out) {
  auto it = p->ffts->find(-4);
  if (it == p->ffts->end()) {
    cufftHandle h;
    int dims[2] = {p->L, p->L};
    COV3D_TRY(check_cufft(cufftPlanMany(&h, 2, dims, nullptr, 1, p->L * p->L, nullptr, 1, p->L * p->L, CUFFT_C2C, p->L),
                          "cufftPlanMany(coarse planes)"));
    it = p->ffts->emplace(-4, h).first;
  }
  *out = it->second;
  return check_cufft(cufftSetStream(it->second, p->stream), "cufftSetStream");
}

static int fft(cufftHandle h, float2 *g, int dir) {
  return check_cufft(cufftExecC2C(h, reinterpret_cast<cufftComplex *>(g), reinterpret_cast<cufftComplex *>(g), dir),
                     "cufftExecC2C");
}

int mean_accumulate(cov3d_plan *p, const void *d_images, const float *d_ctf, const float *d_offsets,
                    const float *d_contrasts, void *d_grids, int accumulate) {
  if (p->point_kind == kPointsNone || p->n_points != p->n_images * (int64_t)p->L * p->L || p->points_L != p->L) {
    set_error("mean_accumulate needs points for n_images x L^2 pixels (setpts / setrot with points_L = L)");
    return COV3D_EINVAL;
  }
  const int64_t M = p->n_points, n3 = (int64_t)p->n * p->n * p->n;
  COV3D_TRY(grow(p->q, M * 16));
  float2 *vals = p->q.as<float2>();
  if (!accumulate) COV3D_TRY(launch_zero(p, d_grids, 2 * n3 * 8));
  mean_values_kernel<<<nb(M), 256, 0, p->stream>>>(static_cast<const float2 *>(d_images), d_ctf, d_offsets,
                                                   d_contrasts, p->n_images, p->L, vals);
  COV3D_LAUNCHED("mean_values_kernel");
  EpilogueArgs e{nullptr, 1, 1.0f / (float)p->L};
  return launch_spread(p, vals, 1, M, 2, e, d_grids, 1, n3, 0);
}

int regularize_lhs(cov3d_plan *p, const void *d_lhs, float *d_out) {
  const int n = p->n;
  const int64_t n3 = (int64_t)n * n * n;
  const int h = n / 2;
  const double rmax = sqrt(3.0 * (double)h * (double)h);
  const int nshell = (int)ceil(rmax);
  if (nshell < 1) {
    set_error("regularize_lhs needs a grid of size >= 2");
    return COV3D_EINVAL;
  }
  COV3D_TRY(grow(p->cgw, (int64_t)2 * nshell * 8));
  double *sums = p->cgw.as<double>(), *counts = sums + nshell;
  COV3D_CUDA(cudaMemsetAsync(sums, 0, (size_t)2 * nshell * 8, p->stream));
  const size_t smem = (size_t)2 * nshell * 8;
  if (smem > 48 * 1024) {
    set_error("regularize_lhs: grid too large for the shell histogram");
    return COV3D_EINVAL;
  }
  shell_sum_kernel<<<n, 256, smem, p->stream>>>(static_cast<const float2 *>(d_lhs), n, nshell, sums, counts);
  COV3D_LAUNCHED("shell_sum_kernel");
  regularize_kernel<<<nb(n3), 256, 0, p->stream>>>(static_cast<const float2 *>(d_lhs), n, nshell, sums, counts, d_out);
  return launched("regularize_kernel");
}

int mean_init(cov3d_plan *p, const void *d_rhs, const float *d_reg, void *d_b, void *d_x0) {
  const int L = p->L, n = p->n;
  const int64_t n3 = (int64_t)n * n * n;
  COV3D_TRY(grow(p->fine, n3 * 8));
  float2 *fine = p->fine.as<float2>();
  cufftHandle h;
  COV3D_TRY(get_fft(p, 1, &h));
  if (d_b) {
    load_centered_kernel<<<nb(n3), 256, 0, p->stream>>>(static_cast<const float2 *>(d_rhs), nullptr, nullptr, n, fine);
    COV3D_LAUNCHED("load_centered_kernel");
    COV3D_TRY(fft(h, fine, CUFFT_INVERSE));
    crop_kernel<<<capped((int64_t)L * L), 256, 0, p->stream>>>(fine, L, n, static_cast<float2 *>(d_b), 0, nullptr, nullptr);
    COV3D_LAUNCHED("crop_kernel");
  }
  if (d_x0) {
    load_centered_kernel<<<nb(n3), 256, 0, p->stream>>>(static_cast<const float2 *>(d_rhs), nullptr, d_reg, n, fine);
    COV3D_LAUNCHED("load_centered_kernel");
    COV3D_TRY(fft(h, fine, CUFFT_INVERSE));
    crop_kernel<<<capped((int64_t)L * L), 256, 0, p->stream>>>(fine, L, n, static_cast<float2 *>(d_x0), 1, nullptr, nullptr);
    COV3D_LAUNCHED("crop_kernel");
  }
  return COV3D_OK;
}

int circulant_symbol(cov3d_plan *p, const float *d_reg, float *d_sym) {
  const int L = p->L, n = p->n;
  const int64_t n3 = (int64_t)n * n * n, L3 = (int64_t)L * L * L;
  COV3D_TRY(grow(p->fine, n3 * 8));
  COV3D_TRY(grow(p->cgw, L3 * 8));
  float2 *fine = p->fine.as<float2>(), *c = p->cgw.as<float2>();
  cufftHandle h, hc;
  COV3D_TRY(get_fft(p, 1, &h));
  COV3D_TRY(get_fft_coarse(p, &hc));
  load_centered_kernel<<<nb(n3), 256, 0, p->stream>>>(nullptr, d_reg, nullptr, n, fine);
  COV3D_LAUNCHED("load_centered_kernel");
  COV3D_TRY(fft(h, fine, CUFFT_INVERSE));
  circulant_gather_kernel<<<nb(L3), 256, 0, p->stream>>>(fine, L, n, c);
  COV3D_LAUNCHED("circulant_gather_kernel");
  COV3D_TRY(fft(hc, c, CUFFT_FORWARD));
  symbol_store_kernel<<<nb(L3), 256, 0, p->stream>>>(c, L, 1e-30f, d_sym);
  return launched("symbol_store_kernel");
}

int cg_solve(cov3d_plan *p, const float *d_lhs, const void *d_b, void *d_x, double rtol, int maxiter, int precond,
             const float *d_sym, int *iters, double *relres, double *d_history, int poll_every) {
  const int L = p->L, n = p->n;
  const int64_t L3 = (int64_t)L * L * L, n3 = (int64_t)n * n * n;
  // workspace: state, r, p, Ap, z
  const int64_t state_bytes = 256;
  COV3D_TRY(grow(p->cgw, state_bytes + 4 * L3 * 8));
  COV3D_TRY(grow(p->fine, n3 * 8));
  CgState *st = p->cgw.as<CgState>();
  float2 *r = reinterpret_cast<float2 *>(p->cgw.as<char>() + state_bytes);
  float2 *pv = r + L3, *ap = pv + L3, *z = ap + L3;
  float2 *fine = p->fine.as<float2>();
  const float2 *b = static_cast<const float2 *>(d_b);
  float2 *x = static_cast<float2 *>(d_x);
  cudaStream_t s = p->stream;
  cufftHandle h, hc = 0, hp = 0, h0 = 0;
  COV3D_TRY(get_fft(p, 1, &h));
  // the L^3 preconditioner: 2D transforms of the L planes around the fused axis-0 kernel where
  // it covers L, else a cuFFT 3D transform and fine_diag_kernel
  const bool coarse_fused = precond == 2 && axis0_fused_size(L);
  cufftHandle hcp = 0;
  if (coarse_fused) COV3D_TRY(get_fft_coarse_planes(p, &hcp));
  else if (precond == 2) COV3D_TRY(get_fft_coarse(p, &hc));
  // even L: pruned transforms (the input has L nonzero planes, only L planes of the output are
  // kept): 2D FFTs over the support planes and an out-of-place 1D FFT along axis 0 into `full`,
  // whose other planes the 2D inverse never needs; `fine` keeps zeros off its support planes
  const bool pruned = (L % 2 == 0) && n >= L + 2;
  // with pruning and a grid size the fused axis-0 kernel covers, the axis-0 transforms and the
  // diagonal are one in-place pass over the support planes of `fine`
  const bool fused = pruned && axis0_fused_size(n);
  // for n = 128 .. 512 the whole operator runs on hand-written line DFTs (no cuFFT)
  const bool lines3 = fused && pruned3_size(n) && p->n == n;
  float2 *full = fine;
  if (pruned) {
    if (!fused) {
      COV3D_TRY(grow(p->fine2, n3 * 8));
      full = p->fine2.as<float2>();
      COV3D_TRY(get_fft_axis0(p, &h0));
    }
    if (!lines3) {
      COV3D_TRY(get_fft_planes(p, &hp));
      COV3D_CUDA(cudaMemsetAsync(fine, 0, (size_t)n3 * 8, s));
    }
  }
  const int64_t half_off = (int64_t)(n - L / 2) * n * n;  // second block of support planes
  COV3D_CUDA(cudaMemsetAsync(st, 0, sizeof(CgState), s));

  // out = crop(ifft3(diag^(+-1) * fft3(pad(in)))), with <p, out> into st->pap when dotp is given
  auto apply_op = [&](const float2 *in, float2 *out, int divide, const float2 *dotp, const CgState *gate) -> int {
    if (lines3) return pruned3(p, in, fine, out, dotp, d_lhs, divide, L, n, gate, st);
    if (fused) {
      pad_support_kernel<<<capped((int64_t)L * n), 256, 0, s>>>(in, L, n, fine, gate);
      COV3D_LAUNCHED("pad_support_kernel");
      COV3D_TRY(fft2(hp, fine, fine, CUFFT_FORWARD));
      COV3D_TRY(fft2(hp, fine + half_off, fine + half_off, CUFFT_FORWARD));
      COV3D_TRY(launch_axis0_diag(p, fine, d_lhs, L, n, divide, 1.0f, gate));
      COV3D_TRY(fft2(hp, fine, fine, CUFFT_INVERSE));
      COV3D_TRY(fft2(hp, fine + half_off, fine + half_off, CUFFT_INVERSE));
      crop_kernel<<<capped((int64_t)L * L), 256, 0, s>>>(fine, L, n, out, 0, dotp,
                                                          dotp ? st : const_cast<CgState *>(gate));
      return launched("crop_kernel");
    }
    if (pruned) {
      pad_support_kernel<<<capped((int64_t)L * n), 256, 0, s>>>(in, L, n, fine, gate);
      COV3D_LAUNCHED("pad_support_kernel");
      COV3D_TRY(fft2(hp, fine, fine, CUFFT_FORWARD));
      COV3D_TRY(fft2(hp, fine + half_off, fine + half_off, CUFFT_FORWARD));
      COV3D_TRY(fft2(h0, fine, full, CUFFT_FORWARD));
    } else {
      pad_kernel<<<capped((int64_t)n * n), 256, 0, s>>>(in, L, n, fine, gate);
      COV3D_LAUNCHED("pad_kernel");
      COV3D_TRY(fft(h, fine, CUFFT_FORWARD));
    }
    fine_diag_kernel<<<capped((int64_t)n * n), 256, 0, s>>>(full, d_lhs, n, divide, 1.0f, gate);
    COV3D_LAUNCHED("fine_diag_kernel");
    if (pruned) {
      COV3D_TRY(fft2(h0, full, full, CUFFT_INVERSE));
      COV3D_TRY(fft2(hp, full, full, CUFFT_INVERSE));
      COV3D_TRY(fft2(hp, full + half_off, full + half_off, CUFFT_INVERSE));
    } else {
      COV3D_TRY(fft(h, fine, CUFFT_INVERSE));
    }
    crop_kernel<<<capped((int64_t)L * L), 256, 0, s>>>(full, L, n, out, 0, dotp,
                                                        dotp ? st : const_cast<CgState *>(gate));
    return launched("crop_kernel");
  };
  auto apply_A = [&](const float2 *in, float2 *out, const float2 *dotp, const CgState *gate) -> int {
    return apply_op(in, out, 0, dotp, gate);
  };
  // z = M(r)
  auto apply_M = [&](const float2 *in, float2 *out, const CgState *gate) -> int {
    if (precond == 1) return apply_op(in, out, 1, nullptr, gate);
    if (coarse_fused) {
      COV3D_TRY(fft2(hcp, in, out, CUFFT_FORWARD));
      COV3D_TRY(launch_axis0_diag(p, out, d_sym, 2 * L, L, 1, 1.0f / (float)L3, gate));
      return fft2(hcp, out, out, CUFFT_INVERSE);
    }
    copy_kernel<<<nb(L3), 256, 0, s>>>(in, out, L3);
    COV3D_LAUNCHED("copy_kernel");
    COV3D_TRY(fft(hc, out, CUFFT_FORWARD));
    fine_diag_kernel<<<capped((int64_t)L * L), 256, 0, s>>>(out, d_sym, L, 1, 1.0f / (float)L3, gate);
    COV3D_LAUNCHED("fine_diag_kernel");
    return fft(hc, out, CUFFT_INVERSE);
  };

  // r = b - A x0;  z = M r;  p = z
  COV3D_TRY(apply_A(x, r, nullptr, nullptr));
  residual_kernel<<<capped(nb(L3)), 256, 0, s>>>(b, r, L3, st);
  COV3D_LAUNCHED("residual_kernel");
  if (precond) {
    COV3D_TRY(apply_M(r, z, nullptr));
    dot_rz_kernel<<<capped(nb(L3)), 256, 0, s>>>(r, z, L3, st);
    COV3D_LAUNCHED("dot_rz_kernel");
    copy_kernel<<<nb(L3), 256, 0, s>>>(z, pv, L3);
  } else {
    copy_kernel<<<nb(L3), 256, 0, s>>>(r, pv, L3);
  }
  COV3D_LAUNCHED("copy_kernel");
  init_kernel<<<1, 1, 0, s>>>(st, precond ? 1 : 0, d_history);
  COV3D_LAUNCHED("init_kernel");
  CgState hs{};
  COV3D_CUDA(cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  COV3D_CUDA(cudaStreamSynchronize(s));
  if (hs.b2 == 0.0) {  // b = 0: the solution is 0 (the reference would divide 0 by 0)
    COV3D_CUDA(cudaMemsetAsync(x, 0, L3 * 8, s));
    if (iters) *iters = 0;
    if (relres) *relres = 0.0;
    return COV3D_OK;
  }

  for (int it = 0; it < maxiter; ++it) {
    COV3D_TRY(apply_A(pv, ap, pv, st));
    update_kernel<<<capped(nb(L3)), 256, 0, s>>>(x, r, pv, ap, L3, st);
    COV3D_LAUNCHED("update_kernel");
    check_kernel<<<1, 1, 0, s>>>(st, rtol, precond ? 1 : 0, d_history, maxiter);
    COV3D_LAUNCHED("check_kernel");
    const float2 *zz = r;
    if (precond) {
      COV3D_TRY(apply_M(r, z, st));
      dot_rz_kernel<<<capped(nb(L3)), 256, 0, s>>>(r, z, L3, st);
      COV3D_LAUNCHED("dot_rz_kernel");
      zz = z;
    }
    direction_kernel<<<capped(nb(L3)), 256, 0, s>>>(pv, zz, L3, st);
    COV3D_LAUNCHED("direction_kernel");
    roll_kernel<<<1, 1, 0, s>>>(st);
    COV3D_LAUNCHED("roll_kernel");
    if ((it + 1) % poll_every == 0 || it + 1 == maxiter) {
      COV3D_CUDA(cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
      COV3D_CUDA(cudaStreamSynchronize(s));
      if (hs.done) break;
    }
  }
  COV3D_CUDA(cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  COV3D_CUDA(cudaStreamSynchronize(s));
  const double rel = sqrt(hs.rr_new / hs.b2);
  if (iters) *iters = hs.iters;
  if (relres) *relres = rel;
  if (hs.done == 3 || !(rel == rel)) {
    set_error("CG produced a non-finite residual");
    return COV3D_ENONFINITE;
  }
  if (hs.done != 1) {
    set_error("CG stopped at maxiter=%d with relative residual %.3e", maxiter, rel);
    return COV3D_EMAXITER;
  }
  return COV3D_OK;
}

}  // namespace cov3d

using namespace cov3d;

extern "C" {

int cov3d_mean_accumulate(cov3d_plan *plan, const void *d_images, const float *d_ctf, const float *d_offsets,
                          const float *d_contrasts, void *d_grids, int accumulate) {
  if (!plan || plan->n <= 0 || !d_images || !d_grids) {
    set_error("invalid mean_accumulate arguments");
    return COV3D_EINVAL;
  }
  return mean_accumulate(plan, d_images, d_ctf, d_offsets, d_contrasts, d_grids, accumulate);
}

int cov3d_regularize_lhs(cov3d_plan *plan, const void *d_lhs, float *d_reg_lhs) {
  if (!plan || plan->n <= 0 || !d_lhs || !d_reg_lhs) {
    set_error("invalid regularize_lhs arguments");
    return COV3D_EINVAL;
  }
  return regularize_lhs(plan, d_lhs, d_reg_lhs);
}

int cov3d_mean_init(cov3d_plan *plan, const void *d_rhs, const float *d_reg_lhs, void *d_b, void *d_x0) {
  if (!plan || plan->n <= 0 || !d_rhs || (d_x0 && !d_reg_lhs) || (!d_b && !d_x0)) {
    set_error("invalid mean_init arguments");
    return COV3D_EINVAL;
  }
  return mean_init(plan, d_rhs, d_reg_lhs, d_b, d_x0);
}

int cov3d_circulant_symbol(cov3d_plan *plan, const float *d_reg_lhs, float *d_symbol) {
  if (!plan || plan->n <= 0 || !d_reg_lhs || !d_symbol) {
    set_error("invalid circulant_symbol arguments");
    return COV3D_EINVAL;
  }
  return circulant_symbol(plan, d_reg_lhs, d_symbol);
}

int cov3d_cg_solve(cov3d_plan *plan, const float *d_reg_lhs, const void *d_b, void *d_x, double rtol, int maxiter,
                   int precond, const float *d_symbol, int *iters, double *relres, double *d_history) {
  if (!plan || plan->n <= 0 || !d_reg_lhs || !d_b || !d_x || maxiter < 1 || !(rtol > 0.0) || precond < 0 ||
      precond > 2 || (precond == 2 && !d_symbol)) {
    set_error("invalid cg_solve arguments");
    return COV3D_EINVAL;
  }
  return cg_solve(plan, d_reg_lhs, d_b, d_x, rtol, maxiter, precond, d_symbol, iters, relres, d_history, 8);
}

}  // extern "C"
