// Mean-volume reconstruction on the device: backprojection of the images and of the squared
// CTFs into the centered fine grid (reference reconstruct_mean, mean.py:145-259), the
// shell-floor regularisation of the kernel (regularize_lhs, mean.py:135-142), the
// Fourier-diagonal first solve, and the conjugate-gradient correction for the zero padding
// (complex_conjugate_gradient + correct_upsampling_padding, mean.py:43-132):
//
//   A(x) = crop_L( ifft3( lhs * fft3( pad_n(x) ) ) )      (centered transforms, ifft / n^3)
//
// For even L and fine grids of n = 128 .. 512 the operator runs on the hand-written pruned line
// DFTs of line_fft.cu (pad, crop and the diagonal fused in); at n = 64 the axis-0 transform
// and the diagonal are fused between cuFFT 2D transforms of the support planes; otherwise it is
// pad + cuFFT + diagonal multiply + inverse cuFFT + crop.  The vector updates
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
  const bool lines3 = fused && line_transforms_apply(p) && p->n == n;
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
    const int *stop = gate ? &gate->done : nullptr;
    if (lines3) return cg_operator_lines(p, in, fine, out, dotp, d_lhs, divide, stop, dotp ? &st->done : stop, st->pap);
    if (fused) {
      pad_support_kernel<<<capped((int64_t)L * n), 256, 0, s>>>(in, L, n, fine, gate);
      COV3D_LAUNCHED("pad_support_kernel");
      COV3D_TRY(fft2(hp, fine, fine, CUFFT_FORWARD));
      COV3D_TRY(fft2(hp, fine + half_off, fine + half_off, CUFFT_FORWARD));
      COV3D_TRY(launch_axis0_diag(p, fine, d_lhs, L, n, divide, 1.0f, stop));
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
      COV3D_TRY(launch_axis0_diag(p, out, d_sym, 2 * L, L, 1, 1.0f / (float)L3, gate ? &gate->done : nullptr));
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

  // one iteration: every kernel is a no-op once the device state says done
  auto iteration = [&]() -> int {
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
    return launched("roll_kernel");
  };
  // poll_every iterations captured once as a CUDA graph on a side stream (a capture cannot run
  // on the legacy default stream), then replayed on the plan's stream until the state says done:
  // one launch per poll_every iterations instead of about 14 per iteration (learned-PC solve at
  // L = 128: 0.221 -> 0.194 s, plain CG 1.39 -> 1.25 s)
  {
    const cudaStream_t s0 = s;
    cudaStream_t cs = nullptr;
    COV3D_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    const cufftHandle hs_all[] = {h, hc, hp, h0, hcp};
    auto set_streams = [&](cudaStream_t to) -> int {
      p->stream = to;
      s = to;
      for (cufftHandle hh : hs_all)
        if (hh) COV3D_TRY(check_cufft(cufftSetStream(hh, to), "cufftSetStream"));
      return COV3D_OK;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const long long l0 = cov3d_launch_count();
    int rc = set_streams(cs);
    if (rc == COV3D_OK) rc = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
    if (rc == COV3D_OK) {
      for (int k = 0; k < poll_every && rc == COV3D_OK; ++k) rc = iteration();
      const int rc2 = check_cuda(cudaStreamEndCapture(cs, &graph), "end capture");
      if (rc == COV3D_OK) rc = rc2;
    }
    const long long per_replay = cov3d_launch_count() - l0;
    const int rc3 = set_streams(s0);
    if (rc == COV3D_OK) rc = rc3;
    if (rc == COV3D_OK) rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
    for (int it = 0; rc == COV3D_OK && it < maxiter; it += poll_every) {
      rc = check_cuda(cudaGraphLaunch(exec, s0), "graph launch");
      count_launches(per_replay);
      if (rc == COV3D_OK) rc = check_cuda(cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s0), "poll");
      if (rc == COV3D_OK) rc = check_cuda(cudaStreamSynchronize(s0), "poll sync");
      if (rc == COV3D_OK && hs.done) break;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (rc != COV3D_OK) return rc;
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
