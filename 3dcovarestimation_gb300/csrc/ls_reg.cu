// Fourier regulariser of the least-squares covariance cost, inside the fused step
// (covar_sgd.py:1308-1313, cost_fourier_domain):
//
//   R = s * sum_ab |K_ab|^2,  K = X X^H,  X = reshape(sqrt(fr) * G, (n, r n^2)),  s = reg_scale / L^4
//
// where G is the (r, n, n, n) centered Fourier grid of the eigenvolumes.  The reference takes
// the reshape's row count from vols[0].shape[0], i.e. the fine-grid size n, so row a of X holds
// the centered planes a*r .. a*r + r - 1 of the flattened (channel, axis-0) index; K is n x n.
// Its conjugate-Wirtinger derivative, added to the gradient grid before the spread, is
//
//   dR / d conj(G) = 2 s sqrt(fr) * unreshape(K X).
//
// The contractions are plain complex GEMMs over r n^2 (FP32, cuBLAS: a Hermitian rank-k update
// for K and a Hermitian multiply for K X); the kernels here gather X from the FFT-native grid,
// reduce R and scatter the derivative back.

#include <cublas_v2.h>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

// One block per (channel, storage plane, storage row): X[c][centered cell] = sqrt(fr) * G[c][cell].
__global__ void ls_gather_kernel(const float2 *__restrict__ g, const float *__restrict__ fr, int64_t frs, int nchan,
                                 int n, float2 *__restrict__ x) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  for (int64_t row = blockIdx.x; row < nchan * n2; row += gridDim.x) {
    const int c = (int)(row / n2);
    const int64_t rr = row - c * n2;
    const int s0 = (int)(rr / n), s1 = (int)(rr - (int64_t)s0 * n);
    const int64_t crow = ((int64_t)native_to_centered(s0, n) * n + native_to_centered(s1, n)) * n;
    const float2 *src = g + c * n3 + rr * n;
    const float *f = fr + c * frs + crow;
    float2 *dst = x + c * n3 + crow;
    for (int s2 = threadIdx.x; s2 < n; s2 += blockDim.x) {
      const int c2 = native_to_centered(s2, n);
      const float w = sqrtf(__ldg(f + c2));
      const float2 v = src[s2];
      dst[c2] = make_float2(w * v.x, w * v.y);
    }
  }
}

// gg[c][cell] += coef * sqrt(fr) * Y[c][centered cell]
__global__ void ls_scatter_kernel(const float2 *__restrict__ y, const float *__restrict__ fr, int64_t frs, int nchan,
                                  int n, float coef, float2 *__restrict__ gg) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  for (int64_t row = blockIdx.x; row < nchan * n2; row += gridDim.x) {
    const int c = (int)(row / n2);
    const int64_t rr = row - c * n2;
    const int s0 = (int)(rr / n), s1 = (int)(rr - (int64_t)s0 * n);
    const int64_t crow = ((int64_t)native_to_centered(s0, n) * n + native_to_centered(s1, n)) * n;
    const float2 *src = y + c * n3 + crow;
    const float *f = fr + c * frs + crow;
    float2 *dst = gg + c * n3 + rr * n;
    for (int s2 = threadIdx.x; s2 < n; s2 += blockDim.x) {
      const int c2 = native_to_centered(s2, n);
      const float w = coef * sqrtf(__ldg(f + c2));
      const float2 v = src[c2];
      const float2 o = dst[s2];
      dst[s2] = make_float2(fmaf(w, v.x, o.x), fmaf(w, v.y, o.y));
    }
  }
}

// s * sum_ab |K_ab|^2 from the lower triangle of the Hermitian K (column-major, n x n), in FP64.
__global__ void ls_value_kernel(const float2 *__restrict__ k, int n, double s, double *__restrict__ acc) {
  double part = 0.0;
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    if (i < j) continue;
    const float2 v = k[e];
    const double a = (double)v.x * v.x + (double)v.y * v.y;
    part += i == j ? a : 2.0 * a;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  __shared__ double wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wsum[warp] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
    if (t != 0.0) atomicAdd(acc, s * t);
  }
}

int check_blas(cublasStatus_t st, const char *what) {
  if (st == CUBLAS_STATUS_SUCCESS) return COV3D_OK;
  set_error("%s failed (cuBLAS status %d)", what, (int)st);
  return COV3D_ECUDA;
}

}  // namespace

void release_blas(cov3d_plan *p) {
  if (p->blas) cublasDestroy(static_cast<cublasHandle_t>(p->blas));
  p->blas = nullptr;
}

// The regulariser's workspace (X, K X and K: 2 r n^3 + n^2 complex) and the cuBLAS handle,
// created once; later calls at the same or a smaller rank allocate nothing.
int reserve_ls_reg(cov3d_plan *p, int r) {
  const int64_t n = p->n;
  COV3D_TRY(grow(p->lsw, (2 * r * n * n * n + n * n) * 8));
  if (!p->blas) {
    cublasHandle_t h = nullptr;
    COV3D_TRY(check_blas(cublasCreate(&h), "cublasCreate"));
    p->blas = h;
    COV3D_TRY(check_blas(cublasSetMathMode(h, CUBLAS_DEFAULT_MATH), "cublasSetMathMode"));  // FP32, no TF32
  }
  return COV3D_OK;
}

int launch_ls_reg(cov3d_plan *p, const void *grid, void *ggrid, const float *fr, int64_t fr_stride, int r, double s,
                  double *cost_acc) {
  const int n = p->n;
  const int64_t n3 = (int64_t)n * n * n;
  const int64_t kdim = (int64_t)r * n * n;  // length of a row of X
  if (kdim > 0x7fffffff) {
    set_error("least-squares regulariser: r * n^2 = %lld exceeds the GEMM's int range", (long long)kdim);
    return COV3D_EINVAL;
  }
  COV3D_TRY(reserve_ls_reg(p, r));
  float2 *x = p->lsw.as<float2>();
  float2 *y = x + r * n3;
  float2 *kmat = y + r * n3;
  cublasHandle_t h = static_cast<cublasHandle_t>(p->blas);
  COV3D_TRY(check_blas(cublasSetStream(h, p->stream), "cublasSetStream"));
  const unsigned rows = (unsigned)(r * (int64_t)n * n < 4864 ? r * (int64_t)n * n : 4864);
  ls_gather_kernel<<<rows, 128, 0, p->stream>>>(static_cast<const float2 *>(grid), fr, fr_stride, r, n, x);
  COV3D_LAUNCHED("ls_gather_kernel");
  // X as a column-major kdim x n matrix Xt (its memory, row-major n x kdim): Xt^H Xt = conj(K)
  // (= K^T, Hermitian), lower triangle; then Xt conj(K) = (K X)^T, i.e. K X in row-major memory
  const float one = 1.0f, zero = 0.0f;
  const cuComplex cone = make_cuComplex(1.0f, 0.0f), czero = make_cuComplex(0.0f, 0.0f);
  COV3D_TRY(check_blas(cublasCherk(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_C, n, (int)kdim, &one,
                                   reinterpret_cast<const cuComplex *>(x), (int)kdim, &zero,
                                   reinterpret_cast<cuComplex *>(kmat), n),
                       "cublasCherk"));
  ls_value_kernel<<<64, 256, 0, p->stream>>>(kmat, n, s, cost_acc);
  COV3D_LAUNCHED("ls_value_kernel");
  COV3D_TRY(check_blas(cublasChemm(h, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, (int)kdim, n, &cone,
                                   reinterpret_cast<const cuComplex *>(kmat), n, reinterpret_cast<const cuComplex *>(x),
                                   (int)kdim, &czero, reinterpret_cast<cuComplex *>(y), (int)kdim),
                       "cublasChemm"));
  ls_scatter_kernel<<<rows, 128, 0, p->stream>>>(y, fr, fr_stride, r, n, (float)(2.0 * s),
                                                  static_cast<float2 *>(ggrid));
  return launched("ls_scatter_kernel");
}

}  // namespace cov3d
