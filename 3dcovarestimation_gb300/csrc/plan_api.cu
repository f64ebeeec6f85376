// C ABI entry points: plan lifecycle, point setting, the NUFFT / projection operators and the
// fused covariance cost.  Declarations and reference citations are in include/cov3d_gb300.h.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <new>
#include <vector>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {
thread_local char g_err[512] = "";
}

namespace {
std::atomic<long long> g_launches{0};
const char *kPhaseNames[kNumPhases] = {"sort", "pack", "fft_forward", "interp", "gram", "solve",
                                       "wpass", "spread", "regulariser", "fft_inverse", "unpack"};
}  // namespace

int launched(const char *name) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return check_cuda(cudaGetLastError(), name);
}

void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

PhaseScope::PhaseScope(cov3d_plan *p, int phase) : p_(p) {
  if (!p->timing) return;
  auto &pool = *p->ev_pool;
  while (pool.size() < p->ev_next + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      p_ = nullptr;
      return;
    }
    pool.push_back(e);
  }
  cudaEvent_t start = pool[p->ev_next];
  stop_ = pool[p->ev_next + 1];
  p->ev_next += 2;
  p->ev_phase->push_back(phase);
  cudaEventRecord(start, p->stream);
}

PhaseScope::~PhaseScope() {
  if (p_ && p_->timing && stop_) cudaEventRecord(stop_, p_->stream);
}

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return COV3D_OK;
  set_error("%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return COV3D_ENOMEM;
  }
  return COV3D_ECUDA;
}

int check_cufft(cufftResult r, const char *what) {
  if (r == CUFFT_SUCCESS) return COV3D_OK;
  set_error("%s: cuFFT error %d", what, (int)r);
  return r == CUFFT_ALLOC_FAILED ? COV3D_ENOMEM : COV3D_ECUFFT;
}

int grow(DevBuf &b, int64_t bytes) {
  if (bytes <= b.cap) return COV3D_OK;
  if (b.ptr) {
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.cap = 0;
  }
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, (size_t)bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc(%lld bytes) failed: %s", (long long)bytes, cudaGetErrorString(e));
    return COV3D_ENOMEM;
  }
  b.ptr = p;
  b.cap = bytes;
  return COV3D_OK;
}

void release(DevBuf &b) {
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.cap = 0;
}

PointGeom make_geom(const cov3d_plan *p) {
  PointGeom g{};
  g.kind = p->point_kind;
  g.pts = p->pts.as<float>();
  g.rot = p->rot.as<float>();
  g.Lp = p->points_L;
  g.P = p->points_L * p->points_L;
  g.n = p->n;
  g.mapping = p->kernel == COV3D_KERNEL_ES ? kMapES : kMapGridSample;
  g.wrap = p->wrap;
  g.s_es = (float)((double)p->n / (2.0 * kPi));
  g.half_n = (float)(p->n / 2);
  g.gs_scale = (float)(((double)p->n / (double)(p->n - 1)) / kPi);
  g.gs_off = (p->n % 2 == 0) ? (float)(1.0 / (double)(p->n - 1)) : 0.0f;
  g.plane_half = 0.5f * (float)p->points_L;
  return g;
}

KernelSpec make_kernel(const cov3d_plan *p) {
  KernelSpec k{};
  k.type = p->kernel;
  k.width = p->kernel == COV3D_KERNEL_NEAREST ? 1 : p->kernel == COV3D_KERNEL_LINEAR ? 2 : p->width;
  k.beta = (float)p->beta;
  k.periodic = p->kernel == COV3D_KERNEL_ES ? 1 : 0;
  return k;
}

namespace {

// Gauss-Legendre nodes and weights on [-1, 1] by Newton iteration on P_N.
void gauss_legendre(int N, std::vector<double> &x, std::vector<double> &w) {
  x.assign(N, 0.0);
  w.assign(N, 0.0);
  for (int i = 0; i < N; ++i) {
    double z = std::cos(kPi * (i + 0.75) / (N + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= N; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = N * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-15) break;
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

double es_value(double x, int width, double beta) {
  const double u = 2.0 * x / width;
  if (std::fabs(u) >= 1.0) return 0.0;
  return std::exp(beta * (std::sqrt(1.0 - u * u) - 1.0));
}

// psi_hat(alpha) = 2 * int_0^{w/2} psi(x) cos(alpha x) dx
double es_fourier(double alpha, int width, double beta, const std::vector<double> &xq, const std::vector<double> &wq) {
  const double half = width / 2.0;
  double s = 0.0;
  for (size_t i = 0; i < xq.size(); ++i) {
    const double x = (xq[i] + 1.0) * half / 2.0;
    s += wq[i] * half / 2.0 * es_value(x, width, beta) * std::cos(alpha * x);
  }
  return 2.0 * s;
}

// Per-axis deapodisation factors for voxel j (offset k = j - L/2).
void grid_correction_1d(const cov3d_plan *p, std::vector<double> &g) {
  const int L = p->L;
  g.assign(L, 1.0);
  if (p->kernel == COV3D_KERNEL_ES) {
    std::vector<double> xq, wq;
    gauss_legendre(200, xq, wq);
    for (int j = 0; j < L; ++j) {
      const int k = j - L / 2;
      g[j] = es_fourier(2.0 * kPi * k / p->n, p->width, p->beta, xq, wq);
    }
  } else {
    // covar.py:55-63: pixel_pos = pi * (arange(-(L//2), (L-1)//2+1) / L) / upsample, sinc,
    // values below 1e-6 replaced by 1, squared for bilinear
    for (int j = 0; j < L; ++j) {
      const double pos = kPi * ((double)(j - L / 2) / L) / p->upsample;
      double s = pos == 0.0 ? 1.0 : std::sin(pos) / pos;
      if (s < 1e-6) s = 1.0;
      if (p->kernel == COV3D_KERNEL_LINEAR) s = s * s;
      g[j] = s;
    }
  }
}

int finish_points(cov3d_plan *p) {
  p->n_points = p->n_images * (int64_t)p->points_L * p->points_L;
  PhaseScope ps(p, kPhaseSort);
  return sort_points(p);
}

bool valid(const cov3d_plan *p) { return p != nullptr && p->n > 0; }

}  // namespace
}  // namespace cov3d

using namespace cov3d;

extern "C" {

int cov3d_abi_version(void) { return COV3D_ABI_VERSION; }

int cov3d_last_error(char *buf, int len) {
  if (!buf || len <= 0) return COV3D_EINVAL;
  std::snprintf(buf, (size_t)len, "%s", g_err);
  return COV3D_OK;
}

const char *cov3d_status_string(int status) {
  switch (status) {
    case COV3D_OK: return "ok";
    case COV3D_EINVAL: return "invalid argument";
    case COV3D_ENOMEM: return "out of device memory";
    case COV3D_ECUDA: return "CUDA error";
    case COV3D_ECUFFT: return "cuFFT error";
    case COV3D_ENONFINITE: return "non-finite value";
    case COV3D_EMAXITER: return "maximum number of iterations reached";
    case COV3D_ESTATE: return "call out of order";
    default: return "unknown status";
  }
}

int cov3d_plan_create(int L, int n_trans, double eps, const cov3d_opts *opts, cov3d_plan **out) {
  if (!out) {
    set_error("plan output pointer is null");
    return COV3D_EINVAL;
  }
  *out = nullptr;
  cov3d_opts o{};
  o.kernel = COV3D_KERNEL_ES;
  o.upsample = 2;
  o.compensated = 1;
  if (opts) o = *opts;
  if (o.upsample <= 0) o.upsample = 2;
  if (L < 2 || L > 1024 || n_trans < 1 || n_trans > 64) {
    set_error("invalid plan size L=%d n_trans=%d", L, n_trans);
    return COV3D_EINVAL;
  }
  if (o.kernel < COV3D_KERNEL_ES || o.kernel > COV3D_KERNEL_NEAREST) {
    set_error("unknown kernel %d", o.kernel);
    return COV3D_EINVAL;
  }
  const int n = L * o.upsample;
  if (n > 2048) {
    set_error("fine grid n=%d too large", n);
    return COV3D_EINVAL;
  }
  cov3d_plan *p = new (std::nothrow) cov3d_plan();
  if (!p) {
    set_error("host allocation failed");
    return COV3D_ENOMEM;
  }
  p->L = L;
  p->n = n;
  p->upsample = o.upsample;
  p->kernel = o.kernel;
  p->n_trans = n_trans;
  p->compensated = o.compensated ? 1 : 0;
  p->stream = static_cast<cudaStream_t>(o.stream);
  if (o.kernel == COV3D_KERNEL_ES) {
    int w = o.width;
    if (w <= 0) {
      // the reference clamps eps to 10x machine epsilon (nufft_plan.py:286)
      const double e = std::fmax(eps, 10.0 * 1.1920928955078125e-07);
      w = (int)std::ceil(-std::log10(e / 10.0));
    }
    if (w < 4 || w > 8) {
      set_error("ES width %d unsupported (4..8)", w);
      delete p;
      return COV3D_EINVAL;
    }
    p->width = w;
    p->beta = o.beta > 0.0 ? o.beta : 0.97 * kPi * (1.0 - 1.0 / (2.0 * o.upsample)) * w;
    // subproblems of up to 416 points: the row-group spreading stages 260 bytes per point, and
    // 416 points are the most that keep two of its blocks on an SM; fewer subproblems flush
    // fewer tile rows (spread 17.5 -> 16.6 ms against 288 points)
    p->max_sub = 416;
  } else {
    p->width = o.kernel == COV3D_KERNEL_LINEAR ? 2 : 1;
    p->beta = 0.0;
    // the narrow windows' spreading stages about 284 bytes per point: 384 points keep two blocks
    // per SM (bilinear spread 4.62 -> 4.36 ms against 288)
    p->max_sub = 384;
  }
  const int bs = 8;
  if (o.bin_size != 0 && o.bin_size != 8) {
    set_error("bin_size must be 0 or 8");
    delete p;
    return COV3D_EINVAL;
  }
  for (int d = 0; d < 3; ++d) {
    p->bins.bs[d] = bs;
    p->bins.nb[d] = (n + bs - 1) / bs;
  }
  p->bins.nbins = (int64_t)p->bins.nb[0] * p->bins.nb[1] * p->bins.nb[2];
  p->ffts = new (std::nothrow) std::map<int, cufftHandle>();
  p->ev_pool = new (std::nothrow) std::vector<cudaEvent_t>();
  p->ev_phase = new (std::nothrow) std::vector<int>();
  int st = check_cuda(cudaGetDevice(&p->device), "cudaGetDevice");
  std::vector<double> g;
  grid_correction_1d(p, g);
  std::vector<float> gf(g.begin(), g.end());
  if (st == COV3D_OK) st = grow(p->gc1d, L * 4);
  if (st == COV3D_OK) st = check_cuda(cudaMemcpy(p->gc1d.ptr, gf.data(), L * 4, cudaMemcpyHostToDevice), "cudaMemcpy");
  if (st == COV3D_OK) st = grow(p->acc, 64 * sizeof(double));
  if (st == COV3D_OK) st = check_cuda(cudaMallocHost(&p->h_acc, 64 * sizeof(double)), "cudaMallocHost");
  if (st != COV3D_OK || !p->ffts || !p->ev_pool || !p->ev_phase) {
    cov3d_plan_destroy(p);
    return st != COV3D_OK ? st : COV3D_ENOMEM;
  }
  p->h_gc1d = new double[L];
  for (int j = 0; j < L; ++j) p->h_gc1d[j] = g[j];
  *out = p;
  return COV3D_OK;
}

int cov3d_plan_reserve(cov3d_plan *p, int64_t max_images, int points_L, int nchan, int flags) {
  if (!valid(p) || max_images < 0 || points_L < 1 || nchan < 1 || nchan > p->n_trans) {
    set_error("invalid reserve arguments (nchan must be in 1..n_trans)");
    return COV3D_EINVAL;
  }
  const int64_t P = (int64_t)points_L * points_L;
  const int64_t M = max_images * P;
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  COV3D_TRY(reserve_sort(p, M));
  COV3D_TRY(grow(p->rot, max_images * 9 * 4));
  if (flags & COV3D_RESERVE_POINTS) COV3D_TRY(grow(p->pts, max_images * 3 * P * 4));
  // the covariance step: fine grid and its gradient, projections, per-image matrices
  COV3D_TRY(grow(p->fine, n3 * nchan * 8));
  COV3D_TRY(grow(p->fine2, n3 * nchan * 8));
  COV3D_TRY(grow(p->q, M * nchan * 8));
  COV3D_TRY(grow(p->small, max_images * (nchan * nchan * 8 * 2 + nchan * 8 * 2 + 8 + 8) + 64));
  COV3D_TRY(grow(p->ctfc, max_images * (int64_t)sizeof(CtfCoef)));
  if (line_transforms_apply(p)) COV3D_TRY(ensure_twiddles(p, p->n));
  // the cuFFT plans (and their work areas) of the step's transforms where the line DFTs do not
  // apply: the pruned 2D + axis-0 pair for even L, the full 3D transform of nchan channels else
  cufftHandle h = 0;
  if (prunable(p)) {
    if (!(line_transforms_apply(p) && p->n <= 256)) {
      COV3D_TRY(get_fft_planes(p, &h));
      COV3D_TRY(get_fft_axis0(p, &h));
    }
  } else {
    COV3D_TRY(get_fft(p, nchan, &h));
  }
  if (flags & COV3D_RESERVE_GRAM_BF16) COV3D_TRY(reserve_gram_bf16(p, (int)max_images, (int)P, nchan));
  if (flags & COV3D_RESERVE_LS_REG) COV3D_TRY(reserve_ls_reg(p, nchan));
  return check_cuda(cudaStreamSynchronize(p->stream), "reserve");
}

int cov3d_plan_destroy(cov3d_plan *p) {
  if (!p) return COV3D_OK;
  if (p->ffts) {
    for (auto &kv : *p->ffts) cufftDestroy(kv.second);
    delete p->ffts;
  }
  DevBuf *bufs[] = {&p->gc1d, &p->pts, &p->rot, &p->bin_count, &p->bin_off, &p->sub_off, &p->pt_bin, &p->pt_rank,
                    &p->sorted, &p->sub_bin, &p->sub_first, &p->sub_count, &p->nsub, &p->fine, &p->fine2, &p->q,
                    &p->small, &p->acc, &p->cgw, &p->xbf, &p->gsum, &p->fftw, &p->ctfc, &p->lsw};
  for (DevBuf *b : bufs) release(*b);
  release_blas(p);
  if (p->h_acc) cudaFreeHost(p->h_acc);
  if (p->ev_pool) {
    for (cudaEvent_t e : *p->ev_pool) cudaEventDestroy(e);
    delete p->ev_pool;
  }
  delete p->ev_phase;
  delete[] p->h_gc1d;
  delete p;
  return COV3D_OK;
}

int cov3d_plan_set_stream(cov3d_plan *p, void *stream) {
  if (!valid(p)) {
    set_error("invalid plan");
    return COV3D_EINVAL;
  }
  p->stream = static_cast<cudaStream_t>(stream);
  return COV3D_OK;
}

int cov3d_plan_info(const cov3d_plan *p, int *n, int *width, double *beta) {
  if (!valid(p)) {
    set_error("invalid plan");
    return COV3D_EINVAL;
  }
  if (n) *n = p->n;
  if (width) *width = p->width;
  if (beta) *beta = p->beta;
  return COV3D_OK;
}

int cov3d_setpts(cov3d_plan *p, const float *d_pts, int64_t n_images, int points_L, int64_t img_stride,
                 int64_t row_stride, int wrap) {
  if (!valid(p) || !d_pts || n_images <= 0 || points_L <= 0) {
    set_error("invalid setpts arguments");
    return COV3D_EINVAL;
  }
  const int64_t P = (int64_t)points_L * points_L;
  if (row_stride != P || img_stride < 3 * P) {
    set_error("points must have contiguous rows (row_stride == L^2) and img_stride >= 3 L^2");
    return COV3D_EINVAL;
  }
  COV3D_TRY(grow(p->pts, n_images * 3 * P * 4));
  COV3D_CUDA(cudaMemcpy2DAsync(p->pts.ptr, (size_t)(3 * P * 4), d_pts, (size_t)(img_stride * 4), (size_t)(3 * P * 4),
                               (size_t)n_images, cudaMemcpyDeviceToDevice, p->stream));
  p->point_kind = kPointsExplicit;
  p->n_images = n_images;
  p->points_L = points_L;
  p->wrap = wrap ? 1 : 0;
  return finish_points(p);
}

int cov3d_setrot(cov3d_plan *p, const float *d_rot, int64_t n_images, int points_L) {
  if (!valid(p) || !d_rot || n_images <= 0 || points_L <= 0) {
    set_error("invalid setrot arguments");
    return COV3D_EINVAL;
  }
  COV3D_TRY(grow(p->rot, n_images * 9 * 4));
  COV3D_CUDA(cudaMemcpyAsync(p->rot.ptr, d_rot, (size_t)(n_images * 9 * 4), cudaMemcpyDeviceToDevice, p->stream));
  p->point_kind = kPointsRotations;
  p->n_images = n_images;
  p->points_L = points_L;
  p->wrap = 1;
  return finish_points(p);
}

// The projection epilogue / prologue of a call: the per-pixel filter array, or the CTF computed
// from per-image parameters (coefficients prepared once per call), Nyquist zeroing, scale.
static int epilogue_args(cov3d_plan *p, const float *d_ctf, int flags, float scale, EpilogueArgs *e) {
  e->ctf = (flags & COV3D_APPLY_CTF) && !(flags & COV3D_APPLY_CTF_PARAMS) ? d_ctf : nullptr;
  e->nyquist = (flags & COV3D_APPLY_NYQUIST) ? 1 : 0;
  e->scale = scale;
  e->ctfc = nullptr;
  if (flags & COV3D_APPLY_CTF_PARAMS) COV3D_TRY(prepare_ctf_coef(p, d_ctf, p->n_images, p->points_L, &e->ctfc));
  return COV3D_OK;
}

static int layout_shift(const cov3d_plan *p, const cov3d_grid_layout *l) {
  return l->order == COV3D_GRID_CENTERED ? 0 : p->n - p->n / 2;
}

int cov3d_interp(cov3d_plan *p, const void *d_grid, const cov3d_grid_layout *layout, int nchan, void *d_out,
                 int64_t out_point_stride, int64_t out_chan_stride, const float *d_ctf, int flags, float scale) {
  if (!valid(p) || !d_grid || !layout || !d_out || nchan < 1 || layout->cell_stride < 1 || layout->chan_stride < 0) {
    set_error("invalid interp arguments");
    return COV3D_EINVAL;
  }
  if ((flags & (COV3D_APPLY_CTF | COV3D_APPLY_CTF_PARAMS)) && !d_ctf) {
    set_error("COV3D_APPLY_CTF / COV3D_APPLY_CTF_PARAMS without a filter or parameter array");
    return COV3D_EINVAL;
  }
  GridArgs g{d_grid, layout->cell_stride, layout->chan_stride, layout_shift(p, layout)};
  EpilogueArgs e;
  COV3D_TRY(epilogue_args(p, d_ctf, flags, scale, &e));
  return launch_interp(p, g, nchan, d_out, out_point_stride, out_chan_stride, e);
}

int cov3d_spread(cov3d_plan *p, const void *d_values, int64_t in_point_stride, int64_t in_chan_stride, int nchan,
                 const float *d_ctf, int flags, float scale, void *d_grid, const cov3d_grid_layout *layout,
                 int accumulate) {
  if (!valid(p) || !d_values || !d_grid || !layout || nchan < 1 || layout->cell_stride < 1) {
    set_error("invalid spread arguments");
    return COV3D_EINVAL;
  }
  if ((flags & (COV3D_APPLY_CTF | COV3D_APPLY_CTF_PARAMS)) && !d_ctf) {
    set_error("COV3D_APPLY_CTF / COV3D_APPLY_CTF_PARAMS without a filter or parameter array");
    return COV3D_EINVAL;
  }
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  if (!accumulate) {
    const bool chan_first = layout->cell_stride == 1 && layout->chan_stride == n3;
    const bool chan_last = layout->chan_stride == 1 && layout->cell_stride == nchan;
    if (!chan_first && !chan_last && nchan > 1) {
      set_error("a strided output grid must be zeroed by the caller (accumulate=1)");
      return COV3D_EINVAL;
    }
    COV3D_TRY(launch_zero(p, d_grid, n3 * nchan * 8));
  }
  EpilogueArgs e;
  COV3D_TRY(epilogue_args(p, d_ctf, flags, scale, &e));
  return launch_spread(p, d_values, in_point_stride, in_chan_stride, nchan, e, d_grid, layout->cell_stride,
                       layout->chan_stride, layout_shift(p, layout));
}

int cov3d_spread_unaggregated(cov3d_plan *p, const void *d_values, int64_t in_point_stride, const float *d_ctf,
                              int flags, float scale, void *d_grids) {
  if (!valid(p) || !d_values || !d_grids) {
    set_error("invalid spread_unaggregated arguments");
    return COV3D_EINVAL;
  }
  if (p->kernel == COV3D_KERNEL_ES) {
    set_error("unaggregated spreading is provided for the grid_sample kernels");
    return COV3D_EINVAL;
  }
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  COV3D_TRY(launch_zero(p, d_grids, p->n_images * n3 * 8));
  EpilogueArgs e;
  COV3D_TRY(epilogue_args(p, d_ctf, flags, scale, &e));
  return launch_spread_unaggregated(p, d_values, in_point_stride, e, d_grids);
}

// type 2 with the projection epilogue, output (point, channel) at out[point * ops + ch * ocs]
static int type2(cov3d_plan *p, const float *d_vol_real, const void *d_vol_complex, int nchan, void *d_out,
                 int64_t ops, int64_t ocs, const EpilogueArgs &e) {
  if (!valid(p) || (!d_vol_real && !d_vol_complex) || !d_out || nchan < 1 || nchan > p->n_trans) {
    set_error("invalid type-2 arguments (nchan must be in 1..n_trans)");
    return COV3D_EINVAL;
  }
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  COV3D_TRY(grow(p->fine, n3 * nchan * 8));
  COV3D_TRY(launch_pack(p, d_vol_real, d_vol_complex, nullptr, 1, nchan, p->fine.ptr));
  cufftHandle fft;
  COV3D_TRY(get_fft(p, nchan, &fft));
  COV3D_TRY(check_cufft(cufftExecC2C(fft, p->fine.as<cufftComplex>(), p->fine.as<cufftComplex>(), CUFFT_FORWARD),
                        "cufftExecC2C(forward)"));
  GridArgs g{p->fine.ptr, 1, n3, p->n - p->n / 2};
  return launch_interp(p, g, nchan, d_out, ops, ocs, e);
}

int cov3d_fine_grid(cov3d_plan *p, const float *d_vol_real, const void *d_vol_complex, int nchan, void *d_grid) {
  if (!valid(p) || (!d_vol_real && !d_vol_complex) || !d_grid || nchan < 1 || nchan > p->n_trans) {
    set_error("invalid fine-grid arguments (nchan must be in 1..n_trans)");
    return COV3D_EINVAL;
  }
  COV3D_TRY(launch_pack(p, d_vol_real, d_vol_complex, nullptr, 1, nchan, d_grid));
  cufftHandle fft;
  COV3D_TRY(get_fft(p, nchan, &fft));
  return check_cufft(cufftExecC2C(fft, static_cast<cufftComplex *>(d_grid), static_cast<cufftComplex *>(d_grid),
                                  CUFFT_FORWARD),
                     "cufftExecC2C(forward)");
}

int cov3d_execute_type2(cov3d_plan *p, const float *d_vol_real, const void *d_vol_complex, int nchan, void *d_out) {
  EpilogueArgs e{nullptr, 0, 1.0f};
  return type2(p, d_vol_real, d_vol_complex, nchan, d_out, 1, p ? p->n_points : 0, e);
}

int cov3d_project(cov3d_plan *p, const float *d_vol_real, const void *d_vol_complex, int nchan, void *d_out,
                  int64_t out_point_stride, int64_t out_chan_stride, const float *d_ctf, int flags, float scale) {
  if ((flags & (COV3D_APPLY_CTF | COV3D_APPLY_CTF_PARAMS)) && !d_ctf) {
    set_error("COV3D_APPLY_CTF / COV3D_APPLY_CTF_PARAMS without a filter or parameter array");
    return COV3D_EINVAL;
  }
  if (!valid(p)) {
    set_error("invalid plan");
    return COV3D_EINVAL;
  }
  EpilogueArgs e;
  COV3D_TRY(epilogue_args(p, d_ctf, flags, scale, &e));
  return type2(p, d_vol_real, d_vol_complex, nchan, d_out, out_point_stride, out_chan_stride, e);
}

// type 1 with the backprojection prologue, input (point, channel) at values[point * ips + ch * ics]
static int type1(cov3d_plan *p, const void *d_values, int64_t ips, int64_t ics, int nchan, void *d_vol_out,
                 const EpilogueArgs &e) {
  if (!valid(p) || !d_values || !d_vol_out || nchan < 1 || nchan > p->n_trans) {
    set_error("invalid type-1 arguments (nchan must be in 1..n_trans)");
    return COV3D_EINVAL;
  }
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  COV3D_TRY(grow(p->fine, n3 * nchan * 8));
  COV3D_TRY(launch_zero(p, p->fine.ptr, n3 * nchan * 8));
  COV3D_TRY(launch_spread(p, d_values, ips, ics, nchan, e, p->fine.ptr, 1, n3, p->n - p->n / 2));
  cufftHandle fft;
  COV3D_TRY(get_fft(p, nchan, &fft));
  COV3D_TRY(check_cufft(cufftExecC2C(fft, p->fine.as<cufftComplex>(), p->fine.as<cufftComplex>(), CUFFT_INVERSE),
                        "cufftExecC2C(inverse)"));
  return launch_unpack_complex(p, p->fine.ptr, nchan, 1, d_vol_out);
}

int cov3d_execute_type1(cov3d_plan *p, const void *d_values, int nchan, void *d_vol_out) {
  EpilogueArgs e{nullptr, 0, 1.0f};
  return type1(p, d_values, 1, p ? p->n_points : 0, nchan, d_vol_out, e);
}

int cov3d_backproject(cov3d_plan *p, const void *d_values, int64_t in_point_stride, int64_t in_chan_stride, int nchan,
                      const float *d_ctf, int flags, float scale, void *d_vol_out) {
  if ((flags & (COV3D_APPLY_CTF | COV3D_APPLY_CTF_PARAMS)) && !d_ctf) {
    set_error("COV3D_APPLY_CTF / COV3D_APPLY_CTF_PARAMS without a filter or parameter array");
    return COV3D_EINVAL;
  }
  if (!valid(p)) {
    set_error("invalid plan");
    return COV3D_EINVAL;
  }
  EpilogueArgs e;
  COV3D_TRY(epilogue_args(p, d_ctf, flags, scale, &e));
  return type1(p, d_values, in_point_stride, in_chan_stride, nchan, d_vol_out, e);
}

int cov3d_grid_correction(const cov3d_plan *p, float *d_out) {
  if (!valid(p) || !d_out) {
    set_error("invalid grid_correction arguments");
    return COV3D_EINVAL;
  }
  return launch_gc_volume(p, d_out);
}

int cov3d_covar_cost_grad(cov3d_plan *p, const cov3d_cost_args *args, double *cost, float *d_grad_vectors,
                          float *d_grad_log_sqrt, double *d_per_image_cost) {
  if (!valid(p) || !args) {
    set_error("invalid cost arguments");
    return COV3D_EINVAL;
  }
  return covar_cost_grad(p, args, cost, args->d_cost, d_grad_vectors, d_grad_log_sqrt, d_per_image_cost);
}

long long cov3d_launch_count(void) { return g_launches.load(); }

const char *cov3d_phase_name(int phase) { return phase >= 0 && phase < kNumPhases ? kPhaseNames[phase] : nullptr; }

int cov3d_plan_timing(cov3d_plan *p, int enable) {
  if (!valid(p)) {
    set_error("invalid plan");
    return COV3D_EINVAL;
  }
  p->timing = enable ? 1 : 0;
  p->ev_next = 0;
  p->ev_phase->clear();
  return COV3D_OK;
}

int cov3d_plan_timing_read(cov3d_plan *p, double *ms, int *counts, int n_phases) {
  if (!valid(p) || !ms || !counts || n_phases < kNumPhases) {
    set_error("invalid timing_read arguments (need %d phases)", (int)kNumPhases);
    return COV3D_EINVAL;
  }
  for (int i = 0; i < kNumPhases; ++i) {
    ms[i] = 0.0;
    counts[i] = 0;
  }
  COV3D_CUDA(cudaStreamSynchronize(p->stream));
  const auto &pool = *p->ev_pool;
  for (size_t k = 0; k < p->ev_phase->size(); ++k) {
    float t = 0.f;
    COV3D_CUDA(cudaEventElapsedTime(&t, pool[2 * k], pool[2 * k + 1]));
    ms[(*p->ev_phase)[k]] += t;
    counts[(*p->ev_phase)[k]] += 1;
  }
  p->ev_next = 0;
  p->ev_phase->clear();
  return COV3D_OK;
}

int cov3d_gram(void *stream, int n_images, int P, int r, const void *d_q, int64_t img_stride, int64_t point_stride,
               int64_t chan_stride, const void *d_images, void *d_gram, void *d_h, float *d_yy) {
  if (n_images < 1 || P < 1 || !d_q || !d_images || !d_gram || !d_h || !d_yy) {
    set_error("invalid gram arguments");
    return COV3D_EINVAL;
  }
  return launch_gram(static_cast<cudaStream_t>(stream), n_images, P, r, d_q, img_stride, point_stride, chan_stride,
                     d_images, d_gram, d_h, d_yy);
}

int cov3d_gram_bf16(cov3d_plan *p, int n_images, int P, int r, const void *d_q, int64_t img_stride,
                    int64_t point_stride, int64_t chan_stride, const void *d_images, void *d_gram, void *d_h,
                    float *d_yy) {
  if (!valid(p) || n_images < 1 || P < 1 || !d_q || !d_images || !d_gram || !d_h || !d_yy) {
    set_error("invalid gram_bf16 arguments");
    return COV3D_EINVAL;
  }
  COV3D_TRY(launch_gram_bf16(p, p->stream, n_images, P, r, d_q, img_stride, point_stride, chan_stride, d_images, d_gram,
                             d_h, d_yy));
  return read_gram_bf16_error(p, p->stream, n_images, r);
}

int cov3d_cost_solve(void *stream, int n_images, int r, int objective, const void *d_gram, const void *d_h,
                     double noise_var, const double *d_linv, double wscale, double cscale, void *d_C, void *d_u,
                     double *d_cost_b, double *d_cost_sum, void *d_z, void *d_m, int *d_bad) {
  if (n_images < 1 || !d_gram || !d_h || !d_bad || !(noise_var > 0.0) || (objective != 0 && objective != 1) ||
      ((d_C == nullptr) != (d_u == nullptr))) {
    set_error("invalid cost_solve arguments");
    return COV3D_EINVAL;
  }
  return launch_solve(static_cast<cudaStream_t>(stream), n_images, r, objective, d_gram, d_h, noise_var, d_linv,
                      wscale, cscale, d_C, d_u, d_cost_b, d_cost_sum, d_z, d_m, d_bad);
}

int cov3d_wpass(void *stream, int n_images, int P, int r, const void *d_q, int64_t img_stride, int64_t point_stride,
                int64_t chan_stride, const void *d_images, const void *d_C, const void *d_u, void *d_w,
                int64_t w_img_stride, int64_t w_point_stride, int64_t w_chan_stride) {
  if (n_images < 1 || P < 1 || r < 1 || r > 32 || !d_q || !d_images || !d_C || !d_u || !d_w) {
    set_error("invalid wpass arguments");
    return COV3D_EINVAL;
  }
  return launch_wpass(static_cast<cudaStream_t>(stream), n_images, P, r, d_q, img_stride, point_stride, chan_stride,
                      d_images, d_C, d_u, d_w, w_img_stride, w_point_stride, w_chan_stride);
}

}  // extern "C"
