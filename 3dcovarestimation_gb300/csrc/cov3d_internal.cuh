// Internal declarations shared by the translation units of libcov3d_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <map>
#include <vector>
#include <string>

#include "cov3d_gb300.h"

namespace cov3d {

constexpr float kPiF = 3.14159265358979323846f;
constexpr double kPi = 3.14159265358979323846;

// ----------------------------------------------------------------------------- errors

void set_error(const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
int check_cufft(cufftResult r, const char *what);

#define COV3D_TRY(expr)                 \
  do {                                  \
    int _st = (expr);                   \
    if (_st != COV3D_OK) return _st;    \
  } while (0)

#define COV3D_CUDA(expr) COV3D_TRY(::cov3d::check_cuda((expr), #expr))
// Counts one kernel launch of this library and checks the launch error.
int launched(const char *name);
// adds n kernel launches to the library's count (each replay of a captured CUDA graph)
void count_launches(long long n);
#define COV3D_LAUNCHED(name) COV3D_TRY(::cov3d::launched(name))

// ----------------------------------------------------------------------------- geometry

// How a nonuniform point's fine-grid fractional index is obtained.
enum PointKind { kPointsNone = 0, kPointsExplicit = 1, kPointsRotations = 2 };
// How a frequency maps to a fractional centered-grid index.
enum Mapping { kMapES = 0, kMapGridSample = 1 };

struct PointGeom {
  int kind;           // PointKind
  const float *pts;   // explicit: contiguous (N, 3, P) frequencies
  const float *rot;   // rotations: (N, 9) row-major
  int Lp;             // image edge (points per image = Lp*Lp)
  int P;              // Lp*Lp
  int n;              // fine grid edge
  int mapping;        // Mapping
  int wrap;           // wrap explicit points to [-pi, pi)
  float s_es;         // n / (2 pi)
  float half_n;       // n / 2 (integer division) as float
  float gs_scale;     // float32((n/(n-1))/pi)
  float gs_off;       // float32(1/(n-1)) for even n, else 0
  float plane_half;   // Lp / 2 (may be .5) as float
};

// Interpolation kernel descriptor.
struct KernelSpec {
  int type;     // cov3d_kernel
  int width;    // taps per axis
  float beta;   // ES shape
  int periodic; // 1 = wrap cell indices mod n, 0 = zero padding
};

// Bin grid used for point sorting / spreading tiles.
struct Bins {
  int bs[3];   // bin edge per axis
  int nb[3];   // bins per axis
  int64_t nbins;
};

// ----------------------------------------------------------------------------- plan
}  // namespace cov3d

namespace cov3d {
// Grow-only device buffer owned by a plan.
struct DevBuf {
  void *ptr = nullptr;
  int64_t cap = 0;  // bytes
  template <typename T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};
int grow(DevBuf &b, int64_t bytes);
void release(DevBuf &b);
}  // namespace cov3d

struct cov3d_plan {
  int L = 0, n = 0, upsample = 2, kernel = COV3D_KERNEL_ES, width = 6;
  double beta = 0.0;
  int compensated = 1;
  int n_trans = 1;
  cudaStream_t stream = nullptr;
  int device = 0;

  cov3d::DevBuf gc1d;          // float deapodisation factors per axis (L)
  double *h_gc1d = nullptr;    // host copy (double)

  // points
  int point_kind = cov3d::kPointsNone;
  int wrap = 0;
  int64_t n_images = 0;
  int points_L = 0;
  int64_t n_points = 0;
  cov3d::DevBuf pts;           // explicit points copy (N, 3, P) float
  cov3d::DevBuf rot;           // rotations (N, 9) float

  // sort / subproblems
  cov3d::Bins bins{};
  int max_sub = 288;
  cov3d::DevBuf bin_count;     // int (nbins + 1), last = dead points
  cov3d::DevBuf bin_off;       // int (nbins + 2)
  cov3d::DevBuf sub_off;       // int (nbins + 1)
  cov3d::DevBuf pt_bin, pt_rank;              // int (M)
  cov3d::DevBuf sorted;        // SortedPoint (M), bin-sorted order
  cov3d::DevBuf sub_bin, sub_first, sub_count;  // int (max subproblems)
  cov3d::DevBuf nsub;          // int scalar

  // workspaces
  cov3d::DevBuf fine, fine2;   // complex fine grids (n^3 * channels)
  cov3d::DevBuf q;             // per-point values (points * r) complex
  cov3d::DevBuf small;         // per-image small matrices
  cov3d::DevBuf acc;           // double accumulators
  cov3d::DevBuf cgw;           // mean / CG workspace (state, vectors, shell sums)
  cov3d::DevBuf xbf, gsum;     // BF16 Gram operands and real Gram sums
  cov3d::DevBuf ctfc;          // per-image CTF coefficients (CtfCoef) from CTF parameters
  cov3d::DevBuf lsw;           // least-squares regulariser: X, K X (r n^3 complex each) and K (n^2)
  void *blas = nullptr;        // cuBLAS handle of the least-squares regulariser (created on first use)
  cov3d::DevBuf fftw;          // twiddles exp(-2 pi i j / fftw_n) of the fused axis-0 CG transform
  int fftw_n = 0;
  double *h_acc = nullptr;     // pinned host mirror of acc (64 doubles)
  std::map<int, cufftHandle> *ffts = nullptr;  // cuFFT plans by channel count

  // phase timing (CUDA events on the plan's stream), see cov3d_plan_timing
  int timing = 0;
  std::vector<cudaEvent_t> *ev_pool = nullptr;
  size_t ev_next = 0;
  std::vector<int> *ev_phase = nullptr;  // phase of each recorded (start, stop) pair
};

namespace cov3d {

// ----------------------------------------------------------------------------- phases
enum Phase {
  kPhaseSort = 0, kPhasePack, kPhaseFftFwd, kPhaseInterp, kPhaseGram, kPhaseSolve, kPhaseWpass, kPhaseSpread,
  kPhaseReg, kPhaseFftInv, kPhaseUnpack, kNumPhases
};

// Records CUDA events around a phase when the plan's timing is enabled.
class PhaseScope {
 public:
  PhaseScope(cov3d_plan *p, int phase);
  ~PhaseScope();
 private:
  cov3d_plan *p_;
  cudaEvent_t stop_ = nullptr;
};

// ----------------------------------------------------------------------------- helpers

PointGeom make_geom(const cov3d_plan *p);
KernelSpec make_kernel(const cov3d_plan *p);
int get_fft(cov3d_plan *p, int nchan, cufftHandle *out);
int get_fft_planes(cov3d_plan *p, cufftHandle *out);
int get_fft_axis0(cov3d_plan *p, cufftHandle *out);
int fft2(cufftHandle h, const float2 *in, float2 *out, int dir);

// line_fft.cu: hand-written line DFTs of the fine grid.  `stop` points at a done flag (kernels
// return once it is nonzero) or is null.
bool axis0_fused_size(int n);
bool line_transforms_apply(const cov3d_plan *p);
int ensure_twiddles(cov3d_plan *p, int n);
int launch_axis0_diag(cov3d_plan *p, float2 *g, const float *diag, int L, int n, int divide, float scale,
                      const int *stop);
int cg_operator_lines(cov3d_plan *p, const float2 *in, float2 *fine, float2 *out, const float2 *dotp,
                      const float *diag, int divide, const int *stop, const int *stop_last, double *dot);
int step_forward_lines(cov3d_plan *p, const float *vec, const float *logs, const float *gc, int r, float2 *stage,
                       float2 *grid, const float *fr, int64_t fr_stride, double coef, double *cost);
int step_inverse_lines(cov3d_plan *p, float2 *grad_grid, const float *vec, const float *logs, const float *gc, int r,
                       float *gvec, double *glog);
inline bool prunable(const cov3d_plan *p) { return p->L % 2 == 0 && p->n >= p->L + 2; }

// points_sort.cu
int sort_points(cov3d_plan *p);
int reserve_sort(cov3d_plan *p, int64_t M);
// gram_tc.cu: the BF16 Gram's operand and sum buffers for B images of P pixels at rank r
int reserve_gram_bf16(cov3d_plan *p, int B, int P, int r);

// interp.cu
struct GridArgs {
  const void *grid;
  int64_t cell_stride, chan_stride;
  int shift;  // storage = (centered + shift) mod n
};
// Per-image coefficients of the CTF phase, prepared from the CTF parameters by
// prepare_ctf_coef (grid_ops.cu) and evaluated per pixel by ctf_eval (cov3d_device.cuh):
// gamma(ka, kb) = c0 K + c1 D + c2 X + d K^2 - ps at the pixel offsets (ka, kb) from the image
// centre (row, column), K = ka^2 + kb^2, D = ka^2 - kb^2, X = 2 ka kb; c0..c2 as float pairs
// (hi + lo) whose sum carries the double-precision coefficient.
struct CtfCoef {
  float c0h, c0l, c1h, c1l, c2h, c2l;
  float d, ps, sw, w;  // K^2 coefficient, phase shift (rad), sqrt(1 - w^2), amplitude contrast
  float pad0, pad1;
};

struct EpilogueArgs {
  const float *ctf;  // (n_images, P) or null
  int nyquist;       // zero row/col 0 when Lp even
  float scale;
  const CtfCoef *ctfc = nullptr;  // per-image CTF coefficients (used when ctf is null), or null
};
// Coefficients of n_images CTFs from their parameters (n_images, COV3D_CTF_NPARAMS) into the
// plan's workspace; *out receives the device pointer.
int prepare_ctf_coef(cov3d_plan *p, const float *params, int64_t n_images, int L, const CtfCoef **out);
int launch_interp(cov3d_plan *p, const GridArgs &g, int nchan, void *out, int64_t out_ps, int64_t out_cs,
                  const EpilogueArgs &e);

// spread.cu
int launch_spread(cov3d_plan *p, const void *values, int64_t in_ps, int64_t in_cs, int nchan, const EpilogueArgs &e,
                  void *grid, int64_t cell_stride, int64_t chan_stride, int shift);
int launch_spread_unaggregated(cov3d_plan *p, const void *values, int64_t in_ps, const EpilogueArgs &e,
                               void *grids);

// grid_ops.cu
int launch_pack(cov3d_plan *p, const float *vol_real, const void *vol_cplx, const float *log_scale, int use_gc,
                int nchan, void *fine);
int launch_unpack_complex(cov3d_plan *p, const void *fine, int nchan, int use_gc, void *out);
int launch_unpack_grad(cov3d_plan *p, const void *fine, const float *vectors, const float *log_scale, int use_gc,
                       int nchan, float *grad_vec, double *grad_log_acc);
int launch_ml_reg(cov3d_plan *p, const void *grid, void *ggrid, const float *fr, int64_t fr_stride, int nchan, double coef,
                  double *cost_acc, int init);
int launch_gc_volume(const cov3d_plan *p, float *out);
int launch_zero(cov3d_plan *p, void *ptr, int64_t bytes);
int launch_ls_reg(cov3d_plan *p, const void *grid, void *ggrid, const float *fr, int64_t fr_stride, int r, double s,
                  double *cost_acc);
void release_blas(cov3d_plan *p);
int reserve_ls_reg(cov3d_plan *p, int r);

// gram_solve.cu
int launch_gram_bf16(cov3d_plan *p, cudaStream_t st, int B, int P, int r, const void *q, int64_t is, int64_t ps,
                     int64_t cs, const void *images, void *gram, void *h, float *yy);
int read_gram_bf16_error(cov3d_plan *p, cudaStream_t st, int B, int r);
int launch_gram(cudaStream_t st, int B, int P, int r, const void *q, int64_t is, int64_t ps, int64_t cs,
                const void *images, void *gram, void *h, float *yy);
int launch_wpass(cudaStream_t st, int B, int P, int r, const void *q, int64_t is, int64_t ps, int64_t cs,
                 const void *images, const void *C, const void *u, void *w, int64_t wis, int64_t wps, int64_t wcs);
int launch_solve(cudaStream_t st, int B, int r, int objective, const void *gram, const void *h, double s2,
                 const double *linv, double wscale, double cscale, void *C, void *u, double *cost_b, double *cost_sum,
                 void *z, void *m, int *bad);
int covar_cost_grad(cov3d_plan *p, const cov3d_cost_args *a, double *h_cost, double *d_cost, float *d_grad_vectors,
                    float *d_grad_log_sqrt, double *d_per_image_cost);

}  // namespace cov3d
