/*
 * cov3d_gb300.h -- C ABI of the GB300-native COV3D hot path.
 *
 * Plain C: every argument is a scalar, a plain struct of scalars, or a raw pointer.
 * Pointers named d_* are device pointers; the library never allocates or frees caller
 * memory.  Every entry point returns a cov3d_status code (0 on success); the text of
 * the last error of the calling thread is available from cov3d_last_error().
 *
 * Geometry and conventions (identical to the reference COV3D package):
 *  - volumes are L^3, C order, indexed [axis0][axis1][axis2] (axis 2 fastest);
 *  - images are L^2 pixels, row-major; pixel p of image b is nonuniform point b*L^2 + p;
 *  - a point's coordinate row d pairs with volume axis d (reference nufft_plan.py:326,335);
 *  - the fine (upsampled) Fourier grid has n = upsample*L points per axis.  A "centered"
 *    grid holds frequency 2*pi*(m - n/2)/n at index m (reference projection_funcs.py:148-165);
 *    an "fft-native" grid is the raw FFT output, index s = (m - n/2) mod n.
 *
 * Kernels (interpolation / spreading weights):
 *  - COV3D_KERNEL_ES:      exponential of semicircle, width w, periodic wrap (the exact
 *                          NUFFT of reference nufft_plan.py:245-392, cuFINUFFT semantics);
 *  - COV3D_KERNEL_LINEAR:  trilinear with zero padding, align_corners (grid_sample, the
 *                          reference's NufftPlanDiscretized mode="bilinear", nufft_plan.py:67-242);
 *  - COV3D_KERNEL_NEAREST: nearest neighbour with zero padding (mode="nearest").
 *
 * Threading: a plan is not thread safe; all work is enqueued on the plan's stream.
 */
#ifndef COV3D_GB300_H
#define COV3D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COV3D_ABI_VERSION 1

typedef enum {
  COV3D_OK = 0,
  COV3D_EINVAL = 1,     /* bad argument: shape, pointer, option (reference: assert / ValueError) */
  COV3D_ENOMEM = 2,     /* device allocation failed */
  COV3D_ECUDA = 3,      /* CUDA runtime error */
  COV3D_ECUFFT = 4,     /* cuFFT error */
  COV3D_ENONFINITE = 5, /* non-finite value detected in an input or a reduction */
  COV3D_EMAXITER = 6,   /* iterative solve stopped at maxiter without reaching rtol */
  COV3D_ESTATE = 7      /* call out of order (e.g. execute before setpts) */
} cov3d_status;

typedef enum { COV3D_KERNEL_ES = 0, COV3D_KERNEL_LINEAR = 1, COV3D_KERNEL_NEAREST = 2 } cov3d_kernel;

typedef enum { COV3D_GRID_CENTERED = 0, COV3D_GRID_FFT_NATIVE = 1 } cov3d_grid_order;

typedef struct cov3d_plan cov3d_plan;

/* Plan options.  Replaces the keyword arguments the reference passes to cuFINUFFT / FINUFFT
 * (nufft_plan.py:296-316: eps, gpu_method, gpu_sort) and to NufftPlanDiscretized
 * (nufft_plan.py:84-92: upsample_factor, mode). */
typedef struct {
  int kernel;        /* cov3d_kernel */
  int upsample;      /* sigma; fine grid n = upsample * L (>= 1) */
  int width;         /* ES width w in [2, 16]; 0 = from eps: ceil(-log10(eps/10)) */
  double beta;       /* ES shape; 0 = 0.97*pi*(1 - 1/(2 sigma))*w */
  int compensated;   /* 1 = TwoSum-compensated FP32 spreading in shared memory */
  int bin_size;      /* spatial bin edge in fine-grid cells (0 or 8; spreading tiles are 8^3 bins) */
  void *stream;      /* cudaStream_t for all work of this plan (NULL = legacy default) */
} cov3d_opts;

/* Layout of a complex64 fine grid in device memory.  Element (cell, channel) lives at
 * base + cell_index*cell_stride + channel*chan_stride (strides in complex elements), where
 * cell_index = (s0*n + s1)*n + s2 and s_d is the storage coordinate given by `order`. */
typedef struct {
  int order;            /* cov3d_grid_order */
  int64_t cell_stride;  /* 1 for channels-first (r, n, n, n); r for channels-last (n, n, n, r) */
  int64_t chan_stride;  /* n^3 for channels-first; 1 for channels-last */
} cov3d_grid_layout;

/* Epilogue / prologue flags of the projection operators (reference projection_funcs.py:346-399). */
#define COV3D_APPLY_NYQUIST 1 /* zero pixel row 0 and column 0 when L is even */
#define COV3D_APPLY_CTF 2     /* multiply by a per-pixel real filter (B, L*L) */
#define COV3D_APPLY_CTF_PARAMS 4 /* multiply by the CTF computed from per-image parameters: the d_ctf
                                    argument then holds (B, COV3D_CTF_NPARAMS) floats */
/* CTF parameters per image, in order: pixel size (A), defocus u (A), defocus v (A), astigmatism
 * angle (degrees), voltage (kV), spherical aberration Cs (mm), amplitude contrast, phase shift
 * (degrees) -- the columns of the reference's ctf_params (source.py:157-172), which it hands to
 * cryoDRGN's compute_ctf. */
#define COV3D_CTF_NPARAMS 8

/* ------------------------------------------------------------------ library */

int cov3d_abi_version(void);
/* Copies the calling thread's last error message (NUL terminated, truncated to len). */
int cov3d_last_error(char *buf, int len);
/* Static description of a status code. */
const char *cov3d_status_string(int status);

/* ------------------------------------------------------------------ plans
 * Mirrors the cuFINUFFT plan lifecycle the reference binds through cufinufft.Plan:
 * construction nufft_plan.py:288-316, setpts :318-336, execute :338-392, destruction on GC.
 */

/* Create a plan for L^3 volumes.  eps is the requested accuracy for the ES kernel (the
 * reference clamps it to max(eps, 10*machine eps), nufft_plan.py:286).  n_trans is the number
 * of volumes transformed together (reference batch_size = rank r); it sizes the fine-grid
 * workspace and cuFFT plan used by the type-1/type-2 and cost entry points. */
int cov3d_plan_create(int L, int n_trans, double eps, const cov3d_opts *opts, cov3d_plan **plan);
int cov3d_plan_destroy(cov3d_plan *plan);

/* Size every workspace of the plan for batches of up to max_images images of points_L^2 points
 * and nchan channels (the covariance step at rank nchan, the sort, the rotations, the in-kernel
 * CTF coefficients, the line-DFT twiddles or, where those do not apply, the cuFFT plans), so
 * that later calls within those sizes allocate nothing (cuFINUFFT sizes its plan at
 * construction, nufft_plan.py:288-316).  Without it the plan grows its buffers on first
 * use.  flags: COV3D_RESERVE_POINTS also sizes the copy of
 * explicit points (setpts), COV3D_RESERVE_GRAM_BF16 the BF16 Gram's operands,
 * COV3D_RESERVE_LS_REG the least-squares Fourier regulariser's workspace (2 nchan n^3 + n^2
 * complex) and its cuBLAS handle. */
#define COV3D_RESERVE_POINTS 1
#define COV3D_RESERVE_GRAM_BF16 2
#define COV3D_RESERVE_LS_REG 4
int cov3d_plan_reserve(cov3d_plan *plan, int64_t max_images, int points_L, int nchan, int flags);
int cov3d_plan_set_stream(cov3d_plan *plan, void *stream);
/* Reports n (fine grid edge), width and beta actually used. */
int cov3d_plan_info(const cov3d_plan *plan, int *n, int *width, double *beta);

/* Set nonuniform points.  d_pts holds n_images blocks of 3 rows of points_L^2 float32
 * frequencies in radians, i.e. the reference's (N, 3, L^2) pts_rot tensor
 * (NufftPlan.setpts nufft_plan.py:318-336; NufftPlanDiscretized.setpts :94-118).
 * img_stride / row_stride are element strides (3*L^2 and L^2 for a contiguous tensor).
 * wrap = 1 wraps to [-pi, pi) as NufftPlan.setpts does (:327).  The points are copied. */
int cov3d_setpts(cov3d_plan *plan, const float *d_pts, int64_t n_images, int points_L, int64_t img_stride,
                 int64_t row_stride, int wrap);

/* Set points from per-image rotation matrices d_rot (n_images, 3, 3) row-major float32:
 * the points of image b are flip_axis0(R_b @ pi*[x, y, 0]) wrapped to [-pi, pi), generated on
 * the fly (reference PoseModule.forward poses.py:237-269, CovarDataset.compute_pts_rot
 * dataset.py:146-164).  Nothing of size (N, 3, L^2) is materialised. */
int cov3d_setrot(cov3d_plan *plan, const float *d_rot, int64_t n_images, int points_L);

/* Interpolate nchan channels of a complex fine grid at the plan's points (type-2 spreading
 * step; the reference's grid_sample forward nufft_plan.py:120-169 for LINEAR/NEAREST).
 * Output element (point, channel) goes to d_out[point*out_point_stride + ch*out_chan_stride].
 * flags: COV3D_APPLY_NYQUIST / COV3D_APPLY_CTF with d_ctf (n_images, L^2); every output is
 * multiplied by `scale` (vol_forward's 1/L, projection_funcs.py:370). */
int cov3d_interp(cov3d_plan *plan, const void *d_grid, const cov3d_grid_layout *layout, int nchan, void *d_out,
                 int64_t out_point_stride, int64_t out_chan_stride, const float *d_ctf, int flags, float scale);

/* Exact adjoint of cov3d_interp: spread nchan channels of point values into a fine grid
 * (the reference's grid_sample backward, execute_adjoint nufft_plan.py:171-200).  The grid is
 * zeroed first unless accumulate != 0.  flags / scale as in cov3d_interp (im_backward's
 * CTF multiply, Nyquist zeroing and 1/L, projection_funcs.py:385-399). */
int cov3d_spread(cov3d_plan *plan, const void *d_values, int64_t in_point_stride, int64_t in_chan_stride,
                 int nchan, const float *d_ctf, int flags, float scale, void *d_grid, const cov3d_grid_layout *layout,
                 int accumulate);

/* Per-image adjoint without the sum over images (execute_adjoint_unaggregated,
 * nufft_plan.py:202-242): d_grids is (n_images, n, n, n) centered complex64, one channel. */
int cov3d_spread_unaggregated(cov3d_plan *plan, const void *d_values, int64_t in_point_stride, const float *d_ctf,
                              int flags, float scale, void *d_grids);

/* Type-2 NUFFT of nchan <= n_trans spatial volumes (real float32 if d_vol_real != NULL, else
 * complex64 d_vol_complex), each L^3: deapodise + zero-pad + FFT + interpolate.  Output is
 * (nchan, n_points) complex64 (NufftPlan.execute_forward, nufft_plan.py:338-364). */
int cov3d_execute_type2(cov3d_plan *plan, const float *d_vol_real, const void *d_vol_complex, int nchan, void *d_out);

/* Type-1 NUFFT (exact adjoint of type 2): (nchan, n_points) complex64 -> (nchan, L^3)
 * complex64 (NufftPlan.execute_adjoint, nufft_plan.py:366-392). */
int cov3d_execute_type1(cov3d_plan *plan, const void *d_values, int nchan, void *d_vol_out);

/* CTF images (n_images, L, L) float32 from per-image parameters (n_images, COV3D_CTF_NPARAMS):
 * the reference's ImageSource.get_ctf (source.py:157-172), which evaluates cryoDRGN's
 * compute_ctf on its frequency lattice (row index = first frequency coordinate).  The phase is
 * formed in double-float arithmetic and reduced modulo 2 pi before the float sine and cosine. */
int cov3d_ctf_images(void *stream, const float *d_params, int64_t n_images, int L, float *d_out);

/* The exact projection operator: cov3d_execute_type2 with vol_forward's epilogue fused into the
 * interpolation (Nyquist zeroing, CTF multiply or CTF from parameters, scale; the reference's
 * vol_forward on a NufftPlan, projection_funcs.py:321-370), output element (point, channel) at
 * d_out[point*out_point_stride + ch*out_chan_stride]. */
int cov3d_project(cov3d_plan *plan, const float *d_vol_real, const void *d_vol_complex, int nchan, void *d_out,
                  int64_t out_point_stride, int64_t out_chan_stride, const float *d_ctf, int flags, float scale);

/* The first half of cov3d_execute_type2 alone: deapodise + zero-pad + FFT of nchan volumes into
 * the caller's (nchan, n^3) complex64 buffer in FFT-native order (cov3d_grid_layout
 * {COV3D_GRID_FFT_NATIVE, 1, n^3}), so that a loop over batches of points with fixed volumes
 * transforms them once and calls cov3d_interp per batch; the reference's latentMAP re-executes
 * its plan on the same eigenvolumes for every batch (wiener_coords.py:131-139). */
int cov3d_fine_grid(cov3d_plan *plan, const float *d_vol_real, const void *d_vol_complex, int nchan, void *d_grid);

/* Its exact adjoint: cov3d_execute_type1 with im_backward's prologue fused into the spreading
 * (projection_funcs.py:373-399); (point, channel) input at d_values[point*in_point_stride +
 * ch*in_chan_stride], (nchan, L^3) complex64 output. */
int cov3d_backproject(cov3d_plan *plan, const void *d_values, int64_t in_point_stride, int64_t in_chan_stride,
                      int nchan, const float *d_ctf, int flags, float scale, void *d_vol_out);

/* Deapodisation factors of the plan's kernel on the L^3 voxel grid, float32 (the ES
 * analogue of VolumeBase.init_grid_correction, covar.py:45-65). */
int cov3d_grid_correction(const cov3d_plan *plan, float *d_out);

/* ------------------------------------------------------------------ covariance SGD
 * One fused evaluation of the covariance cost and its exact gradient with respect to the
 * Covar parameters (vectors (r, L^3), log_sqrt_eigenvals (r)), replacing
 * Covar.get_vectors_fourier_domain (covar.py:440-446) + cost_maximum_liklihood_fourier_domain
 * (covar_sgd.py:1350-1399) / cost_fourier_domain (:1290-1347) + autograd backward as driven
 * by CovarTrainer.run_batch (covar_sgd.py:199-229).  The gradient is the hand-written adjoint:
 * per-image r x r Gram + FP64 Hermitian solve, then backprojection of the cost's derivative
 * with respect to the projections through the exact adjoint of the interpolation.
 * Points must be set (setpts/setrot) for n_images = B images of L^2 pixels. */
typedef struct {
  int objective;            /* 0 = maximum likelihood (default objective), 1 = least squares */
  int rank;                 /* r <= n_trans */
  const float *d_vectors;   /* (r, L^3) float32 */
  const float *d_log_sqrt;  /* (r) float32 */
  const void *d_images;     /* (B, L^2) complex64, Fourier domain (centered) */
  const float *d_ctf;       /* (B, L^2) float32 or NULL */
  double noise_var;         /* Fourier-domain noise variance (dataset noise_var * L^2) */
  double reg_scale;         /* reg / N (covar_sgd.py:357) */
  const float *d_fourier_reg; /* (n^3) float32 centered, or NULL; one array per eigenvolume, (r, n^3),
                                 with fourier_reg_per_channel.  ML: reg_scale sum fr |G|^2 / (2 noise_var)
                                 (:1373-1376); LS: reg_scale |X X^H|_F^2 / L^4 with X the (n, r n^2)
                                 reshape of sqrt(fr) G, as the reference reshapes it (:1308-1313; two
                                 FP32 cuBLAS GEMMs over r n^2, workspace 2 r n^3 complex on first use) */
  int use_grid_correction;  /* divide by the kernel's deapodisation factors (init_grid_correction) */
  double *d_cost;           /* optional device scalar receiving the cost (no host sync needed) */
  int gram_bf16;            /* 1: per-image Gram contractions in BF16 on the tensor cores (FP32
                               accumulation, cov3d_gram_bf16); 0: FP32 on the CUDA cores */
  int ctf_params;           /* 1: d_ctf holds (B, COV3D_CTF_NPARAMS) CTF parameters and the CTF is
                               computed in the kernels (nothing of size (B, L^2)); 0: d_ctf is (B, L^2) */
  int fourier_reg_per_channel; /* 0: d_fourier_reg is one (n^3) array for every eigenvolume; 1: it is
                               (r, n^3), one per eigenvolume, as CovarTrainer.compute_fourier_reg_term
                               builds it (covar_sgd.py:420-430) */
} cov3d_cost_args;

/* Outputs: d_grad_vectors (r, L^3) float32, d_grad_log_sqrt (r) float32, optional
 * d_per_image_cost (B) float64 (the mean_aggregate=False data term), optional args->d_cost.
 * When `cost` (host) is not NULL the call synchronises the plan's stream and stores the
 * cost there; otherwise it returns without waiting for the GPU. */
int cov3d_covar_cost_grad(cov3d_plan *plan, const cov3d_cost_args *args, double *cost, float *d_grad_vectors,
                          float *d_grad_log_sqrt, double *d_per_image_cost);

/* ------------------------------------------------------------------ instrumentation
 * No reference counterpart beyond its time.time() epoch timing (covar_sgd.py:386-389). */

/* Number of kernels this library has launched since it was loaded (all threads). */
long long cov3d_launch_count(void);
/* Name of timing phase k (0 <= k < COV3D_NUM_PHASES), or NULL. */
const char *cov3d_phase_name(int phase);
#define COV3D_NUM_PHASES 11
/* Enable (1) or disable (0) CUDA-event timing of the plan's phases; clears recorded events. */
int cov3d_plan_timing(cov3d_plan *plan, int enable);
/* Synchronise the plan's stream, sum the recorded durations per phase into ms[n_phases] and
 * counts[n_phases] (n_phases >= COV3D_NUM_PHASES), and clear the record. */
int cov3d_plan_timing_read(cov3d_plan *plan, double *ms, int *counts, int n_phases);

/* ------------------------------------------------------------------ per-image r x r algebra
 * Plan-independent building blocks of the covariance cost, its adjoint and the latent-MAP
 * solve.  Image b's projections are r complex64 channels over P pixels: element (p, i) at
 * d_q[b*img_stride + p*point_stride + i*chan_stride]; its Fourier image is d_images[b*P + p]. */

/* gram (n_images, r, r) = conj(Q)^T Q, h (n_images, r) = conj(Q)^T y, yy (n_images) = |y|^2:
 * the batched products of compute_latentMAP_batch (wiener_coords.py:192-194) and of
 * raw_cost_fourier_domain (covar_sgd.py:1327-1328).  r <= 32. */
int cov3d_gram(void *stream, int n_images, int P, int r, const void *d_q, int64_t img_stride, int64_t point_stride,
               int64_t chan_stride, const void *d_images, void *d_gram, void *d_h, float *d_yy);

/* Per-image FP64 solve of m = gram/noise_var + Linv (Linv = d_linv (r, r) float64, or the
 * identity when NULL), b = h/noise_var, z = m^-1 b (compute_latentMAP_batch, wiener_coords.py:
 * 168-203).  objective 0 (ML): cost_b = cscale*(-Re(b^H z) + logdet m)/2 and the adjoint
 * coefficients C = wscale*(conj(m^-1) + conj(z) z^T)/(2 noise_var), u = -wscale*conj(z)/(2
 * noise_var).  objective 1 (LS): cost_b = cscale*(-2|h|^2 + ||gram||_F^2 + 2 noise_var tr gram),
 * C = wscale*(2 conj(gram) + 2 noise_var I), u = -2 wscale conj(h).  Every output pointer may
 * be NULL.  d_bad is set to 1 when some m is not positive definite. */
int cov3d_cost_solve(void *stream, int n_images, int r, int objective, const void *d_gram, const void *d_h,
                     double noise_var, const double *d_linv, double wscale, double cscale, void *d_C, void *d_u,
                     double *d_cost_b, double *d_cost_sum, void *d_z, void *d_m, int *d_bad);

/* W = C Q + u y per image and pixel (the derivative of the per-image cost with respect to
 * conj(Q)); W may alias Q when the strides are equal. */
int cov3d_wpass(void *stream, int n_images, int P, int r, const void *d_q, int64_t img_stride, int64_t point_stride,
                int64_t chan_stride, const void *d_images, const void *d_C, const void *d_u, void *d_w,
                int64_t w_img_stride, int64_t w_point_stride, int64_t w_chan_stride);

/* ------------------------------------------------------------------ mean volume and its CG solve */

/* Backproject one batch for the mean (reconstruct_mean's loop body, cov3d/mean.py:196-215):
 * d_grids (2, n, n, n) centered complex64 receives channel 0 = sum im_backward(y * phase(-offset),
 * c * ctf) (the rhs) and channel 1 = sum im_backward(c * ctf, c * ctf) / L (the kernel, lhs),
 * with Nyquist zeroing and the 1/L of im_backward.  d_images (n_images, L^2) complex64 Fourier
 * images; d_ctf (n_images, L^2), d_offsets (n_images, 2) in pixels and d_contrasts (n_images)
 * may be NULL.  The plan's points (setpts / setrot with points_L = L) give the poses; the
 * reference uses the nearest-neighbour plan at upsampling 2 (mean.py:185).  The grids are
 * zeroed first unless accumulate != 0. */
int cov3d_mean_accumulate(cov3d_plan *plan, const void *d_images, const float *d_ctf, const float *d_offsets,
                          const float *d_contrasts, void *d_grids, int accumulate);

/* regularize_lhs (cov3d/mean.py:135-142): d_reg_lhs = max(|lhs|, 1e-3 * Fourier-shell mean of
 * Re lhs), clamped at 1e-8.  d_lhs (n, n, n) centered complex64, d_reg_lhs (n, n, n) float. */
int cov3d_regularize_lhs(cov3d_plan *plan, const void *d_lhs, float *d_reg_lhs);

/* Right-hand side and starting point of correct_upsampling_padding (cov3d/mean.py:124-128,
 * 238-239): d_b = crop_L(centered_ifft3(rhs)) and d_x0 = Re crop_L(centered_ifft3(rhs / reg_lhs))
 * as complex, both (L, L, L) complex64; either output may be NULL (d_reg_lhs only needed for
 * d_x0). */
int cov3d_mean_init(cov3d_plan *plan, const void *d_rhs, const float *d_reg_lhs, void *d_b, void *d_x0);

/* No counterpart in the reference: the optimal circulant approximation (T. Chan) of the CG
 * operator A(x) = crop(ifft3(reg_lhs * fft3(pad x))) on the L^3 grid, as its Fourier symbol
 * d_symbol (L, L, L) float, centered order; the preconditioner of cov3d_cg_solve(precond=2). */
int cov3d_circulant_symbol(cov3d_plan *plan, const float *d_reg_lhs, float *d_symbol);

/* complex_conjugate_gradient on the operator of correct_upsampling_padding (cov3d/mean.py:43-132):
 * solves A x = b with A(x) = crop_L(centered_ifft3(reg_lhs * centered_fft3(pad_n(x)))), d_x
 * (L^3 complex64) holding the starting point on entry; stops when ||r|| < rtol ||b|| (FP64
 * inner products) or after maxiter iterations.  precond: 0 none (the reference), 1 the
 * Fourier-diagonal 1 / reg_lhs on the fine grid, 2 division by d_symbol (L^3 float, centered)
 * in the L^3 Fourier domain.  *iters receives the loop index at which it stopped (the
 * reference's num_iter), *relres ||r|| / ||b||; d_history (maxiter + 1 doubles, may be NULL)
 * the relative residual before the loop and after each iteration.  Returns COV3D_EMAXITER
 * (with d_x holding the last iterate) when the tolerance was not reached.  The iterations run as
 * replays of a CUDA graph of 8 iterations that the call captures on its own side stream and
 * launches on the plan's stream; the host reads the state between replays, so the call
 * synchronises the plan's stream and cannot itself run inside a caller's stream capture. */
int cov3d_cg_solve(cov3d_plan *plan, const float *d_reg_lhs, const void *d_b, void *d_x, double rtol, int maxiter,
                   int precond, const float *d_symbol, int *iters, double *relres, double *d_history);

/* No counterpart in the reference (its contraction is a batched complex GEMM at the input
 * precision): the outputs of cov3d_gram with BF16 inputs and FP32 accumulation on the tensor
 * cores (tcgen05).  Q and y are rounded to BF16 (relative error 2^-9 per element); the plan
 * provides the workspace (n_images * (2r+2) * P BF16 values).  Requires 2(r+1) <= 128. */
int cov3d_gram_bf16(cov3d_plan *plan, int n_images, int P, int r, const void *d_q, int64_t img_stride,
                    int64_t point_stride, int64_t chan_stride, const void *d_images, void *d_gram, void *d_h,
                    float *d_yy);

/* ------------------------------------------------------------------ learned CG preconditioner
 * No counterpart in the reference.  Layers of the small 3D U-Net that predicts a correction of
 * the circulant CG preconditioner from the kernel density, forward and backward, so that the
 * network is trained and run by this library.  Tensors are (N, C, D, H, W) float32, contiguous;
 * weights (Cout, Cin, k, k, k) with k = ksize in {1, 3}; stride 1, zero padding k / 2.  All
 * calls are asynchronous on `stream`. */

/* y = conv(x, w) + bias (bias may be NULL), ReLU applied when relu != 0. */
int cov3d_conv3d_forward(void *stream, const float *d_x, int N, int Cin, int D, int H, int W, const float *d_w,
                         const float *d_bias, int Cout, int ksize, int relu, float *d_y);

/* gx = gradient of sum(gy * conv(x, w)) with respect to x; d_wt_scratch holds Cout * Cin * k^3
 * floats (the flipped, channel-transposed kernel). */
int cov3d_conv3d_backward_data(void *stream, const float *d_gy, int N, int Cout, int D, int H, int W,
                               const float *d_w, int Cin, int ksize, float *d_wt_scratch, float *d_gx);

/* gw (Cout, Cin, k^3) and gb (Cout, may be NULL) = gradients of sum(gy * (conv(x, w) + b)),
 * overwritten. */
int cov3d_conv3d_backward_weight(void *stream, const float *d_x, const float *d_gy, int N, int Cin, int Cout, int D,
                                 int H, int W, int ksize, float *d_gw, float *d_gb);

/* gx = gy where y > 0, else 0 (may run in place on gy). */
int cov3d_relu_backward(void *stream, const float *d_y, const float *d_gy, int64_t count, float *d_gx);

/* 2x average pooling: direction 0 forward (NC, D, H, W) -> (NC, D/2, H/2, W/2), 1 its adjoint
 * (d_in the gradient of the pooled volume, d_out (NC, D, H, W)). */
int cov3d_avgpool2(void *stream, const float *d_in, int64_t NC, int D, int H, int W, int direction, float *d_out);

/* 2x nearest upsampling: direction 0 forward (NC, d, h, w) -> (NC, 2d, 2h, 2w), 1 its adjoint
 * (sum over the 8 children; d_in (NC, 2d, 2h, 2w), d_out (NC, d, h, w)). */
int cov3d_upsample2(void *stream, const float *d_in, int64_t NC, int d, int h, int w, int direction, float *d_out);

/* Cubic resampling: direction 0 trilinear (align_corners = False) (NC, d^3) -> (NC, D^3);
 * 1 its adjoint (NC, D^3) -> (NC, d^3); 2 block mean (NC, D^3) -> (NC, d^3), D a multiple of d. */
int cov3d_resample3d(void *stream, const float *d_in, int64_t NC, int d, int D, int direction, float *d_out);

/* ------------------------------------------------------------------ allocation-free variant
 * No counterpart in the reference.  Same result as cov3d_gram followed by cov3d_cost_solve
 * (objective 0, no adjoint coefficients, no costs) for callers that cannot let a library
 * allocate device memory: their own pool owns the GPU, or cudaMalloc's device-wide
 * synchronisation is not acceptable on their call path.  The intermediates live in a 4 MiB
 * file-scope device array that each GPU loading the library keeps until exit; the call
 * allocates nothing (no cudaMalloc / cudaFree / allocating library routine).  Two caveats:
 * the first launch of the solve kernel at a given rank may make the driver enlarge its
 * per-thread local-memory reservation (the kernel's r x r working arrays), so warm up once
 * at the largest rank you will use; and the array's device address is looked up once per
 * device and kept, which assumes the runtime's primary context on that device for the life
 * of the process (after cudaDeviceReset, or with another context current, the kept address
 * is stale: do not call this entry point then).
 * Limit: n_images * (8 r^2 + 8 r + 4) bytes plus alignment must fit in 4 MiB (e.g. 4,700
 * images at r = 10); larger requests return COV3D_EINVAL with the limit in the message.
 * The first call on each device looks up the array's device address (cudaGetSymbolAddress)
 * with that device current; make that first call before any stream capture.  All calls share
 * the one array and it keeps the last call's contents: calls that overlap on the GPU (other
 * streams, other host threads) race, so serialise them.  d_z (n_images, r) complex64 and/or
 * d_m (n_images, r, r) complex64 receive the results; d_bad (optional, device int) receives 1
 * when some m is not positive definite, else 0. */
int cov3d_latent_map_noalloc(void *stream, int n_images, int P, int r, const void *d_q, int64_t img_stride,
                             int64_t point_stride, int64_t chan_stride, const void *d_images, double noise_var,
                             const double *d_linv, void *d_z, void *d_m, int *d_bad);

#ifdef __cplusplus
}
#endif

#endif /* COV3D_GB300_H */
