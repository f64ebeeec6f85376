// Fine-grid packing around cuFFT: deapodisation + zero padding + centering as one pass
// before the forward FFT, and crop + deapodisation after the inverse (reference
// Covar.get_vectors_fourier_domain covar.py:440-446 / pad_tensor + centered_fft3
// projection_funcs.py:11-165, whose fftshift/ifftshift/pad copies are folded into index maps).
//
// Storage order of the fine grid is the raw FFT order: voxel offset k = j - L/2 sits at
// storage index k mod n, so no shift pass is needed on either side of the FFT.  Fine grids are
// channels-first (nchan planes of n^3 cells) so cuFFT runs unit-stride batched transforms.
#include "cov3d_device.cuh"

namespace cov3d {

namespace {

// storage coordinate -> voxel index j in [0, L), or -1 when the cell is zero padding
__device__ __forceinline__ int storage_to_voxel(int s, int L, int n) {
  const int half = L / 2;
  if (s < L - half) return s + half;
  if (s >= n - half) return s - n + half;
  return -1;
}

__device__ __forceinline__ int voxel_to_storage(int j, int L, int n) {
  const int k = j - L / 2;
  return k < 0 ? k + n : k;
}

__global__ void pack_kernel(const float *__restrict__ vr, const float2 *__restrict__ vc,
                            const float *__restrict__ logs, const float *__restrict__ gc, int nchan, int L, int n,
                            float2 *__restrict__ fine) {
  const int64_t n3 = (int64_t)n * n * n;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= n3) return;
  const int s2 = (int)(cell % n);
  const int s1 = (int)((cell / n) % n);
  const int s0 = (int)(cell / ((int64_t)n * n));
  const int j0 = storage_to_voxel(s0, L, n), j1 = storage_to_voxel(s1, L, n), j2 = storage_to_voxel(s2, L, n);
  float2 *out = fine + cell;
  if (j0 < 0 || j1 < 0 || j2 < 0) {
    for (int c = 0; c < nchan; ++c) out[c * n3] = make_float2(0.f, 0.f);
    return;
  }
  const int64_t L3 = (int64_t)L * L * L;
  const int64_t v = ((int64_t)j0 * L + j1) * L + j2;
  const float g = gc ? 1.0f / (__ldg(gc + j0) * __ldg(gc + j1) * __ldg(gc + j2)) : 1.0f;
  for (int c = 0; c < nchan; ++c) {
    const float sc = logs ? g * expf(__ldg(logs + c)) : g;
    float2 x = vr ? make_float2(__ldg(vr + c * L3 + v), 0.f) : vc[c * L3 + v];
    out[c * n3] = make_float2(x.x * sc, x.y * sc);
  }
}

__global__ void unpack_complex_kernel(const float2 *__restrict__ fine, const float *__restrict__ gc, int nchan, int L,
                                      int n, float2 *__restrict__ out) {
  const int64_t L3 = (int64_t)L * L * L;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= L3) return;
  const int j2 = (int)(v % L), j1 = (int)((v / L) % L), j0 = (int)(v / ((int64_t)L * L));
  const int64_t cell =
      ((int64_t)voxel_to_storage(j0, L, n) * n + voxel_to_storage(j1, L, n)) * n + voxel_to_storage(j2, L, n);
  const float g = gc ? 1.0f / (__ldg(gc + j0) * __ldg(gc + j1) * __ldg(gc + j2)) : 1.0f;
  for (int c = 0; c < nchan; ++c) {
    const float2 x = fine[(int64_t)c * n * n * n + cell];
    out[c * L3 + v] = make_float2(x.x * g, x.y * g);
  }
}

// Gradient w.r.t. the Covar parameters from the inverse-FFT'd fine-grid gradient:
// dcost/dV = 2 Re(.) / gc on the cropped voxels; d/dvectors = dV * exp(s);
// d/dlog_sqrt = sum dV * V (accumulated in double).
__global__ void unpack_grad_kernel(const float2 *__restrict__ fine, const float *__restrict__ vectors,
                                   const float *__restrict__ logs, const float *__restrict__ gc, int nchan, int L,
                                   int n, float *__restrict__ gvec, double *__restrict__ glog) {
  // capped grid walking voxel rows; one FP64 atomic per block and channel for d/dlog_sqrt
  const int64_t L3 = (int64_t)L * L * L;
  const int64_t n3 = (int64_t)n * n * n;
  for (int c = 0; c < nchan; ++c) {
    const float e = expf(__ldg(logs + c));
    double part = 0.0;
    for (int64_t row = blockIdx.x; row < (int64_t)L * L; row += gridDim.x) {
      const int j0 = (int)(row / L), j1 = (int)(row - (int64_t)j0 * L);
      const float2 *src = fine + (int64_t)c * n3 + ((int64_t)voxel_to_storage(j0, L, n) * n + voxel_to_storage(j1, L, n)) * n;
      const float g01 = gc ? 1.0f / (__ldg(gc + j0) * __ldg(gc + j1)) : 1.0f;
      for (int j2 = threadIdx.x; j2 < L; j2 += blockDim.x) {
        const float g = gc ? g01 / __ldg(gc + j2) : 1.0f;
        const int64_t v = row * L + j2;
        const float dV = 2.0f * src[voxel_to_storage(j2, L, n)].x * g;
        const float vec = __ldg(vectors + c * L3 + v);
        gvec[c * L3 + v] = dV * e;
        part += (double)(dV * (vec * e));
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    __shared__ double wp[32];
    if ((threadIdx.x & 31) == 0) wp[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += wp[i];
      if (t != 0.0) atomicAdd(glog + c, t);
    }
    __syncthreads();
  }
}

// ML Fourier regulariser reg_scale * sum |G|^2 fr / (2 s2) (covar_sgd.py:1373-1376): adds its
// conjugate-Wirtinger derivative coef * fr * G to the fine-grid gradient (or, with `init`,
// writes it there, so the grid needs no zeroing before the spread), accumulates its value.
__global__ void ml_reg_kernel(const float2 *__restrict__ grid, float2 *__restrict__ gg, const float *__restrict__ fr,
                              int64_t frs, int nchan, int n, double coef, double *__restrict__ cost, int init) {
  // capped grid walking whole rows (no per-element division); the channel sum of one cell is
  // FP32, the running sum over cells FP64, one FP64 atomic per block
  const int64_t n3 = (int64_t)n * n * n;
  const int half = n / 2;
  const float cfs = (float)coef;
  // 16-byte accesses need an even row length and 16-byte aligned grids
  // (with one regulariser per channel, frs != 0, the scalar path below reads each channel's)
  const bool vec = frs == 0 && (n & 1) == 0 &&
                   ((reinterpret_cast<uintptr_t>(grid) | reinterpret_cast<uintptr_t>(gg)) & 15) == 0;
  double part = 0.0;
  for (int64_t row = blockIdx.x; row < (int64_t)n * n; row += gridDim.x) {
    int s0 = (int)(row / n), s1 = (int)(row - (int64_t)s0 * n);
    s0 = s0 + half >= n ? s0 + half - n : s0 + half;
    s1 = s1 + half >= n ? s1 + half - n : s1 + half;
    const float *frow = fr + ((int64_t)s0 * n + s1) * n;
    if (vec) {  // two cells per thread, 16-byte loads, four channels' loads in flight
      for (int s2 = 2 * threadIdx.x; s2 < n; s2 += 2 * blockDim.x) {
        const int c2a = s2 + half >= n ? s2 + half - n : s2 + half;
        const int c2b = s2 + 1 + half >= n ? s2 + 1 + half - n : s2 + 1 + half;
        const float wa = __ldg(frow + c2a), wb = __ldg(frow + c2b);
        const float cfa = cfs * wa, cfb = cfs * wb;
        const int64_t cell = row * n + s2;
        const float4 *src = reinterpret_cast<const float4 *>(grid + cell);
        float4 *dst = reinterpret_cast<float4 *>(gg + cell);
        const int64_t cstep = n3 / 2;  // one channel, in float4
        float pa = 0.0f, pb = 0.0f;
        int c = 0;
        for (; c + 4 <= nchan; c += 4) {
          float4 x[4], y[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) x[u] = __ldg(src + (c + u) * cstep);
#pragma unroll
          for (int u = 0; u < 4; ++u) y[u] = init ? make_float4(0.f, 0.f, 0.f, 0.f) : dst[(c + u) * cstep];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            dst[(c + u) * cstep] = make_float4(fmaf(cfa, x[u].x, y[u].x), fmaf(cfa, x[u].y, y[u].y),
                                               fmaf(cfb, x[u].z, y[u].z), fmaf(cfb, x[u].w, y[u].w));
            pa = fmaf(x[u].x, x[u].x, fmaf(x[u].y, x[u].y, pa));
            pb = fmaf(x[u].z, x[u].z, fmaf(x[u].w, x[u].w, pb));
          }
        }
        for (; c < nchan; ++c) {
          const float4 x = __ldg(src + c * cstep);
          const float4 y = init ? make_float4(0.f, 0.f, 0.f, 0.f) : dst[c * cstep];
          dst[c * cstep] = make_float4(fmaf(cfa, x.x, y.x), fmaf(cfa, x.y, y.y), fmaf(cfb, x.z, y.z), fmaf(cfb, x.w, y.w));
          pa = fmaf(x.x, x.x, fmaf(x.y, x.y, pa));
          pb = fmaf(x.z, x.z, fmaf(x.w, x.w, pb));
        }
        part += (double)(wa * pa) + (double)(wb * pb);
      }
      continue;
    }
    for (int s2 = threadIdx.x; s2 < n; s2 += blockDim.x) {
      const int c2 = s2 + half >= n ? s2 + half - n : s2 + half;
      const int64_t cell = row * n + s2;
      float p32 = 0.0f;
      for (int c = 0; c < nchan; ++c) {
        const float w = __ldg(frow + c * frs + c2);
        const float cf = cfs * w;
        const float2 x = grid[c * n3 + cell];
        float2 y = init ? make_float2(0.f, 0.f) : gg[c * n3 + cell];
        y.x = fmaf(cf, x.x, y.x);
        y.y = fmaf(cf, x.y, y.y);
        gg[c * n3 + cell] = y;
        p32 = fmaf(w, fmaf(x.x, x.x, x.y * x.y), p32);
      }
      part += (double)p32;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  __shared__ double warp_part[32];
  if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += warp_part[i];
    if (s != 0.0) atomicAdd(cost, s * coef);
  }
}

__global__ void gc_volume_kernel(const float *__restrict__ gc, int L, float *__restrict__ out) {
  const int64_t L3 = (int64_t)L * L * L;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= L3) return;
  const int j2 = (int)(v % L), j1 = (int)((v / L) % L), j0 = (int)(v / ((int64_t)L * L));
  out[v] = gc[j0] * gc[j1] * gc[j2];
}

inline unsigned nblocks(int64_t n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

int launch_pack(cov3d_plan *p, const float *vol_real, const void *vol_cplx, const float *log_scale, int use_gc,
                int nchan, void *fine) {
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  pack_kernel<<<nblocks(n3), 256, 0, p->stream>>>(vol_real, static_cast<const float2 *>(vol_cplx), log_scale,
                                                  use_gc ? p->gc1d.as<float>() : nullptr, nchan, p->L, p->n,
                                                  static_cast<float2 *>(fine));
  return launched("pack_kernel");
}

int launch_unpack_complex(cov3d_plan *p, const void *fine, int nchan, int use_gc, void *out) {
  const int64_t L3 = (int64_t)p->L * p->L * p->L;
  unpack_complex_kernel<<<nblocks(L3), 256, 0, p->stream>>>(static_cast<const float2 *>(fine),
                                                            use_gc ? p->gc1d.as<float>() : nullptr, nchan, p->L,
                                                            p->n, static_cast<float2 *>(out));
  return launched("unpack_complex_kernel");
}

int launch_unpack_grad(cov3d_plan *p, const void *fine, const float *vectors, const float *log_scale, int use_gc,
                       int nchan, float *grad_vec, double *grad_log_acc) {
  const int64_t L3 = (int64_t)p->L * p->L * p->L;
  const int64_t rows = (int64_t)p->L * p->L;
  (void)L3;
  const int threads = p->L >= 256 ? 256 : (p->L + 31) / 32 * 32;  // one voxel row per pass
  unpack_grad_kernel<<<(unsigned)(rows < 2432 ? rows : 2432), threads, 0, p->stream>>>(static_cast<const float2 *>(fine), vectors, log_scale,
                                                         use_gc ? p->gc1d.as<float>() : nullptr, nchan, p->L, p->n,
                                                         grad_vec, grad_log_acc);
  return launched("unpack_grad_kernel");
}

int launch_ml_reg(cov3d_plan *p, const void *grid, void *ggrid, const float *fr, int64_t fr_stride, int nchan,
                  double coef, double *cost_acc, int init) {
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  const int64_t rows = (int64_t)p->n * p->n;
  const unsigned blocks = (unsigned)(rows < 2432 ? rows : 2432);  // 16 blocks of 4 warps per SM
  (void)n3;
  ml_reg_kernel<<<blocks, 128, 0, p->stream>>>(static_cast<const float2 *>(grid), static_cast<float2 *>(ggrid), fr,
                                               fr_stride, nchan, p->n, coef, cost_acc, init);
  return launched("ml_reg_kernel");
}

int launch_gc_volume(const cov3d_plan *p, float *out) {
  const int64_t L3 = (int64_t)p->L * p->L * p->L;
  gc_volume_kernel<<<nblocks(L3), 256, 0, p->stream>>>(p->gc1d.as<float>(), p->L, out);
  return launched("gc_volume_kernel");
}

int launch_zero(cov3d_plan *p, void *ptr, int64_t bytes) {
  return check_cuda(cudaMemsetAsync(ptr, 0, (size_t)bytes, p->stream), "cudaMemsetAsync");
}

// Pruned transforms (even L): the zero-padded volume has L nonzero planes of n (the first and
// last L/2 in FFT-native order) and only those planes of an inverse transform are cropped, so a
// 3D transform is a batched 2D FFT over the L/2 support planes of each half (key -2) and a 1D FFT
// along axis 0 over all n^2 lines (key -3).
int get_fft_planes(cov3d_plan *p, cufftHandle *out) {
  auto it = p->ffts->find(-2);
  if (it == p->ffts->end()) {
    cufftHandle h;
    int dims[2] = {p->n, p->n};
    COV3D_TRY(check_cufft(cufftPlanMany(&h, 2, dims, nullptr, 1, p->n * p->n, nullptr, 1, p->n * p->n, CUFFT_C2C,
                                        p->L / 2),
                          "cufftPlanMany(planes)"));
    it = p->ffts->emplace(-2, h).first;
  }
  *out = it->second;
  return check_cufft(cufftSetStream(it->second, p->stream), "cufftSetStream");
}

int get_fft_axis0(cov3d_plan *p, cufftHandle *out) {
  auto it = p->ffts->find(-3);
  if (it == p->ffts->end()) {
    cufftHandle h;
    int dims[1] = {p->n};
    const int nn = p->n * p->n;
    COV3D_TRY(check_cufft(cufftPlanMany(&h, 1, dims, dims, nn, 1, dims, nn, 1, CUFFT_C2C, nn), "cufftPlanMany(axis0)"));
    it = p->ffts->emplace(-3, h).first;
  }
  *out = it->second;
  return check_cufft(cufftSetStream(it->second, p->stream), "cufftSetStream");
}

int fft2(cufftHandle h, const float2 *in, float2 *out, int dir) {
  return check_cufft(cufftExecC2C(h, reinterpret_cast<cufftComplex *>(const_cast<float2 *>(in)),
                                  reinterpret_cast<cufftComplex *>(out), dir),
                     "cufftExecC2C");
}

int get_fft(cov3d_plan *p, int nchan, cufftHandle *out) {
  auto it = p->ffts->find(nchan);
  if (it != p->ffts->end()) {
    *out = it->second;
    return check_cufft(cufftSetStream(it->second, p->stream), "cufftSetStream");
  }
  cufftHandle h;
  int dims[3] = {p->n, p->n, p->n};
  const int n3 = p->n * p->n * p->n;
  // channels-first: nchan contiguous n^3 transforms (unit stride, distance n^3)
  COV3D_TRY(check_cufft(cufftPlanMany(&h, 3, dims, dims, 1, n3, dims, 1, n3, CUFFT_C2C, nchan), "cufftPlanMany"));
  (*p->ffts)[nchan] = h;
  *out = h;
  return check_cufft(cufftSetStream(h, p->stream), "cufftSetStream");
}

}  // namespace cov3d

// ----------------------------------------------------------------------------- CTF from parameters
namespace cov3d {
namespace {

// CtfCoef of one image from its parameters q[0..7] = pixel size (A), defocus u and v (A),
// astigmatism angle (degrees), voltage (kV), spherical aberration (mm), amplitude contrast,
// phase shift (degrees): the CTF sqrt(1 - w^2) sin(gamma) - w cos(gamma) with
// gamma = 2 pi (-df lambda s^2 / 2 + Cs lambda^3 s^4 / 4) - phase shift, the defocus along the
// frequency's direction df = (dfu + dfv + (dfu - dfv) cos(2 (angle - astigmatism angle))) / 2 and
// the relativistic electron wavelength lambda = 12.2639 / sqrt(V + 0.97845e-6 V^2) (V in volts):
// the standard weak-phase CTF in the form cryoDRGN's compute_ctf evaluates for the reference
// (source.py:157-172), frequency s at pixel (row a, column b) = (a - L/2, b - L/2) / (L * pixel).
// In double precision; the angle-dependent defocus is expanded with cos 2(t - d) = cos 2t cos 2d +
// sin 2t sin 2d, cos 2t = (x^2 - y^2) / K, sin 2t = 2 x y / K, so no per-pixel angle is needed.
__device__ CtfCoef make_ctf_coef(const float *q, int L) {
  const double pi = 3.14159265358979323846;
  const double apix = q[0], dfu = q[1], dfv = q[2], ang = (double)q[3] * pi / 180.0;
  const double volt = (double)q[4] * 1e3, cs = (double)q[5] * 1e7, w = q[6], ps = (double)q[7] * pi / 180.0;
  const double lam = 12.2639 / sqrt(volt + 0.97845e-6 * volt * volt);
  const double u2 = 1.0 / (((double)L * apix) * ((double)L * apix));
  const double a = -pi * lam * u2;
  const double c0 = a * 0.5 * (dfu + dfv);
  const double c1 = a * 0.5 * (dfu - dfv) * cos(2.0 * ang);
  const double c2 = a * 0.5 * (dfu - dfv) * sin(2.0 * ang);
  CtfCoef c;
  c.c0h = (float)c0;
  c.c0l = (float)(c0 - (double)c.c0h);
  c.c1h = (float)c1;
  c.c1l = (float)(c1 - (double)c.c1h);
  c.c2h = (float)c2;
  c.c2l = (float)(c2 - (double)c.c2h);
  c.d = (float)(0.5 * pi * cs * lam * lam * lam * u2 * u2);
  c.ps = (float)ps;
  c.sw = (float)sqrt(1.0 - w * w);
  c.w = (float)w;
  c.pad0 = c.pad1 = 0.0f;
  return c;
}

__global__ void ctf_coef_kernel(const float *__restrict__ prm, int64_t n, int L, CtfCoef *__restrict__ out) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < n) out[b] = make_ctf_coef(prm + b * COV3D_CTF_NPARAMS, L);
}

// One block per image: its coefficients once, then every pixel.
__global__ void ctf_images_kernel(const float *__restrict__ prm, int L, float *__restrict__ out) {
  __shared__ CtfCoef c;
  const int64_t b = blockIdx.x;
  if (threadIdx.x == 0) c = make_ctf_coef(prm + b * COV3D_CTF_NPARAMS, L);
  __syncthreads();
  const int P = L * L;
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    const int row = p / L, col = p - (p / L) * L;
    out[b * P + p] = ctf_eval(c, row - L / 2, col - L / 2);
  }
}

}  // namespace

int prepare_ctf_coef(cov3d_plan *p, const float *params, int64_t n_images, int L, const CtfCoef **out) {
  COV3D_TRY(grow(p->ctfc, n_images * (int64_t)sizeof(CtfCoef)));
  ctf_coef_kernel<<<(unsigned)((n_images + 127) / 128), 128, 0, p->stream>>>(params, n_images, L,
                                                                           p->ctfc.as<CtfCoef>());
  COV3D_LAUNCHED("ctf_coef_kernel");
  *out = p->ctfc.as<CtfCoef>();
  return COV3D_OK;
}

}  // namespace cov3d

extern "C" int cov3d_ctf_images(void *stream, const float *d_params, int64_t n_images, int L, float *d_out) {
  using namespace cov3d;
  if (!d_params || !d_out || n_images < 0 || L < 1) {
    set_error("invalid ctf_images arguments");
    return COV3D_EINVAL;
  }
  if (n_images == 0) return COV3D_OK;
  ctf_images_kernel<<<(unsigned)n_images, 256, 0, static_cast<cudaStream_t>(stream)>>>(d_params, L, d_out);
  COV3D_LAUNCHED("ctf_images_kernel");
  return COV3D_OK;
}
