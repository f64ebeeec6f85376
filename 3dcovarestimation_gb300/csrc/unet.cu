// Kernels of the learned CG preconditioner: a small 3D U-Net that maps features of the mean's
// kernel density (on a 32^3 grid) to a log-correction of the circulant preconditioner symbol.
// No counterpart in the reference.  Forward and backward of every layer are here, so the
// network is trained on the device by these kernels:
//   conv3d (kernel 1 or 3, stride 1, zero padding, optional fused ReLU), its data and weight
//   gradients, the ReLU gradient, 2x average pooling, 2x nearest upsampling, trilinear
//   resampling (align_corners = False) and its adjoint, and integer-factor block averaging.
// Layout: (batch, channels, D, H, W) float32, contiguous.  Weights (Cout, Cin, k, k, k).
// The volumes are small (32^3, 16..96 channels): the kernels are latency-bound, FP32 on the
// CUDA cores with weights staged in shared memory.
#include "cov3d_internal.cuh"

namespace cov3d {

namespace {

constexpr int kCoBlock = 8;   // output channels per thread in the forward convolution
constexpr int kCiChunk = 16;  // input channels staged in shared memory per pass

inline unsigned nb(int64_t n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

// y[n, co, v] = b[co] + sum_ci sum_t w[co, ci, t] x[n, ci, v + off(t)]   (ReLU when relu)
template <int K>
__global__ void __launch_bounds__(256) conv3d_fwd_kernel(const float *__restrict__ x, const float *__restrict__ w,
                                                         const float *__restrict__ bias, float *__restrict__ y, int Cin,
                                                         int Cout, int D, int H, int W, int relu) {
  constexpr int T = K * K * K, R = K / 2;
  __shared__ float sw[kCoBlock * kCiChunk * T];
  const int64_t DHW = (int64_t)D * H * W;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int co0 = blockIdx.y * kCoBlock;
  const int n = blockIdx.z;
  const bool live = v < DHW;
  const int iw = live ? (int)(v % W) : 0, ih = live ? (int)((v / W) % H) : 0, id = live ? (int)(v / ((int64_t)W * H)) : 0;
  float acc[kCoBlock];
#pragma unroll
  for (int j = 0; j < kCoBlock; ++j) acc[j] = (bias && co0 + j < Cout) ? bias[co0 + j] : 0.0f;
  const float *xn = x + (int64_t)n * Cin * DHW;
  for (int ci0 = 0; ci0 < Cin; ci0 += kCiChunk) {
    const int cc = min(kCiChunk, Cin - ci0);
    __syncthreads();
    for (int i = threadIdx.x; i < kCoBlock * kCiChunk * T; i += blockDim.x) {
      const int j = i / (kCiChunk * T), rem = i - j * (kCiChunk * T), ci = rem / T, t = rem - ci * T;
      sw[i] = (co0 + j < Cout && ci < cc) ? w[((int64_t)(co0 + j) * Cin + ci0 + ci) * T + t] : 0.0f;
    }
    __syncthreads();
    if (live) {
      for (int ci = 0; ci < cc; ++ci) {
        const float *xc = xn + (int64_t)(ci0 + ci) * DHW;
#pragma unroll
        for (int t = 0; t < T; ++t) {
          const int dz = t / (K * K) - R, dy = (t / K) % K - R, dx = t % K - R;
          const int z = id + dz, yy = ih + dy, xx = iw + dx;
          const bool in = z >= 0 && z < D && yy >= 0 && yy < H && xx >= 0 && xx < W;
          const float xv = in ? __ldg(xc + ((int64_t)z * H + yy) * W + xx) : 0.0f;
#pragma unroll
          for (int j = 0; j < kCoBlock; ++j) acc[j] = fmaf(sw[(j * kCiChunk + ci) * T + t], xv, acc[j]);
        }
      }
    }
  }
  if (!live) return;
#pragma unroll
  for (int j = 0; j < kCoBlock; ++j) {
    if (co0 + j < Cout) {
      const float a = acc[j];
      y[((int64_t)n * Cout + co0 + j) * DHW + v] = relu ? fmaxf(a, 0.0f) : a;
    }
  }
}

// w'[ci, co, t] = w[co, ci, T - 1 - t]: the data gradient of a convolution is the convolution of
// the output gradient with the flipped, channel-transposed kernel.
__global__ void flip_transpose_kernel(const float *__restrict__ w, int Cout, int Cin, int T, float *__restrict__ wt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)Cout * Cin * T) return;
  const int t = (int)(i % T), ci = (int)((i / T) % Cin), co = (int)(i / ((int64_t)T * Cin));
  wt[((int64_t)ci * Cout + co) * T + (T - 1 - t)] = w[i];
}

// gw[co, ci, t] = sum_n sum_v gy[n, co, v] x[n, ci, v + off(t)];  gb[co] = sum gy[n, co, v]
// (one block per (ci, co); the ci = 0 blocks also reduce the bias gradient)
template <int K>
__global__ void __launch_bounds__(256) conv3d_wgrad_kernel(const float *__restrict__ x, const float *__restrict__ gy,
                                                           float *__restrict__ gw, float *__restrict__ gb, int N,
                                                           int Cin, int Cout, int D, int H, int W) {
  constexpr int T = K * K * K, R = K / 2;
  const int ci = blockIdx.x, co = blockIdx.y;
  const int64_t DHW = (int64_t)D * H * W;
  float acc[T + 1];
#pragma unroll
  for (int t = 0; t <= T; ++t) acc[t] = 0.0f;
  for (int n = 0; n < N; ++n) {
    const float *g = gy + ((int64_t)n * Cout + co) * DHW;
    const float *xc = x + ((int64_t)n * Cin + ci) * DHW;
    for (int64_t v = threadIdx.x; v < DHW; v += blockDim.x) {
      const float gv = __ldg(g + v);
      acc[T] += gv;
      const int iw = (int)(v % W), ih = (int)((v / W) % H), id = (int)(v / ((int64_t)W * H));
#pragma unroll
      for (int t = 0; t < T; ++t) {
        const int z = id + t / (K * K) - R, yy = ih + (t / K) % K - R, xx = iw + t % K - R;
        const bool in = z >= 0 && z < D && yy >= 0 && yy < H && xx >= 0 && xx < W;
        acc[t] = fmaf(gv, in ? __ldg(xc + ((int64_t)z * H + yy) * W + xx) : 0.0f, acc[t]);
      }
    }
  }
  __shared__ float red[8][T + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t <= T; ++t) {
    float s = acc[t];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[warp][t] = s;
  }
  __syncthreads();
  for (int t = threadIdx.x; t <= T; t += blockDim.x) {
    float s = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k][t];
    if (t < T) {
      gw[((int64_t)co * Cin + ci) * T + t] = s;
    } else if (ci == 0 && gb) {
      gb[co] = s;
    }
  }
}

// gx = gy * (y > 0)
__global__ void relu_bwd_kernel(const float *__restrict__ y, const float *__restrict__ gy, int64_t count,
                                float *__restrict__ gx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) gx[i] = y[i] > 0.0f ? gy[i] : 0.0f;
}

// 2x average pooling of (NC, D, H, W) -> (NC, D/2, H/2, W/2), and its adjoint
__global__ void avgpool2_fwd_kernel(const float *__restrict__ x, int64_t NC, int D, int H, int W, float *__restrict__ y) {
  const int d = D / 2, h = H / 2, w = W / 2;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NC * d * h * w) return;
  const int k = (int)(i % w), j = (int)((i / w) % h), l = (int)((i / ((int64_t)w * h)) % d);
  const int64_t c = i / ((int64_t)w * h * d);
  const float *src = x + c * D * H * W;
  float s = 0.0f;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int e = 0; e < 2; ++e) s += src[((int64_t)(2 * l + a) * H + 2 * j + b) * W + 2 * k + e];
  y[i] = 0.125f * s;
}

__global__ void avgpool2_bwd_kernel(const float *__restrict__ gy, int64_t NC, int D, int H, int W, float *__restrict__ gx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NC * D * H * W) return;
  const int k = (int)(i % W), j = (int)((i / W) % H), l = (int)((i / ((int64_t)W * H)) % D);
  const int64_t c = i / ((int64_t)W * H * D);
  const int d = D / 2, h = H / 2, w = W / 2;
  gx[i] = 0.125f * gy[((c * d + l / 2) * h + j / 2) * w + k / 2];
}

// 2x nearest upsampling of (NC, d, h, w) -> (NC, 2d, 2h, 2w), and its adjoint (sum of children)
__global__ void upsample2_fwd_kernel(const float *__restrict__ x, int64_t NC, int d, int h, int w, float *__restrict__ y) {
  const int D = 2 * d, H = 2 * h, W = 2 * w;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NC * D * H * W) return;
  const int k = (int)(i % W), j = (int)((i / W) % H), l = (int)((i / ((int64_t)W * H)) % D);
  const int64_t c = i / ((int64_t)W * H * D);
  y[i] = x[((c * d + l / 2) * h + j / 2) * w + k / 2];
}

__global__ void upsample2_bwd_kernel(const float *__restrict__ gy, int64_t NC, int d, int h, int w, float *__restrict__ gx) {
  const int D = 2 * d, H = 2 * h, W = 2 * w;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NC * d * h * w) return;
  const int k = (int)(i % w), j = (int)((i / w) % h), l = (int)((i / ((int64_t)w * h)) % d);
  const int64_t c = i / ((int64_t)w * h * d);
  const float *src = gy + c * D * H * W;
  float s = 0.0f;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int e = 0; e < 2; ++e) s += src[((int64_t)(2 * l + a) * H + 2 * j + b) * W + 2 * k + e];
  gx[i] = s;
}

}  // namespace
}  // namespace cov3d

namespace cov3d {
namespace {

// align_corners = False linear interpolation taps along one axis (Din samples -> Dout samples)
__device__ __forceinline__ void lin_taps(int i, int Din, int Dout, int &i0, int &i1, float &f) {
  float s = ((float)i + 0.5f) * ((float)Din / (float)Dout) - 0.5f;
  s = fmaxf(s, 0.0f);
  i0 = min((int)floorf(s), Din - 1);
  i1 = min(i0 + 1, Din - 1);
  f = s - (float)i0;
}

// (NC, d, d, d) -> (NC, D, D, D) trilinear
__global__ void trilinear_fwd_kernel(const float *__restrict__ x, int64_t NC, int d, int D, float *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NC * D * D * D) return;
  const int k = (int)(i % D), j = (int)((i / D) % D), l = (int)((i / ((int64_t)D * D)) % D);
  const int64_t c = i / ((int64_t)D * D * D);
  int a0, a1, b0, b1, e0, e1;
  float fa, fb, fe;
  lin_taps(l, d, D, a0, a1, fa);
  lin_taps(j, d, D, b0, b1, fb);
  lin_taps(k, d, D, e0, e1, fe);
  const float *src = x + c * d * d * d;
  auto at = [&](int a, int b, int e) { return src[((int64_t)a * d + b) * d + e]; };
  const float v0 = (1 - fb) * ((1 - fe) * at(a0, b0, e0) + fe * at(a0, b0, e1)) +
                   fb * ((1 - fe) * at(a0, b1, e0) + fe * at(a0, b1, e1));
  const float v1 = (1 - fb) * ((1 - fe) * at(a1, b0, e0) + fe * at(a1, b0, e1)) +
                   fb * ((1 - fe) * at(a1, b1, e0) + fe * at(a1, b1, e1));
  y[i] = (1 - fa) * v0 + fa * v1;
}

// adjoint of trilinear_fwd (gx must be zeroed)
__global__ void trilinear_bwd_kernel(const float *__restrict__ gy, int64_t NC, int d, int D, float *__restrict__ gx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NC * D * D * D) return;
  const int k = (int)(i % D), j = (int)((i / D) % D), l = (int)((i / ((int64_t)D * D)) % D);
  const int64_t c = i / ((int64_t)D * D * D);
  int a[2], b[2], e[2];
  float fa, fb, fe;
  lin_taps(l, d, D, a[0], a[1], fa);
  lin_taps(j, d, D, b[0], b[1], fb);
  lin_taps(k, d, D, e[0], e[1], fe);
  const float wa[2] = {1 - fa, fa}, wb[2] = {1 - fb, fb}, we[2] = {1 - fe, fe};
  const float g = gy[i];
  float *dst = gx + c * d * d * d;
  for (int p = 0; p < 2; ++p)
    for (int q = 0; q < 2; ++q)
      for (int s = 0; s < 2; ++s) atomicAdd(dst + ((int64_t)a[p] * d + b[q]) * d + e[s], g * wa[p] * wb[q] * we[s]);
}

// (NC, D, D, D) -> (NC, d, d, d), mean over k^3 blocks, k = D / d
__global__ void block_mean_kernel(const float *__restrict__ x, int64_t NC, int D, int d, float *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NC * d * d * d) return;
  const int k = D / d;
  const int e = (int)(i % d), b = (int)((i / d) % d), a = (int)((i / ((int64_t)d * d)) % d);
  const int64_t c = i / ((int64_t)d * d * d);
  const float *src = x + c * D * D * D;
  double s = 0.0;
  for (int p = 0; p < k; ++p)
    for (int q = 0; q < k; ++q)
      for (int r = 0; r < k; ++r) s += src[((int64_t)(a * k + p) * D + b * k + q) * D + e * k + r];
  y[i] = (float)(s / ((double)k * k * k));
}

template <int K>
int launch_conv_fwd(cudaStream_t s, const float *x, int N, int Cin, int D, int H, int W, const float *w,
                    const float *b, int Cout, int relu, float *y) {
  const int64_t DHW = (int64_t)D * H * W;
  dim3 grid(nb(DHW), (Cout + kCoBlock - 1) / kCoBlock, N);
  conv3d_fwd_kernel<K><<<grid, 256, 0, s>>>(x, w, b, y, Cin, Cout, D, H, W, relu);
  return launched("conv3d_fwd_kernel");
}

bool conv_args_ok(int N, int Cin, int Cout, int D, int H, int W, int ksize) {
  return N > 0 && Cin > 0 && Cout > 0 && D > 0 && H > 0 && W > 0 && (ksize == 1 || ksize == 3) && N <= 65535;
}

}  // namespace
}  // namespace cov3d

using namespace cov3d;

extern "C" {

int cov3d_conv3d_forward(void *stream, const float *d_x, int N, int Cin, int D, int H, int W, const float *d_w,
                         const float *d_bias, int Cout, int ksize, int relu, float *d_y) {
  if (!d_x || !d_w || !d_y || !conv_args_ok(N, Cin, Cout, D, H, W, ksize)) {
    set_error("invalid conv3d_forward arguments");
    return COV3D_EINVAL;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return ksize == 3 ? launch_conv_fwd<3>(s, d_x, N, Cin, D, H, W, d_w, d_bias, Cout, relu, d_y)
                    : launch_conv_fwd<1>(s, d_x, N, Cin, D, H, W, d_w, d_bias, Cout, relu, d_y);
}

int cov3d_conv3d_backward_data(void *stream, const float *d_gy, int N, int Cout, int D, int H, int W,
                               const float *d_w, int Cin, int ksize, float *d_wt_scratch, float *d_gx) {
  if (!d_gy || !d_w || !d_gx || !d_wt_scratch || !conv_args_ok(N, Cin, Cout, D, H, W, ksize)) {
    set_error("invalid conv3d_backward_data arguments");
    return COV3D_EINVAL;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int T = ksize * ksize * ksize;
  const int64_t nw = (int64_t)Cout * Cin * T;
  flip_transpose_kernel<<<nb(nw), 256, 0, s>>>(d_w, Cout, Cin, T, d_wt_scratch);
  COV3D_LAUNCHED("flip_transpose_kernel");
  return ksize == 3 ? launch_conv_fwd<3>(s, d_gy, N, Cout, D, H, W, d_wt_scratch, nullptr, Cin, 0, d_gx)
                    : launch_conv_fwd<1>(s, d_gy, N, Cout, D, H, W, d_wt_scratch, nullptr, Cin, 0, d_gx);
}

int cov3d_conv3d_backward_weight(void *stream, const float *d_x, const float *d_gy, int N, int Cin, int Cout, int D,
                                 int H, int W, int ksize, float *d_gw, float *d_gb) {
  if (!d_x || !d_gy || !d_gw || !conv_args_ok(N, Cin, Cout, D, H, W, ksize) || Cin > 65535 || Cout > 65535) {
    set_error("invalid conv3d_backward_weight arguments");
    return COV3D_EINVAL;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dim3 grid(Cin, Cout);
  if (ksize == 3) {
    conv3d_wgrad_kernel<3><<<grid, 256, 0, s>>>(d_x, d_gy, d_gw, d_gb, N, Cin, Cout, D, H, W);
  } else {
    conv3d_wgrad_kernel<1><<<grid, 256, 0, s>>>(d_x, d_gy, d_gw, d_gb, N, Cin, Cout, D, H, W);
  }
  return launched("conv3d_wgrad_kernel");
}

int cov3d_relu_backward(void *stream, const float *d_y, const float *d_gy, int64_t count, float *d_gx) {
  if (!d_y || !d_gy || !d_gx || count < 0) {
    set_error("invalid relu_backward arguments");
    return COV3D_EINVAL;
  }
  if (count == 0) return COV3D_OK;
  relu_bwd_kernel<<<nb(count), 256, 0, static_cast<cudaStream_t>(stream)>>>(d_y, d_gy, count, d_gx);
  return launched("relu_bwd_kernel");
}

/* direction 0: forward (x (NC, D, H, W) -> y (NC, D/2, H/2, W/2)); 1: adjoint (gy -> gx). */
int cov3d_avgpool2(void *stream, const float *d_in, int64_t NC, int D, int H, int W, int direction, float *d_out) {
  if (!d_in || !d_out || NC <= 0 || D < 2 || H < 2 || W < 2 || (D | H | W) & 1) {
    set_error("invalid avgpool2 arguments (even sizes >= 2)");
    return COV3D_EINVAL;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (direction == 0) {
    avgpool2_fwd_kernel<<<nb(NC * (D / 2) * (H / 2) * (W / 2)), 256, 0, s>>>(d_in, NC, D, H, W, d_out);
  } else {
    avgpool2_bwd_kernel<<<nb(NC * D * H * W), 256, 0, s>>>(d_in, NC, D, H, W, d_out);
  }
  return launched("avgpool2_kernel");
}

/* direction 0: forward (x (NC, d, h, w) -> y (NC, 2d, 2h, 2w)); 1: adjoint (gy -> gx). */
int cov3d_upsample2(void *stream, const float *d_in, int64_t NC, int d, int h, int w, int direction, float *d_out) {
  if (!d_in || !d_out || NC <= 0 || d < 1 || h < 1 || w < 1) {
    set_error("invalid upsample2 arguments");
    return COV3D_EINVAL;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (direction == 0) {
    upsample2_fwd_kernel<<<nb(NC * 8 * d * h * w), 256, 0, s>>>(d_in, NC, d, h, w, d_out);
  } else {
    upsample2_bwd_kernel<<<nb(NC * d * h * w), 256, 0, s>>>(d_in, NC, d, h, w, d_out);
  }
  return launched("upsample2_kernel");
}

/* Cubic volumes: direction 0 trilinear (NC, d^3) -> (NC, D^3); 1 its adjoint (gy (NC, D^3) ->
 * gx (NC, d^3), overwritten); 2 block mean (NC, D^3) -> (NC, d^3) with D a multiple of d
 * (d_in is then the D^3 volume). */
int cov3d_resample3d(void *stream, const float *d_in, int64_t NC, int d, int D, int direction, float *d_out) {
  if (!d_in || !d_out || NC <= 0 || d < 1 || D < 1 || direction < 0 || direction > 2 ||
      (direction == 2 && D % d != 0)) {
    set_error("invalid resample3d arguments");
    return COV3D_EINVAL;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (direction == 0) {
    trilinear_fwd_kernel<<<nb(NC * D * D * D), 256, 0, s>>>(d_in, NC, d, D, d_out);
  } else if (direction == 1) {
    COV3D_CUDA(cudaMemsetAsync(d_out, 0, (size_t)(NC * d * d * d) * sizeof(float), s));
    trilinear_bwd_kernel<<<nb(NC * D * D * D), 256, 0, s>>>(d_in, NC, d, D, d_out);
  } else {
    block_mean_kernel<<<nb(NC * d * d * d), 256, 0, s>>>(d_in, NC, D, d, d_out);
  }
  return launched("resample3d_kernel");
}

}  // extern "C"
