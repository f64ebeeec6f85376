// BF16 tensor-core Gram contractions of the covariance cost (tcgen05, accumulators in TMEM).
//
// Per image b the r projections Q_b (P pixels, complex) and the image y_b are stacked as
// C = 2(r+1) real rows X_b = [Re Q_0 .. Re Q_{r-1}, Re y, Im Q_0 .. Im Q_{r-1}, Im y] in BF16
// (pack_x_kernel, rows padded with zeros to a multiple of kKT pixels).  The real Gram
// G_b = X_b X_b^T (FP32 accumulation) holds every per-image contraction the cost needs:
//   gram_ij = sum_p conj(Q_pi) Q_pj = G[i][j] + G[i'][j'] + i (G[i][j'] - G[i'][j]),
//   h_i = the same with j = r (the image), |y|^2 = G[r][r] + G[r'][r'],  k' = k + r + 1
// (gram_kernel in gram_solve.cu computes the same in FP32 on the CUDA cores; the reference uses
// a batched complex GEMM, covar_sgd.py:1381-1399 and wiener_coords.py:168-203).
//
// gram_tc_kernel: one CTA per (group of IMG = 128 / C images, share of the pixels).  The
// group's IMG * C rows form the 128-row A operand of tcgen05.mma (M = 128, K = 16 per
// instruction, BF16 inputs, FP32 accumulator in TMEM); the B operand is the same rows
// (N = IMG * C rounded up to 16), so D = A A^T and the per-image Grams are its diagonal
// blocks.  The block-off-diagonal products are wasted MMA work, which costs nothing
// measurable: the contraction is bound by reading X from HBM.  Operands are staged by cp.async
// into a ring of kStages shared buffers in the canonical no-swizzle K-major layout (8 x 16-byte
// core matrices); one elected thread issues the MMAs and commits each stage to an mbarrier,
// which the loaders wait on before refilling that buffer.  Every wait is bounded: on timeout
// the CTA records an error, drains its copies and frees its TMEM.
#include <cuda_bf16.h>

#include "cov3d_internal.cuh"

namespace cov3d {

namespace {

constexpr int kKT = 128;                       // pixels per stage
constexpr int kStages = 4;                     // ring of shared buffers
constexpr int kRows = 128;                     // MMA M
constexpr int kK16Bytes = kRows * 16 * 2;      // one K=16 slab of the 128-row tile: 4096 bytes
constexpr int kStageBytes = kRows * kKT * 2;   // 32 KiB
constexpr int kThreads = 128;
constexpr int kTmemCols = 128;
constexpr long long kSpinLimit = 1LL << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, K-major, no swizzle: start address, leading-dimension
// (K-direction core-matrix) byte offset, stride-dimension (8-row group) byte offset, version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, absolute LBO mode, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t instr_desc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of (row m, 8-pixel chunk k8) inside a stage buffer
__device__ __forceinline__ uint32_t tile_offset(int m, int k8) {
  return (uint32_t)((k8 >> 1) * kK16Bytes + (m >> 3) * 256 + (k8 & 1) * 128 + (m & 7) * 16);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    gram_tc_kernel(const __nv_bfloat16 *__restrict__ X, int B, int C, int Ppad, int img_per_tile, int N, int ksplit,
                   float *__restrict__ G, int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[kStages];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int group = blockIdx.x / ksplit, part = blockIdx.x - group * ksplit;
  const int img0 = group * img_per_tile;
  const int nimg = min(img_per_tile, B - img0);
  const int rows = nimg * C;  // valid rows of the tile
  const int stages_total = Ppad / kKT;
  const int s_begin = (int)((int64_t)stages_total * part / ksplit);
  const int s_end = (int)((int64_t)stages_total * (part + 1) / ksplit);
  const int S = s_end - s_begin;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < kStages; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[i])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // zero the whole ring once: rows beyond `rows` stay zero for every stage
  for (int i = tid; i < kStages * kStageBytes / 16; i += kThreads)
    reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t sbase = smem_u32(smem);
  const uint32_t idesc = instr_desc_bf16(kRows, N);
  bool ok = true;

  auto load_stage = [&](int s) {  // stage s (relative) into buffer s % kStages
    const uint32_t buf = sbase + (uint32_t)((s % kStages) * kStageBytes);
    const int p0 = (s_begin + s) * kKT;
    for (int e = tid; e < rows * (kKT / 8); e += kThreads) {
      const int m = e / (kKT / 8), k8 = e - m * (kKT / 8);
      const int im = m / C, c = m - im * C;
      const __nv_bfloat16 *src = X + ((int64_t)(img0 + im) * C + c) * Ppad + p0 + k8 * 8;
      cp_async16(buf + tile_offset(m, k8), src);
    }
  };

  // prologue: kStages - 1 stages in flight
  for (int s = 0; s < kStages - 1; ++s) {
    if (s < S) load_stage(s);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  for (int s = 0; s < S; ++s) {
    // refill the buffer that stage s + kStages - 1 uses once the MMAs of stage s - 1 are done
    const int sn = s + kStages - 1;
    if (sn < S) {
      if (sn >= kStages) {  // that buffer was last read by stage sn - kStages = s - 1
        const int prev = sn - kStages;
        ok = ok && mbar_wait(smem_u32(&mbar[prev % kStages]), (uint32_t)((prev / kStages) & 1));
      }
      if (ok) load_stage(sn);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group %0;\n" ::"n"(kStages - 1) : "memory");  // stage s has landed
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (!__syncthreads_and(ok ? 1 : 0)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t buf = sbase + (uint32_t)((s % kStages) * kStageBytes);
#pragma unroll
      for (int kb = 0; kb < kKT / 16; ++kb) {
        const uint64_t ad = smem_desc(buf + kb * kK16Bytes, 128, 256);
        const uint32_t acc = (s > 0 || kb > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(ad), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(&mbar[s % kStages]))
                   : "memory");
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  // the last commit completes after every MMA of this CTA
  if (ok && S > 0) ok = mbar_wait(smem_u32(&mbar[(S - 1) % kStages]), (uint32_t)(((S - 1) / kStages) & 1));
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else if (S > 0) {
    // epilogue: warp w reads TMEM lanes 32w .. 32w+31 = rows m, 8 columns at a time
    const int m = warp * 32 + (tid & 31);
    const int im = m / C, cm = m - (m / C) * C;
    for (int col0 = 0; col0 < N; col0 += 8) {
      uint32_t v[8];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)col0)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (m < rows) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int n = col0 + j;
          if (n < rows && n / C == im) {
            float *dst = G + ((int64_t)(img0 + im) * C + cm) * C + (n - im * C);
            const float x = __uint_as_float(v[j]);
            if (ksplit == 1) {
              *dst = x;
            } else {
              atomicAdd(dst, x);
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// X[b][c][p] (BF16, rows of Ppad pixels, zero beyond P) from Q (point p, channel i) and y
__global__ void pack_x_kernel(const float2 *__restrict__ Q, int64_t q_is, int64_t q_ps, int64_t q_cs,
                              const float2 *__restrict__ Y, int P, int Ppad, int r, __nv_bfloat16 *__restrict__ X) {
  const int b = blockIdx.y;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= Ppad) return;
  const int C = 2 * (r + 1);
  __nv_bfloat16 *xb = X + (int64_t)b * C * Ppad + p;
  const bool in = p < P;
  for (int i = 0; i < r; ++i) {
    const float2 q = in ? Q[(int64_t)b * q_is + (int64_t)p * q_ps + (int64_t)i * q_cs] : make_float2(0.f, 0.f);
    xb[(int64_t)i * Ppad] = __float2bfloat16_rn(q.x);
    xb[(int64_t)(r + 1 + i) * Ppad] = __float2bfloat16_rn(q.y);
  }
  const float2 y = in ? Y[(int64_t)b * P + p] : make_float2(0.f, 0.f);
  xb[(int64_t)r * Ppad] = __float2bfloat16_rn(y.x);
  xb[(int64_t)(2 * r + 1) * Ppad] = __float2bfloat16_rn(y.y);
}

// gram / h / |y|^2 from the real Gram G (C x C per image)
__global__ void gram_from_real_kernel(const float *__restrict__ G, int B, int r, float2 *__restrict__ gram,
                                      float2 *__restrict__ h, float *__restrict__ yy) {
  const int b = blockIdx.x;
  const int C = 2 * (r + 1), o = r + 1;
  const float *g = G + (int64_t)b * C * C;
  for (int e = threadIdx.x; e < (r + 1) * (r + 1); e += blockDim.x) {
    const int i = e / (r + 1), j = e - i * (r + 1);
    const float re = g[i * C + j] + g[(i + o) * C + j + o];
    const float im = g[i * C + j + o] - g[(i + o) * C + j];
    if (i < r && j < r) {
      gram[((int64_t)b * r + i) * r + j] = make_float2(re, im);
    } else if (i < r && j == r) {
      h[(int64_t)b * r + i] = make_float2(re, im);
    } else if (i == r && j == r) {
      yy[b] = re;
    }
  }
}

}  // namespace

int reserve_gram_bf16(cov3d_plan *p, int B, int P, int r) {
  const int C = 2 * (r + 1);
  const int Ppad = (P + kKT - 1) / kKT * kKT;
  COV3D_TRY(grow(p->xbf, (int64_t)B * C * Ppad * 2));
  COV3D_TRY(grow(p->gsum, (int64_t)B * C * C * 4 + 16));
  return COV3D_OK;
}

int launch_gram_bf16(cov3d_plan *p, cudaStream_t st, int B, int P, int r, const void *q, int64_t is, int64_t ps,
                     int64_t cs, const void *images, void *gram, void *h, float *yy) {
  const int C = 2 * (r + 1);
  if (r < 1 || C > kRows) {
    set_error("bf16 Gram: rank %d out of range (C = 2(r+1) <= %d)", r, kRows);
    return COV3D_EINVAL;
  }
  const int Ppad = (P + kKT - 1) / kKT * kKT;
  const int img_per_tile = kRows / C;
  const int N = ((img_per_tile * C + 15) / 16) * 16;
  const int groups = (B + img_per_tile - 1) / img_per_tile;
  const int ksplit = Ppad / kKT >= 2 * kStages ? 2 : 1;
  COV3D_TRY(reserve_gram_bf16(p, B, P, r));
  __nv_bfloat16 *X = p->xbf.as<__nv_bfloat16>();
  float *G = p->gsum.as<float>();
  int *err = reinterpret_cast<int *>(G + (int64_t)B * C * C);
  COV3D_CUDA(cudaMemsetAsync(G, 0, (size_t)B * C * C * 4 + 16, st));
  dim3 pg((Ppad + 255) / 256, B);
  pack_x_kernel<<<pg, 256, 0, st>>>(static_cast<const float2 *>(q), is, ps, cs, static_cast<const float2 *>(images),
                                    P, Ppad, r, X);
  COV3D_LAUNCHED("pack_x_kernel");
  const size_t smem = (size_t)kStages * kStageBytes;
  static bool attr_set = false;
  if (!attr_set) {
    COV3D_CUDA(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  gram_tc_kernel<<<groups * ksplit, kThreads, smem, st>>>(X, B, C, Ppad, img_per_tile, N, ksplit, G, err);
  COV3D_LAUNCHED("gram_tc_kernel");
  gram_from_real_kernel<<<B, 128, 0, st>>>(G, B, r, static_cast<float2 *>(gram), static_cast<float2 *>(h), yy);
  return launched("gram_from_real_kernel");
}

int read_gram_bf16_error(cov3d_plan *p, cudaStream_t st, int B, int r) {
  const int C = 2 * (r + 1);
  int herr = 0;
  const int *err = reinterpret_cast<const int *>(p->gsum.as<float>() + (int64_t)B * C * C);
  COV3D_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  COV3D_CUDA(cudaStreamSynchronize(st));
  if (herr) {
    set_error("bf16 Gram: a pipeline wait timed out");
    return COV3D_ECUDA;
  }
  return COV3D_OK;
}

}  // namespace cov3d
