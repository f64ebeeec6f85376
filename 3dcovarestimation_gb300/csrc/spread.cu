// Spreading ("type-1" half of the NUFFT; exact adjoint of interp.cu, replacing the
// reference's grid_sample backward with FP32 global atomics, nufft_plan.py:171-242).
//
// One thread block per subproblem (<= max_sub points of one spatial bin).  The block
// accumulates its points' kernel footprints into a shared-memory tile covering the bin plus
// a (W-1)-cell halo, then adds the tile to the global grid once.  With `COMP` every shared
// accumulation is compensated: atomicAdd returns the previous value, so the rounding error of
// that exact addition is recovered with Knuth's TwoSum and accumulated in a second tile.
#include "cov3d_device.cuh"

namespace cov3d {

namespace {

struct SpreadParams {
  PointGeom g;
  KernelSpec k;
  Bins bins;
  const int *perm;
  const int *sub_bin;
  const int *sub_first;
  const int *sub_count;
  const int *nsub;
  const float2 *vals;
  int64_t ips, ics;
  int ch0;
  const float *ctf;
  int nyquist;
  float scale;
  float2 *grid;
  int64_t cs, chs;
  int shift;
  int T0, T1, T2;
};

template <bool COMP>
__device__ __forceinline__ void tile_add(float *hi, float *lo, int idx, float v) {
  if (!COMP) {
    atomicAdd(hi + idx, v);
  } else {
    const float old = atomicAdd(hi + idx, v);
    const float s = old + v;
    const float bb = s - old;
    const float err = (old - (s - bb)) + (v - bb);
    if (err != 0.0f) atomicAdd(lo + idx, err);
  }
}

// Prologue factor of im_backward: CTF multiply, Nyquist zeroing, scale (projection_funcs.py:385-399).
__device__ __forceinline__ float prologue(const PointGeom &g, int64_t id, const float *ctf, int nyquist, float scale) {
  float sc = scale;
  if (nyquist && (g.Lp % 2 == 0)) {
    const int64_t b = id / g.P;
    const int p = (int)(id - b * g.P);
    const int row = p / g.Lp;
    const int col = p - row * g.Lp;
    if (row == 0 || col == 0) sc = 0.0f;
  }
  if (ctf) sc *= __ldg(ctf + id);
  return sc;
}

template <int KT, int W, int CH, bool COMP>
__global__ void __launch_bounds__(256) spread_kernel(const SpreadParams a) {
  extern __shared__ float smem[];
  const int sub = blockIdx.x;
  if (sub >= *a.nsub) return;
  const int TT = a.T0 * a.T1 * a.T2;
  float *hi = smem;
  float *lo = smem + 2 * CH * TT;
  const int bin = a.sub_bin[sub];
  const int first = a.sub_first[sub];
  const int cnt = a.sub_count[sub];
  const int nb12 = a.bins.nb[1] * a.bins.nb[2];
  const int ts0 = (bin / nb12) * a.bins.bs[0];
  const int ts1 = ((bin / a.bins.nb[2]) % a.bins.nb[1]) * a.bins.bs[1];
  const int ts2 = (bin % a.bins.nb[2]) * a.bins.bs[2];
  const int n = a.g.n;

  for (int q = threadIdx.x; q < (COMP ? 4 : 2) * CH * TT; q += blockDim.x) smem[q] = 0.0f;
  __syncthreads();

  for (int kk = threadIdx.x; kk < cnt; kk += blockDim.x) {
    const int64_t id = __ldg(a.perm + first + kk);
    const float sc = prologue(a.g, id, a.ctf, a.nyquist, a.scale);
    if (sc == 0.0f) continue;
    float t[3];
    point_index(a.g, id, t);
    float wt[3][W];
    int l[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int c0 = taps<KT, W>(t[d], a.k.beta, wt[d]);
      if (KT == COV3D_KERNEL_ES) c0 = pmod(c0, n);
      l[d] = c0 - (d == 0 ? ts0 : d == 1 ? ts1 : ts2);
    }
    float2 v[CH];
    const float2 *src = a.vals + id * a.ips + (int64_t)a.ch0 * a.ics;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const float2 x = __ldg(src + c * a.ics);
      v[c] = make_float2(x.x * sc, x.y * sc);
    }
#pragma unroll 1
    for (int i0 = 0; i0 < W; ++i0) {
      const int la = l[0] + i0;
      if (KT != COV3D_KERNEL_ES && (la < 0 || wt[0][i0] == 0.0f)) continue;
#pragma unroll
      for (int i1 = 0; i1 < W; ++i1) {
        const int lb = l[1] + i1;
        if (KT != COV3D_KERNEL_ES && (lb < 0 || wt[1][i1] == 0.0f)) continue;
        const float wab = wt[0][i0] * wt[1][i1];
        const int rowi = (la * a.T1 + lb) * a.T2;
#pragma unroll
        for (int i2 = 0; i2 < W; ++i2) {
          const int lc = l[2] + i2;
          if (KT != COV3D_KERNEL_ES && (lc < 0 || wt[2][i2] == 0.0f)) continue;
          const float w = wab * wt[2][i2];
          const int idx = rowi + lc;
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            tile_add<COMP>(hi, lo, (2 * c) * TT + idx, w * v[c].x);
            tile_add<COMP>(hi, lo, (2 * c + 1) * TT + idx, w * v[c].y);
          }
        }
      }
    }
  }
  __syncthreads();

  const int T12 = a.T1 * a.T2;
  for (int q = threadIdx.x; q < TT; q += blockDim.x) {
    const int la = q / T12;
    const int lb = (q / a.T2) % a.T1;
    const int lc = q % a.T2;
    int m0 = ts0 + la, m1 = ts1 + lb, m2 = ts2 + lc;
    if (KT == COV3D_KERNEL_ES) {
      m0 = m0 >= n ? m0 - n : m0;
      m1 = m1 >= n ? m1 - n : m1;
      m2 = m2 >= n ? m2 - n : m2;
    } else if (m0 >= n || m1 >= n || m2 >= n) {
      continue;
    }
    m0 += a.shift;
    m1 += a.shift;
    m2 += a.shift;
    m0 = m0 >= n ? m0 - n : m0;
    m1 = m1 >= n ? m1 - n : m1;
    m2 = m2 >= n ? m2 - n : m2;
    float2 *dst = a.grid + (((int64_t)m0 * n + m1) * n + m2) * a.cs + (int64_t)a.ch0 * a.chs;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      float re = hi[(2 * c) * TT + q];
      float im = hi[(2 * c + 1) * TT + q];
      if (COMP) {
        re += lo[(2 * c) * TT + q];
        im += lo[(2 * c + 1) * TT + q];
      }
      if (re != 0.0f) atomicAdd(&dst[c * a.chs].x, re);
      if (im != 0.0f) atomicAdd(&dst[c * a.chs].y, im);
    }
  }
}

template <int KT, int W, int CH, bool COMP>
int launch_one(const SpreadParams &a, int64_t max_blocks, cudaStream_t st) {
  const int64_t TT = (int64_t)a.T0 * a.T1 * a.T2;
  const size_t smem = (size_t)(COMP ? 4 : 2) * CH * TT * sizeof(float);
  static size_t configured = 0;
  if (smem > 48 * 1024 && smem > configured) {
    cudaError_t e = cudaFuncSetAttribute(spread_kernel<KT, W, CH, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(spread_kernel)");
    configured = smem;
  }
  spread_kernel<KT, W, CH, COMP><<<(unsigned)max_blocks, 256, smem, st>>>(a);
  return launched("spread_kernel");
}

constexpr size_t kSpreadSmemBudget = 112 * 1024;  // two blocks per SM

template <int KT, int W>
int launch_w(SpreadParams a, int nchan, bool comp, int64_t max_blocks, cudaStream_t st) {
  const int64_t TT = (int64_t)a.T0 * a.T1 * a.T2;
  const size_t per_ch = (size_t)(comp ? 4 : 2) * TT * sizeof(float);
  int done = 0;
  while (done < nchan) {
    const int left = nchan - done;
    int ch = 1;
    if (left >= 4 && 4 * per_ch <= kSpreadSmemBudget) ch = 4;
    else if (left >= 2 && 2 * per_ch <= kSpreadSmemBudget) ch = 2;
    if (per_ch > 200 * 1024) {
      set_error("spreading tile of %lld cells does not fit in shared memory; use a smaller bin_size",
                (long long)TT);
      return COV3D_EINVAL;
    }
    a.ch0 = done;
    int s = COV3D_OK;
    if (comp) {
      s = ch == 4 ? launch_one<KT, W, 4, true>(a, max_blocks, st)
        : ch == 2 ? launch_one<KT, W, 2, true>(a, max_blocks, st)
                  : launch_one<KT, W, 1, true>(a, max_blocks, st);
    } else {
      s = ch == 4 ? launch_one<KT, W, 4, false>(a, max_blocks, st)
        : ch == 2 ? launch_one<KT, W, 2, false>(a, max_blocks, st)
                  : launch_one<KT, W, 1, false>(a, max_blocks, st);
    }
    if (s != COV3D_OK) return s;
    done += ch;
  }
  return COV3D_OK;
}

// Per-image adjoint (no sum over images): direct global atomics, one thread per point.
template <int KT, int W>
__global__ void spread_unagg_kernel(PointGeom g, KernelSpec k, int64_t M, const float2 *__restrict__ vals,
                                    int64_t ips, const float *ctf, int nyquist, float scale, float2 *grids) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= M) return;
  const float sc = prologue(g, id, ctf, nyquist, scale);
  if (sc == 0.0f) return;
  const int n = g.n;
  float t[3];
  point_index(g, id, t);
  float wt[3][W];
  int c0[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) c0[d] = taps<KT, W>(t[d], k.beta, wt[d]);
  const float2 x = vals[id * ips];
  const float2 v = make_float2(x.x * sc, x.y * sc);
  float2 *out = grids + (id / g.P) * (int64_t)n * n * n;
  for (int i0 = 0; i0 < W; ++i0) {
    int m0 = c0[0] + i0;
    if (KT == COV3D_KERNEL_ES) m0 = pmod(m0, n);
    else if (m0 < 0 || m0 >= n) continue;
    for (int i1 = 0; i1 < W; ++i1) {
      int m1 = c0[1] + i1;
      if (KT == COV3D_KERNEL_ES) m1 = pmod(m1, n);
      else if (m1 < 0 || m1 >= n) continue;
      for (int i2 = 0; i2 < W; ++i2) {
        int m2 = c0[2] + i2;
        if (KT == COV3D_KERNEL_ES) m2 = pmod(m2, n);
        else if (m2 < 0 || m2 >= n) continue;
        const float w = wt[0][i0] * wt[1][i1] * wt[2][i2];
        float2 *dst = out + ((int64_t)m0 * n + m1) * n + m2;
        atomicAdd(&dst->x, w * v.x);
        atomicAdd(&dst->y, w * v.y);
      }
    }
  }
}

}  // namespace

int launch_spread(cov3d_plan *p, const void *values, int64_t in_ps, int64_t in_cs, int nchan, const EpilogueArgs &e,
                  void *grid, int64_t cell_stride, int64_t chan_stride, int shift) {
  if (p->point_kind == kPointsNone || p->n_points == 0) {
    set_error("no points set");
    return COV3D_ESTATE;
  }
  SpreadParams a{};
  a.g = make_geom(p);
  a.k = make_kernel(p);
  a.bins = p->bins;
  a.perm = p->perm.as<int>();
  a.sub_bin = p->sub_bin.as<int>();
  a.sub_first = p->sub_first.as<int>();
  a.sub_count = p->sub_count.as<int>();
  a.nsub = p->nsub.as<int>();
  a.vals = static_cast<const float2 *>(values);
  a.ips = in_ps;
  a.ics = in_cs;
  a.ctf = e.ctf;
  a.nyquist = e.nyquist;
  a.scale = e.scale;
  a.grid = static_cast<float2 *>(grid);
  a.cs = cell_stride;
  a.chs = chan_stride;
  a.shift = shift;
  const int W = p->kernel == COV3D_KERNEL_NEAREST ? 1 : p->kernel == COV3D_KERNEL_LINEAR ? 2 : p->width;
  a.T0 = p->bins.bs[0] + W - 1;
  a.T1 = p->bins.bs[1] + W - 1;
  a.T2 = p->bins.bs[2] + W - 1;
  const int64_t max_blocks = p->bins.nbins + p->n_points / p->max_sub + 1;
  const bool comp = p->compensated != 0;
  switch (p->kernel) {
    case COV3D_KERNEL_NEAREST: return launch_w<COV3D_KERNEL_NEAREST, 1>(a, nchan, comp, max_blocks, p->stream);
    case COV3D_KERNEL_LINEAR: return launch_w<COV3D_KERNEL_LINEAR, 2>(a, nchan, comp, max_blocks, p->stream);
    default:
      switch (p->width) {
        case 4: return launch_w<COV3D_KERNEL_ES, 4>(a, nchan, comp, max_blocks, p->stream);
        case 5: return launch_w<COV3D_KERNEL_ES, 5>(a, nchan, comp, max_blocks, p->stream);
        case 6: return launch_w<COV3D_KERNEL_ES, 6>(a, nchan, comp, max_blocks, p->stream);
        case 7: return launch_w<COV3D_KERNEL_ES, 7>(a, nchan, comp, max_blocks, p->stream);
        case 8: return launch_w<COV3D_KERNEL_ES, 8>(a, nchan, comp, max_blocks, p->stream);
        default: set_error("unsupported ES width %d (supported: 4..8)", p->width); return COV3D_EINVAL;
      }
  }
}

int launch_spread_unaggregated(cov3d_plan *p, const void *values, int64_t in_ps, const EpilogueArgs &e,
                               void *grids) {
  if (p->point_kind == kPointsNone || p->n_points == 0) {
    set_error("no points set");
    return COV3D_ESTATE;
  }
  const PointGeom g = make_geom(p);
  const KernelSpec k = make_kernel(p);
  const int blocks = (int)((p->n_points + 255) / 256);
  const float2 *v = static_cast<const float2 *>(values);
  float2 *out = static_cast<float2 *>(grids);
  switch (p->kernel) {
    case COV3D_KERNEL_NEAREST:
      spread_unagg_kernel<COV3D_KERNEL_NEAREST, 1>
          <<<blocks, 256, 0, p->stream>>>(g, k, p->n_points, v, in_ps, e.ctf, e.nyquist, e.scale, out);
      break;
    case COV3D_KERNEL_LINEAR:
      spread_unagg_kernel<COV3D_KERNEL_LINEAR, 2>
          <<<blocks, 256, 0, p->stream>>>(g, k, p->n_points, v, in_ps, e.ctf, e.nyquist, e.scale, out);
      break;
    default:
      switch (p->width) {
#define COV3D_UW(Wv)                                                                                     \
  case Wv:                                                                                             \
    spread_unagg_kernel<COV3D_KERNEL_ES, Wv>                                                           \
        <<<blocks, 256, 0, p->stream>>>(g, k, p->n_points, v, in_ps, e.ctf, e.nyquist, e.scale, out); \
    break;
        COV3D_UW(4) COV3D_UW(5) COV3D_UW(6) COV3D_UW(7) COV3D_UW(8)
#undef COV3D_UW
        default: set_error("unsupported ES width %d", p->width); return COV3D_EINVAL;
      }
  }
  return launched("spread_unagg_kernel");
}

}  // namespace cov3d
