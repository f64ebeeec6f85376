// Spreading ("type-1" half of the NUFFT; exact adjoint of interp.cu, replacing the
// reference's grid_sample backward with FP32 global atomics, nufft_plan.py:171-242), over the
// bin-sorted point records of points_sort.cu.  See spread_kernel for the decomposition.
#include <algorithm>
#include <vector>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

constexpr int kBin = 8;
constexpr int kSpreadWarps = 8;
constexpr int kPlanesPerWarp = 4;

struct SpreadParams {
  PointGeom g;
  KernelSpec k;
  Bins bins;
  const SortedPoint *pts;
  const int *sub_bin;
  const int *sub_first;
  const int *sub_count;
  const int *nsub;
  const float2 *vals;
  int64_t ips, ics;
  int ch0;
  int nch;  // channels in this pass (<= 2 * CP)
  const float *ctf;
  int nyquist;
  float scale;
  float2 *grid;
  int64_t cs, chs;
  int shift;
  int max_sub;
  const int *plane_sched;  // kSpreadWarps x kPlanesPerWarp tile planes per warp (-1 = none)
};

// Prologue factor of im_backward: CTF multiply, Nyquist zeroing, scale (projection_funcs.py:385-399).
__device__ __forceinline__ float prologue(const PointGeom &g, int64_t id, const float *ctf, int nyquist, float scale) {
  float sc = scale;
  if (nyquist && on_nyquist(g, id)) sc = 0.0f;
  if (ctf) sc *= __ldg(ctf + id);
  return sc;
}

// Channel pairs per pass (lanes are (window cell, channel pair)); COMP keeps a second
// (compensation) tile, so it uses half as many pairs.
template <int W, bool COMP>
struct SpreadCP {
  // largest W*CP <= 32 whose tile plus staged point values fit in shared memory
  static constexpr int full = W <= 2 ? 8 : W == 4 ? 7 : W == 8 ? 3 : 32 / W;
  static constexpr int value = COMP ? (full / 2 > 0 ? full / 2 : 1) : full;
};

// Per-point record staged once per block: packed window corner (tile-local, biased by 32 so
// zero-padding corners below the tile stay non-negative) and the 3W kernel weights.
template <int W>
struct PointRec {
  static constexpr int FLOATS = (1 + 3 * W + 3) / 4 * 4;
};

// One block per subproblem, tile = bin + (W-1)-cell halo of 2*CP channels in shared memory.
//  1. the block buckets its points by the axis-0 corner of their window (8 buckets);
//  2. warp w owns whole axis-0 planes of the tile (plane_sched balances the work: plane a is
//     reached by the points of min(W, ...) buckets); for every point reaching one of its planes
//     the warp's lanes (j, q) add weight * value to channels 2q, 2q+1 of tile[a][b][corner2 + j]
//     for the W rows b of the window -- contiguous 16-byte read-modify-writes, no bank
//     conflicts, and no two warps ever touch the same cell, so no atomics;
//     with COMP every addition is a TwoSum whose rounding error goes to the second tile;
//  3. the tile is added to the global grid, one complex atomic per cell and channel.
template <int KT, int W, int CP, bool COMP>
__global__ void __launch_bounds__(kSpreadWarps * 32) spread_kernel(const SpreadParams a) {
  constexpr int T = kBin + W - 1;
  constexpr int RG = 32 / (W * CP);  // window rows handled side by side by spare lanes
  constexpr int LANES = W * CP * RG;
  constexpr int TILE4 = T * T * T * CP;
  extern __shared__ float4 smem4[];
  float4 *hi = smem4;
  float4 *lo = smem4 + (COMP ? TILE4 : 0);
  float4 *s_val = smem4 + (COMP ? 2 : 1) * TILE4;  // max_sub * CP: scaled channel pairs per point
  float *s_rec = reinterpret_cast<float *>(s_val + a.max_sub * CP);  // max_sub * PointRec<W>::FLOATS
  int *s_idx = reinterpret_cast<int *>(s_rec + a.max_sub * PointRec<W>::FLOATS);
  int *s_bucket = s_idx + a.max_sub;
  int *s_cnt = s_bucket + a.max_sub;  // kBin
  int *s_off = s_cnt + kBin;          // kBin + 1

  const int sub = blockIdx.x;
  if (sub >= *a.nsub) return;
  const int bin = a.sub_bin[sub];
  const int first = a.sub_first[sub];
  const int cnt = a.sub_count[sub];
  const int nb12 = a.bins.nb[1] * a.bins.nb[2];
  const int ts0 = (bin / nb12) * kBin;
  const int ts1 = ((bin / a.bins.nb[2]) % a.bins.nb[1]) * kBin;
  const int ts2 = (bin % a.bins.nb[2]) * kBin;
  const int n = a.g.n;
  const int tid = threadIdx.x;

  for (int e = tid; e < (COMP ? 2 : 1) * TILE4; e += blockDim.x) smem4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid < kBin) s_cnt[tid] = 0;
  __syncthreads();
  // 1. stage the points' scaled values (im_backward prologue folded in) and bucket the points
  //    by axis-0 window corner
  for (int e = tid; e < cnt * CP; e += blockDim.x) {
    const int k = e / CP, qq = e - (e / CP) * CP;
    const SortedPoint sp = a.pts[first + k];
    const int64_t id = sp_id(sp.idf);
    float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
    if (a.ctf) sc *= __ldg(a.ctf + id);
    const float2 *src = a.vals + id * a.ips + (int64_t)(a.ch0 + 2 * qq) * a.ics;
    const float2 v0 = 2 * qq < a.nch ? __ldg(src) : make_float2(0.f, 0.f);
    const float2 v1 = 2 * qq + 1 < a.nch ? __ldg(src + a.ics) : make_float2(0.f, 0.f);
    s_val[e] = make_float4(v0.x * sc, v0.y * sc, v1.x * sc, v1.y * sc);
  }
  for (int k = tid; k < cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[first + k];
    float w0[W], w1[W], w2[W];
    int c0 = taps<KT, W>(sp.t0, a.k.beta, w0);
    int c1 = taps<KT, W>(sp.t1, a.k.beta, w1);
    int c2 = taps<KT, W>(sp.t2, a.k.beta, w2);
    if (KT == COV3D_KERNEL_ES) {
      c0 = wrap1(c0, n);
      c1 = wrap1(c1, n);
      c2 = wrap1(c2, n);
    }
    float *rec = s_rec + k * PointRec<W>::FLOATS;
    rec[0] = __int_as_float((c0 - ts0 + 32) | ((c1 - ts1 + 32) << 8) | ((c2 - ts2 + 32) << 16));
#pragma unroll
    for (int r = 0; r < W; ++r) {
      rec[1 + r] = w0[r];
      rec[1 + W + r] = w1[r];
      rec[1 + 2 * W + r] = w2[r];
    }
    const int b0 = max(c0 - ts0, 0);
    s_bucket[k] = b0 | (atomicAdd(s_cnt + b0, 1) << 4);
  }
  __syncthreads();
  if (tid == 0) {
    int acc = 0;
    for (int i = 0; i < kBin; ++i) {
      s_off[i] = acc;
      acc += s_cnt[i];
    }
    s_off[kBin] = acc;
  }
  __syncthreads();
  for (int k = tid; k < cnt; k += blockDim.x) {
    const int bk = s_bucket[k];
    s_idx[s_off[bk & 15] + (bk >> 4)] = k;
  }
  __syncthreads();

  // 2. planes of this warp
  const int warp = tid >> 5, lane = tid & 31;
  const int g = lane / (W * CP), lr = lane - g * (W * CP);
  const int j = lr / CP, q = lr - (lr / CP) * CP;
  const bool lane_live = lane < LANES;
  for (int s = 0; s < kPlanesPerWarp; ++s) {
    const int pa = __ldg(a.plane_sched + warp * kPlanesPerWarp + s);
    if (pa < 0) break;
    const int blo = max(0, pa - W + 1), bhi = min(kBin - 1, pa);
    const int i1end = s_off[bhi + 1];
    for (int i = s_off[blo]; i < i1end; ++i) {
      const int kp = s_idx[i];
      const float *rec = s_rec + kp * PointRec<W>::FLOATS;
      const int packed = __float_as_int(rec[0]);
      const int l0 = (packed & 255) - 32, l1 = ((packed >> 8) & 255) - 32, l2 = ((packed >> 16) & 255) - 32;
      const int o0 = pa - l0;  // tap along axis 0 that lands on this plane
      if (o0 >= W) continue;   // zero padding: window clamped into bucket 0 but below this plane
      const int cell2 = l2 + j;
      if (!lane_live || cell2 < 0) continue;
      const float4 vv = s_val[kp * CP + q];
      const float waj = rec[1 + o0] * rec[1 + 2 * W + j];
      float4 *rowp = hi + ((pa * T) * T + cell2) * CP + q;
      float4 *rowl = lo + ((pa * T) * T + cell2) * CP + q;
#pragma unroll
      for (int ii = 0; ii < (W + RG - 1) / RG; ++ii) {
        const int i1 = ii * RG + g;
        if (i1 >= W) break;
        const int r1 = l1 + i1;
        if (KT != COV3D_KERNEL_ES && r1 < 0) continue;
        const float w = waj * rec[1 + W + i1];
        float4 &h = rowp[r1 * T * CP];
        if (!COMP) {
          float4 x = h;
          x.x = fmaf(w, vv.x, x.x);
          x.y = fmaf(w, vv.y, x.y);
          x.z = fmaf(w, vv.z, x.z);
          x.w = fmaf(w, vv.w, x.w);
          h = x;
        } else {
          float4 x = h, e = rowl[r1 * T * CP];
          const float d[4] = {w * vv.x, w * vv.y, w * vv.z, w * vv.w};
          float *xs = &x.x, *es = &e.x;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const float s2 = xs[u] + d[u];
            const float bb = s2 - xs[u];
            es[u] += (xs[u] - (s2 - bb)) + (d[u] - bb);
            xs[u] = s2;
          }
          h = x;
          rowl[r1 * T * CP] = e;
        }
      }
    }
  }
  __syncthreads();

  // 3. add the tile to the global grid: per-row global offsets and per-cell axis-2 offsets first
  long long *s_rowoff = reinterpret_cast<long long *>(s_val);  // reuses the staged values
  int *s_coloff = reinterpret_cast<int *>(s_rowoff + T * T);
  for (int e = tid; e < T * T; e += blockDim.x) {
    const int ra = e / T, rb = e - (e / T) * T;
    int m0 = ts0 + ra, m1 = ts1 + rb;
    bool ok = true;
    if (KT == COV3D_KERNEL_ES) {
      m0 = m0 >= n ? m0 - n : m0;
      m1 = m1 >= n ? m1 - n : m1;
    } else {
      ok = m0 < n && m1 < n;
    }
    m0 += a.shift;
    m1 += a.shift;
    m0 = m0 >= n ? m0 - n : m0;
    m1 = m1 >= n ? m1 - n : m1;
    s_rowoff[e] = ok ? ((int64_t)m0 * n + m1) * n : -1;
  }
  for (int e = tid; e < T; e += blockDim.x) {
    int m2 = ts2 + e;
    bool ok = true;
    if (KT == COV3D_KERNEL_ES) {
      m2 = m2 >= n ? m2 - n : m2;
    } else {
      ok = m2 < n;
    }
    m2 += a.shift;
    m2 = m2 >= n ? m2 - n : m2;
    s_coloff[e] = ok ? m2 : -1;
  }
  __syncthreads();
  for (int e = tid; e < TILE4; e += blockDim.x) {
    const int qq = e % CP;
    const int cell = e / CP;
    const int cc = cell % T, rowi = cell / T;
    const long long ro = s_rowoff[rowi];
    const int co = s_coloff[cc];
    if (ro < 0 || co < 0) continue;
    float4 x = hi[e];
    if (COMP) {
      const float4 c = lo[e];
      x.x += c.x;
      x.y += c.y;
      x.z += c.z;
      x.w += c.w;
    }
    float2 *dst = a.grid + (ro + co) * a.cs + (int64_t)(a.ch0 + 2 * qq) * a.chs;
    if (2 * qq < a.nch && (x.x != 0.0f || x.y != 0.0f)) atomicAdd(dst, make_float2(x.x, x.y));
    if (2 * qq + 1 < a.nch && (x.z != 0.0f || x.w != 0.0f)) atomicAdd(dst + a.chs, make_float2(x.z, x.w));
  }
}

template <int KT, int W, int CP, bool COMP>
int launch_one(const SpreadParams &a, int64_t max_blocks, cudaStream_t st) {
  constexpr int T = kBin + W - 1;
  const size_t smem = (size_t)(COMP ? 2 : 1) * T * T * T * CP * sizeof(float4) +
                      (size_t)a.max_sub * (CP * sizeof(float4) + PointRec<W>::FLOATS * 4 + 2 * sizeof(int)) +
                      (2 * kBin + 1) * sizeof(int);
  if (smem > 227 * 1024) {
    set_error("spreading tile of %zu bytes exceeds shared memory", smem);
    return COV3D_EINVAL;
  }
  if (smem > 32 * 1024) {  // static shared arrays come on top of the dynamic size
    cudaError_t e = cudaFuncSetAttribute(spread_kernel<KT, W, CP, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(spread_kernel)");
  }
  spread_kernel<KT, W, CP, COMP><<<(unsigned)max_blocks, kSpreadWarps * 32, smem, st>>>(a);
  return launched("spread_kernel");
}

template <int KT, int W, bool COMP>
int launch_wc(SpreadParams a, int nchan, int64_t max_blocks, cudaStream_t st) {
  constexpr int CPMAX = SpreadCP<W, COMP>::value;
  int done = 0;
  while (done < nchan) {
    const int left = nchan - done;
    a.ch0 = done;
    int s = COV3D_OK, ch = 0;
    if (left >= 2 * CPMAX || left > 4) {
      ch = left < 2 * CPMAX ? left : 2 * CPMAX;
      a.nch = ch;
      s = launch_one<KT, W, CPMAX, COMP>(a, max_blocks, st);
    } else if (left > 2) {
      ch = left;
      a.nch = ch;
      s = launch_one<KT, W, (CPMAX > 2 ? 2 : CPMAX), COMP>(a, max_blocks, st);
      if (CPMAX < 2) ch = 2 * CPMAX;
    } else {
      ch = left;
      a.nch = ch;
      s = launch_one<KT, W, 1, COMP>(a, max_blocks, st);
    }
    if (s != COV3D_OK) return s;
    done += ch;
  }
  return COV3D_OK;
}

template <int KT, int W>
int launch_w(SpreadParams a, int nchan, bool comp, int64_t max_blocks, cudaStream_t st) {
  return comp ? launch_wc<KT, W, true>(a, nchan, max_blocks, st) : launch_wc<KT, W, false>(a, nchan, max_blocks, st);
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

// Tile planes (axis-0 index a of the bin + halo tile) per warp.  Plane a is reached by the
// points whose axis-0 window corner lies in [a - W + 1, a] (clipped to the bin): planes are
// assigned greedily, heaviest first, to the least loaded warp, so all warps get equal work.
int build_plane_schedule(cov3d_plan *p) {
  const int W = p->kernel == COV3D_KERNEL_NEAREST ? 1 : p->kernel == COV3D_KERNEL_LINEAR ? 2 : p->width;
  const int T = kBin + W - 1;
  std::vector<int> order(T), load(kSpreadWarps, 0), count(kSpreadWarps, 0);
  std::vector<int> sched(kSpreadWarps * kPlanesPerWarp, -1);
  auto reach = [&](int x) {
    const int lo = x - W + 1 > 0 ? x - W + 1 : 0;
    const int hi = x < kBin - 1 ? x : kBin - 1;
    return hi >= lo ? hi - lo + 1 : 0;
  };
  for (int i = 0; i < T; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return reach(x) > reach(y); });
  for (int pa : order) {
    int best = -1;
    for (int w = 0; w < kSpreadWarps; ++w)
      if (count[w] < kPlanesPerWarp && (best < 0 || load[w] < load[best])) best = w;
    if (best < 0) {
      set_error("cannot schedule %d tile planes", T);
      return COV3D_EINVAL;
    }
    sched[best * kPlanesPerWarp + count[best]++] = pa;
    load[best] += reach(pa);
  }
  COV3D_TRY(grow(p->row_order, (int64_t)sched.size() * 4));
  return check_cuda(cudaMemcpy(p->row_order.ptr, sched.data(), sched.size() * 4, cudaMemcpyHostToDevice),
                    "cudaMemcpy(plane schedule)");
}

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
  a.pts = p->sorted.as<SortedPoint>();
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
  a.max_sub = p->max_sub;
  a.plane_sched = p->row_order.as<int>();
  if (p->bins.bs[0] != kBin || p->bins.bs[1] != kBin || p->bins.bs[2] != kBin) {
    set_error("spreading requires %d^3-cell bins", kBin);
    return COV3D_EINVAL;
  }
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
