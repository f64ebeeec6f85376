// Spreading ("type-1" half of the NUFFT; exact adjoint of interp.cu, replacing the
// reference's grid_sample backward with FP32 global atomics, nufft_plan.py:171-242), over the
// bin-sorted point records of points_sort.cu.  See spread_kernel for the decomposition.
#include <algorithm>
#include <vector>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

constexpr int kBin = 8;
constexpr int kSpreadWarps = 16;
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
  const int *plane_sched;  // kSpreadWarps x kPlanesPerWarp tasks 2 * plane + row parity (-1 = none)
};

// Prologue factor of im_backward: CTF multiply, Nyquist zeroing, scale (projection_funcs.py:385-399).
__device__ __forceinline__ float prologue(const PointGeom &g, int64_t id, const float *ctf, int nyquist, float scale) {
  float sc = scale;
  if (nyquist && on_nyquist(g, id)) sc = 0.0f;
  if (ctf) sc *= __ldg(ctf + id);
  return sc;
}

// Channel pairs per pass: lanes are (tile column, channel pair), so T * CP <= 32 with
// T = 8 + W - 1 tile columns; COMP keeps a second (compensation) tile, which leaves room for
// only one pair at W = 8.
template <int W, bool COMP>
struct SpreadCP {
  static constexpr int T = 8 + W - 1;
  static constexpr int value = (COMP && W == 8) ? 1 : 32 / T;
};

constexpr int kLMin = -8;     // window corners relative to the bin lie in [kLMin, kLMin + 16)
constexpr int kKeys = 256;    // sort key (l1 - kLMin) * 16 + (l0 - kLMin)

// Per-point record staged once per block: packed window corner (tile-local, biased by 32 so
// zero-padding corners below the tile stay non-negative) and the 3W kernel weights.
template <int W>
struct PointRec {
  static constexpr int FLOATS = (1 + 3 * W + 3) / 4 * 4;
};

// One block per subproblem, tile = bin + (W-1)-cell halo of 2*CP channels in shared memory.
//  1. the block counting-sorts its points by the (axis-1, axis-0) corner (l1, l0) of their
//     window and stages, in that order, each point's record (packed corner, 3W weights) and
//     CTF-scaled values;
//  2. each warp owns (plane, row parity) tasks: a whole axis-0 plane of the tile, and within it
//     the tile rows of one parity (plane_sched balances the work over the 16 warps).  Lane
//     (q, c) owns tile column c and channel pair q.  For a plane the points with a given l1 and
//     an l0 that reaches the plane are one contiguous range; all of them hit rows l1 .. l1+W-1,
//     so the lane accumulates weight * value for its column and its rows in registers and adds
//     the sums to the tile once per range -- conflict-free 16-byte read-modify-writes, and no
//     two warps ever touch the same cell, so there are no atomics.  With COMP that addition is
//     a TwoSum whose rounding error goes to the second tile (the register sums of a range carry
//     only the rounding of their own terms);
//  3. the tile is added to the global grid, one complex atomic per cell and channel.
template <int KT, int W, int CP, bool COMP>
__global__ void __launch_bounds__(kSpreadWarps * 32) spread_kernel(const SpreadParams a) {
  constexpr int T = kBin + W - 1;
  static_assert(T * CP <= 32, "one lane per tile column and channel pair");
  constexpr int TILE4 = T * T * T * CP;
  constexpr int NR = (W + 1) / 2;  // window rows of one parity, at most
  extern __shared__ float4 smem4[];
  float4 *hi = smem4;
  float4 *lo = smem4 + (COMP ? TILE4 : 0);
  float4 *s_val = smem4 + (COMP ? 2 : 1) * TILE4;  // max_sub * CP, sorted order
  float *s_rec = reinterpret_cast<float *>(s_val + a.max_sub * CP);  // max_sub * PointRec<W>::FLOATS
  int *s_key = reinterpret_cast<int *>(s_rec + a.max_sub * PointRec<W>::FLOATS);  // max_sub
  int *s_cnt = s_key + a.max_sub;  // kKeys
  int *s_off = s_cnt + kKeys;      // kKeys + 1

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
  for (int e = tid; e < kKeys; e += blockDim.x) s_cnt[e] = 0;
  __syncthreads();
  // 1a. sort keys and ranks
  for (int k = tid; k < cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[first + k];
    int c0 = first_cell<KT, W>(sp.t0), c1 = first_cell<KT, W>(sp.t1);
    if (KT == COV3D_KERNEL_ES) {
      c0 = wrap1(c0, n);
      c1 = wrap1(c1, n);
    }
    const int key = (min(max(c1 - ts1 - kLMin, 0), 15) << 4) | min(max(c0 - ts0 - kLMin, 0), 15);
    s_key[k] = key | (atomicAdd(s_cnt + key, 1) << 8);
  }
  __syncthreads();
  if (tid < 32) {  // exclusive scan of the 256 counters by one warp, 8 per lane
    int v[kKeys / 32], sum = 0;
#pragma unroll
    for (int u = 0; u < kKeys / 32; ++u) {
      v[u] = s_cnt[tid * (kKeys / 32) + u];
      sum += v[u];
    }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (tid >= o) incl += t;
    }
    int base = incl - sum;
#pragma unroll
    for (int u = 0; u < kKeys / 32; ++u) {
      s_off[tid * (kKeys / 32) + u] = base;
      base += v[u];
    }
    if (tid == 31) s_off[kKeys] = incl;
  }
  __syncthreads();
  // 1b. records and scaled values (im_backward prologue folded in) in sorted order
  for (int k = tid; k < cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[first + k];
    const int kr = s_key[k];
    const int slot = s_off[kr & 255] + (kr >> 8);
    float w0[W], w1[W], w2[W];
    int c0 = taps<KT, W>(sp.t0, a.k.beta, w0);
    int c1 = taps<KT, W>(sp.t1, a.k.beta, w1);
    int c2 = taps<KT, W>(sp.t2, a.k.beta, w2);
    if (KT == COV3D_KERNEL_ES) {
      c0 = wrap1(c0, n);
      c1 = wrap1(c1, n);
      c2 = wrap1(c2, n);
    }
    float *rec = s_rec + slot * PointRec<W>::FLOATS;
    rec[0] = __int_as_float((c0 - ts0 + 32) | ((c1 - ts1 + 32) << 8) | ((c2 - ts2 + 32) << 16));
#pragma unroll
    for (int r = 0; r < W; ++r) {
      rec[1 + r] = w0[r];
      rec[1 + W + r] = w1[r];
      rec[1 + 2 * W + r] = w2[r];
    }
    const int64_t id = sp_id(sp.idf);
    float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
    if (a.ctf) sc *= __ldg(a.ctf + id);
#pragma unroll
    for (int qq = 0; qq < CP; ++qq) {
      const float2 *src = a.vals + id * a.ips + (int64_t)(a.ch0 + 2 * qq) * a.ics;
      const float2 v0 = 2 * qq < a.nch ? __ldg(src) : make_float2(0.f, 0.f);
      const float2 v1 = 2 * qq + 1 < a.nch ? __ldg(src + a.ics) : make_float2(0.f, 0.f);
      s_val[slot * CP + qq] = make_float4(v0.x * sc, v0.y * sc, v1.x * sc, v1.y * sc);
    }
  }
  __syncthreads();

  // 2. tasks of this warp; lane (q, c): channel pair q, tile column c
  const int warp = tid >> 5, lane = tid & 31;
  const int q = lane / T, c = lane - (lane / T) * T;
  const bool lane_live = q < CP;
  const int qv = lane_live ? q : 0;
  for (int s = 0; s < kPlanesPerWarp; ++s) {
    const int task = __ldg(a.plane_sched + warp * kPlanesPerWarp + s);
    if (task < 0) break;
    const int pa = task >> 1, par = task & 1;
    // corners l0 reaching plane pa: [pa - W + 1, pa]
    const int b0lo = max(pa - W + 1 - kLMin, 0), b0hi = min(pa - kLMin, 15);
    if (b0lo > b0hi) continue;
    for (int b1 = 0; b1 < 16; ++b1) {
      const int ibeg = s_off[(b1 << 4) | b0lo], iend = s_off[((b1 << 4) | b0hi) + 1];
      if (ibeg >= iend) continue;
      const int l1 = b1 + kLMin;
      const int r0 = (par - l1) & 1;  // first window row whose tile row has parity par
      float4 acc[NR];
#pragma unroll
      for (int u = 0; u < NR; ++u) acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      bool touched = false;
      for (int i = ibeg; i < iend; ++i) {
        const float *rec = s_rec + i * PointRec<W>::FLOATS;
        const int packed = __float_as_int(rec[0]);
        const int o0 = pa - ((packed & 255) - 32);  // in [0, W) by the range above
        const int jj = c - (((packed >> 16) & 255) - 32);
        if (!lane_live || jj < 0 || jj >= W) continue;
        touched = true;
        const float w02 = rec[1 + o0] * rec[1 + 2 * W + jj];
        const float4 vv = s_val[i * CP + qv];
#pragma unroll
        for (int u = 0; u < NR; ++u) {
          const int r = r0 + 2 * u;
          if (r < W) {
            const float w = w02 * rec[1 + W + r];
            acc[u].x = fmaf(w, vv.x, acc[u].x);
            acc[u].y = fmaf(w, vv.y, acc[u].y);
            acc[u].z = fmaf(w, vv.z, acc[u].z);
            acc[u].w = fmaf(w, vv.w, acc[u].w);
          }
        }
      }
      if (!touched) continue;
#pragma unroll
      for (int u = 0; u < NR; ++u) {
        const int r = r0 + 2 * u;
        const int r1 = l1 + r;
        if (r >= W || (KT != COV3D_KERNEL_ES && r1 < 0)) continue;
        const int e = ((pa * T + r1) * T + c) * CP + q;
        if (!COMP) {
          float4 x = hi[e];
          x.x += acc[u].x;
          x.y += acc[u].y;
          x.z += acc[u].z;
          x.w += acc[u].w;
          hi[e] = x;
        } else {
          float4 x = hi[e], err = lo[e];
          const float d[4] = {acc[u].x, acc[u].y, acc[u].z, acc[u].w};
          float *xs = &x.x, *es = &err.x;
#pragma unroll
          for (int v = 0; v < 4; ++v) {  // TwoSum (Knuth): xs + d = s2 + rounding error, exactly
            const float s2 = xs[v] + d[v];
            const float bb = s2 - xs[v];
            es[v] += (xs[v] - (s2 - bb)) + (d[v] - bb);
            xs[v] = s2;
          }
          hi[e] = x;
          lo[e] = err;
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
                      (size_t)a.max_sub * (CP * sizeof(float4) + PointRec<W>::FLOATS * 4 + sizeof(int)) +
                      (2 * kKeys + 1) * sizeof(int);
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

// Warp tasks: (tile plane a, row parity) pairs, encoded 2 * a + parity.  Plane a is reached by
// the points whose axis-0 window corner lies in [a - W + 1, a] (clipped to the bin), and a
// parity holds about half of each window's rows: tasks are assigned greedily, heaviest first,
// to the least loaded warp, so all warps get equal work.
int build_plane_schedule(cov3d_plan *p) {
  const int W = p->kernel == COV3D_KERNEL_NEAREST ? 1 : p->kernel == COV3D_KERNEL_LINEAR ? 2 : p->width;
  const int T = kBin + W - 1;
  std::vector<int> order(2 * T), load(kSpreadWarps, 0), count(kSpreadWarps, 0);
  std::vector<int> sched(kSpreadWarps * kPlanesPerWarp, -1);
  auto work = [&](int task) {
    const int x = task >> 1;
    const int lo = x - W + 1 > 0 ? x - W + 1 : 0;
    const int hi = x < kBin - 1 ? x : kBin - 1;
    const int rows = (task & 1) ? W / 2 : (W + 1) / 2;
    return hi >= lo ? (hi - lo + 1) * rows : 0;
  };
  for (int i = 0; i < 2 * T; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work(x) > work(y); });
  for (int task : order) {
    int best = -1;
    for (int w = 0; w < kSpreadWarps; ++w)
      if (count[w] < kPlanesPerWarp && (best < 0 || load[w] < load[best])) best = w;
    if (best < 0) {
      set_error("cannot schedule %d tile planes", T);
      return COV3D_EINVAL;
    }
    sched[best * kPlanesPerWarp + count[best]++] = task;
    load[best] += work(task);
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
