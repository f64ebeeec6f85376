// Spreading ("type-1" half of the NUFFT; exact adjoint of interp.cu, replacing the
// reference's grid_sample backward with FP32 global atomics, nufft_plan.py:171-242).
//
// One thread block per subproblem (<= max_sub points of one 8^3-cell spatial bin), no
// shared-memory atomics on the data path:
//  1. the block counting-sorts its points by their (axis-0, axis-1) window corner inside the
//     bin (64 columns) and stores, per point, its axis-0/1 kernel weights, its axis-2 weights
//     expanded over the tile row, and its CH channel values (times the im_backward prologue:
//     CTF, Nyquist zeroing, scale);
//  2. every thread owns one axis-2 row of the tile (bin + (W-1)-cell halo) and accumulates, in
//     registers, every point whose window covers that row -- the points of the W x W columns
//     around it, walked as one flattened list -- over the whole row; with COMP each register
//     accumulator is Kahan-compensated;
//  3. the tile is added to the global grid once, one complex atomic per cell and channel.
#include <algorithm>
#include <vector>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

constexpr int kBin = 8;           // bin edge (cells); plans use 8^3 bins
constexpr int kSpreadThreads = 256;

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
  const float *ctf;
  int nyquist;
  float scale;
  float2 *grid;
  int64_t cs, chs;
  int shift;
  int max_sub;
  const int *row_order;  // tile rows (a << 8 | b) in decreasing order of work
};

// Prologue factor of im_backward: CTF multiply, Nyquist zeroing, scale (projection_funcs.py:385-399).
__device__ __forceinline__ float prologue(const PointGeom &g, int64_t id, const float *ctf, int nyquist, float scale) {
  float sc = scale;
  if (nyquist && on_nyquist(g, id)) sc = 0.0f;
  if (ctf) sc *= __ldg(ctf + id);
  return sc;
}

template <int W, int CH>
struct RowLayout {
  static constexpr int T = kBin + W - 1;             // tile edge
  static constexpr int T4 = (T + 3) / 4 * 4;         // axis-2 weights padded to float4
  static constexpr int V = 2 * CH;                   // channel values (re, im)
  static constexpr int V4 = (V + 3) / 4 * 4;
  static constexpr int W0 = T4 + V4;                 // axis-0 weights
  static constexpr int W1 = W0 + W;                  // axis-1 weights
  static constexpr int S4 = (W1 + W + 3) / 4;        // float4 groups per record, made odd so that
  static constexpr int STRIDE = 4 * (S4 % 2 ? S4 : S4 + 1);  // records of different points start on
                                                              // different bank groups
};

// Number of bin columns along one axis whose window reaches tile row coordinate x.
template <int W>
__device__ constexpr int reach(int x) {
  const int lo = x - W + 1 > 0 ? x - W + 1 : 0;
  const int hi = x < kBin - 1 ? x : kBin - 1;
  return hi >= lo ? hi - lo + 1 : 0;
}

template <int KT, int W, int CH>
__device__ __forceinline__ void local_corner(const SpreadParams &a, float t, int ts, int &l, float *wt) {
  int c0 = taps<KT, W>(t, a.k.beta, wt);
  if (KT == COV3D_KERNEL_ES) c0 = pmod(c0, a.g.n);
  l = c0 - ts;
}

template <int KT, int W>
__device__ __forceinline__ int local_first(const SpreadParams &a, float t, int ts) {
  int c0 = first_cell<KT, W>(t);
  if (KT == COV3D_KERNEL_ES) c0 = pmod(c0, a.g.n);
  return c0 - ts;
}

template <int KT, int W, int CH, bool COMP>
__global__ void __launch_bounds__(kSpreadThreads, 2) spread_kernel(const SpreadParams a) {
  using Lay = RowLayout<W, CH>;
  constexpr int T = Lay::T;
  extern __shared__ float4 smem4[];
  int *s_cnt = reinterpret_cast<int *>(smem4);     // kBin*kBin
  int *s_off = s_cnt + kBin * kBin;                 // kBin*kBin + 1 (+3 pad)
  int *s_col = s_off + kBin * kBin + 4;             // max_sub
  int *s_rank = s_col + a.max_sub;                  // max_sub
  float *s_rec = reinterpret_cast<float *>(s_rank + a.max_sub);  // max_sub * STRIDE

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

  for (int i = tid; i < kBin * kBin; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  // 1a. column of every point (window corner on axes 0, 1 inside the bin) and its rank
  for (int k = tid; k < cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[first + k];
    const int l0 = local_first<KT, W>(a, sp.t0, ts0);
    const int l1 = local_first<KT, W>(a, sp.t1, ts1);
    const int col = max(l0, 0) * kBin + max(l1, 0);
    s_col[k] = col;
    s_rank[k] = atomicAdd(s_cnt + col, 1);
  }
  __syncthreads();
  if (tid == 0) {
    int acc = 0;
    for (int i = 0; i < kBin * kBin; ++i) {
      s_off[i] = acc;
      acc += s_cnt[i];
    }
    s_off[kBin * kBin] = acc;
  }
  __syncthreads();
  // 1b. point records in column order
  for (int k = tid; k < cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[first + k];
    const int64_t id = sp_id(sp.idf);
    float w0[W], w1[W], w2[W];
    int l0, l1, l2;
    local_corner<KT, W, CH>(a, sp.t0, ts0, l0, w0);
    local_corner<KT, W, CH>(a, sp.t1, ts1, l1, w1);
    local_corner<KT, W, CH>(a, sp.t2, ts2, l2, w2);
    float *rec = s_rec + (s_off[s_col[k]] + s_rank[k]) * Lay::STRIDE;
    float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
    if (a.ctf) sc *= __ldg(a.ctf + id);
#pragma unroll
    for (int c = 0; c < Lay::T4; ++c) rec[c] = 0.0f;
#pragma unroll
    for (int j = 0; j < W; ++j) {
      const int c = l2 + j;
      if (c >= 0 && c < T) rec[c] = w2[j];
    }
    const float2 *src = a.vals + id * a.ips + (int64_t)a.ch0 * a.ics;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const float2 x = sc != 0.0f ? __ldg(src + c * a.ics) : make_float2(0.f, 0.f);
      rec[Lay::T4 + 2 * c] = x.x * sc;
      rec[Lay::T4 + 2 * c + 1] = x.y * sc;
    }
    // zero padding (grid_sample kernels): window cells below the grid were clamped into bin 0;
    // shift their weights so that index (row - corner) still addresses the right tap
    const int s0 = max(-l0, 0), s1 = max(-l1, 0);
#pragma unroll
    for (int j = 0; j < W; ++j) {
      rec[Lay::W0 + j] = 0.0f;
      rec[Lay::W1 + j] = 0.0f;
    }
#pragma unroll
    for (int j = 0; j < W; ++j) {
      if (j >= s0) rec[Lay::W0 + j - s0] = w0[j];
      if (j >= s1) rec[Lay::W1 + j - s1] = w1[j];
    }
  }
  __syncthreads();

  // 2. one axis-2 row of the tile per thread.  The thread walks the points of the W x W
  //    columns around its row as one flattened list, so the lanes of a warp stay converged
  //    (their totals differ far less than their per-column counts).  Rows are handed out in
  //    decreasing order of the number of columns that reach them (halo rows see fewer), so
  //    the rows of one warp carry similar work.
  if (tid >= T * T) return;
  const int packed = __ldg(a.row_order + tid);
  const int ra = packed >> 8, rb = packed & 255;
  float2 acc[T][CH];
  float2 cmp[COMP ? T : 1][COMP ? CH : 1];
#pragma unroll
  for (int c = 0; c < T; ++c)
#pragma unroll
    for (int h = 0; h < CH; ++h) {
      acc[c][h] = make_float2(0.f, 0.f);
      if (COMP) cmp[COMP ? c : 0][COMP ? h : 0] = make_float2(0.f, 0.f);
    }
  int next = 0, p = 0, pend = 0, o0 = 0, o1 = 0;
  while (true) {
    while (p >= pend && next < W * W) {
      const int d0 = next / W, d1 = next - (next / W) * W;
      ++next;
      const int l0 = ra - d0, l1 = rb - d1;
      if (l0 < 0 || l0 >= kBin || l1 < 0 || l1 >= kBin) continue;
      p = s_off[l0 * kBin + l1];
      pend = s_off[l0 * kBin + l1 + 1];
      o0 = d0;
      o1 = d1;
    }
    if (p >= pend) break;
    const float *rec = s_rec + p * Lay::STRIDE;
    ++p;
    const float wab = rec[Lay::W0 + o0] * rec[Lay::W1 + o1];
    float w2[Lay::T4];
#pragma unroll
    for (int q = 0; q < Lay::T4 / 4; ++q) {
      const float4 x = reinterpret_cast<const float4 *>(rec)[q];
      w2[4 * q] = x.x;
      w2[4 * q + 1] = x.y;
      w2[4 * q + 2] = x.z;
      w2[4 * q + 3] = x.w;
    }
    float v[Lay::V4];
#pragma unroll
    for (int q = 0; q < Lay::V4 / 4; ++q) {
      const float4 x = reinterpret_cast<const float4 *>(rec + Lay::T4)[q];
      v[4 * q] = x.x;
      v[4 * q + 1] = x.y;
      v[4 * q + 2] = x.z;
      v[4 * q + 3] = x.w;
    }
#pragma unroll
    for (int c = 0; c < T; ++c) {
      const float w = wab * w2[c];
#pragma unroll
      for (int h = 0; h < CH; ++h) {
        if (!COMP) {
          acc[c][h].x = fmaf(w, v[2 * h], acc[c][h].x);
          acc[c][h].y = fmaf(w, v[2 * h + 1], acc[c][h].y);
        } else {
          float y = w * v[2 * h] - cmp[COMP ? c : 0][COMP ? h : 0].x;
          float t2 = acc[c][h].x + y;
          cmp[COMP ? c : 0][COMP ? h : 0].x = (t2 - acc[c][h].x) - y;
          acc[c][h].x = t2;
          y = w * v[2 * h + 1] - cmp[COMP ? c : 0][COMP ? h : 0].y;
          t2 = acc[c][h].y + y;
          cmp[COMP ? c : 0][COMP ? h : 0].y = (t2 - acc[c][h].y) - y;
          acc[c][h].y = t2;
        }
      }
    }
  }

  // 3. add the row to the global grid
  int m0 = ts0 + ra, m1 = ts1 + rb;
  if (KT == COV3D_KERNEL_ES) {
    m0 = m0 >= n ? m0 - n : m0;
    m1 = m1 >= n ? m1 - n : m1;
  } else if (m0 >= n || m1 >= n) {
    return;
  }
  m0 += a.shift;
  m1 += a.shift;
  m0 = m0 >= n ? m0 - n : m0;
  m1 = m1 >= n ? m1 - n : m1;
  const int64_t row = ((int64_t)m0 * n + m1) * n;
#pragma unroll
  for (int c = 0; c < T; ++c) {
    int m2 = ts2 + c;
    if (KT == COV3D_KERNEL_ES) {
      m2 = m2 >= n ? m2 - n : m2;
    } else if (m2 >= n) {
      continue;
    }
    m2 += a.shift;
    m2 = m2 >= n ? m2 - n : m2;
    float2 *dst = a.grid + (row + m2) * a.cs + (int64_t)a.ch0 * a.chs;
#pragma unroll
    for (int h = 0; h < CH; ++h) {
      float2 val = acc[c][h];
      if (COMP) {
        val.x -= cmp[COMP ? c : 0][COMP ? h : 0].x;
        val.y -= cmp[COMP ? c : 0][COMP ? h : 0].y;
      }
      if (val.x != 0.0f || val.y != 0.0f) atomicAdd(dst + h * a.chs, val);
    }
  }
}

template <int KT, int W, int CH, bool COMP>
size_t smem_bytes(int max_sub) {
  return (size_t)(2 * kBin * kBin + 8 + 2 * max_sub) * sizeof(int) +
         (size_t)max_sub * RowLayout<W, CH>::STRIDE * sizeof(float);
}

template <int KT, int W, int CH, bool COMP>
int launch_one(const SpreadParams &a, int64_t max_blocks, cudaStream_t st) {
  const size_t smem = smem_bytes<KT, W, CH, COMP>(a.max_sub);
  if (smem > 200 * 1024) {
    set_error("spread tile records of %zu bytes exceed shared memory", smem);
    return COV3D_EINVAL;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(spread_kernel<KT, W, CH, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(spread_kernel)");
  }
  spread_kernel<KT, W, CH, COMP><<<(unsigned)max_blocks, kSpreadThreads, smem, st>>>(a);
  return launched("spread_kernel");
}

template <int KT, int W>
int launch_w(SpreadParams a, int nchan, bool comp, int64_t max_blocks, cudaStream_t st) {
  int done = 0;
  while (done < nchan) {
    const int left = nchan - done;
    a.ch0 = done;
    int s = COV3D_OK, ch = 1;
    if (comp) {
      ch = 1;
      s = launch_one<KT, W, 1, true>(a, max_blocks, st);
    } else {
      ch = left >= 2 ? 2 : 1;
      s = ch == 2 ? launch_one<KT, W, 2, false>(a, max_blocks, st) : launch_one<KT, W, 1, false>(a, max_blocks, st);
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

int build_row_order(cov3d_plan *p) {
  const int W = p->kernel == COV3D_KERNEL_NEAREST ? 1 : p->kernel == COV3D_KERNEL_LINEAR ? 2 : p->width;
  const int T = kBin + W - 1;
  auto reach_h = [&](int x) {
    const int lo = x - W + 1 > 0 ? x - W + 1 : 0;
    const int hi = x < kBin - 1 ? x : kBin - 1;
    return hi >= lo ? hi - lo + 1 : 0;
  };
  std::vector<int> rows(T * T);
  for (int q = 0; q < T * T; ++q) rows[q] = q;
  std::stable_sort(rows.begin(), rows.end(), [&](int x, int y) {
    return reach_h(x / T) * reach_h(x % T) > reach_h(y / T) * reach_h(y % T);
  });
  std::vector<int> packed(T * T);
  for (int i = 0; i < T * T; ++i) packed[i] = ((rows[i] / T) << 8) | (rows[i] % T);
  COV3D_TRY(grow(p->row_order, (int64_t)packed.size() * 4));
  return check_cuda(cudaMemcpy(p->row_order.ptr, packed.data(), packed.size() * 4, cudaMemcpyHostToDevice),
                    "cudaMemcpy(row_order)");
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
  a.row_order = p->row_order.as<int>();
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
