// Spreading ("type-1" half of the NUFFT; exact adjoint of interp.cu, replacing the
// reference's grid_sample backward with FP32 global atomics, nufft_plan.py:171-242), over the
// bin-sorted point records of points_sort.cu.  See spread_kernel for the decomposition.

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

constexpr int kBin = 8;
constexpr int kSpreadWarps = 16;

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
  int nch;  // channels of this launch
  const float *ctf;
  int nyquist;
  float scale;
  float2 *grid;
  int64_t cs, chs;
  int shift;
  int max_sub;
};

// Prologue factor of im_backward: CTF multiply, Nyquist zeroing, scale (projection_funcs.py:385-399).
__device__ __forceinline__ float prologue(const PointGeom &g, int64_t id, const float *ctf, int nyquist, float scale) {
  float sc = scale;
  if (nyquist && on_nyquist(g, id)) sc = 0.0f;
  if (ctf) sc *= __ldg(ctf + id);
  return sc;
}

constexpr int kLMin = -8;   // window corners relative to the bin lie in [kLMin, kLMin + 16)
constexpr int kKeys = 256;  // sort key (l1 - kLMin) * 16 + (l0 - kLMin)
constexpr int kMaxCPL = 3;      // channel pairs per lane per group (row tasks)
constexpr int kRowPairCPL = 5;  // channel pairs per lane per group (row-pair tasks)
constexpr int kFoldRanges = 2;  // window-corner rows l1 summed in FP32 between compensated folds

// Per-point record staged once per block, in float2 units (each weight twice, the operand of a
// packed multiply): the axis-0 weights by tile plane and the axis-2 weights by tile column, zero
// outside the point's window, and the W axis-1 weights followed by a zero.  A lane's weight is
// then rec[plane] * rec[W1 + o1] * rec[W2 + column], with no corner arithmetic and no select:
// lanes outside the window read zeros.
template <int W>
struct PointRec {
  static constexpr int T = kBin + W - 1;
  static constexpr int W1 = T;              // axis-1 weights, then the zero slot W1 + W
  static constexpr int W2 = T + W + 1;      // axis-2 weights by column
  static constexpr int F2 = (2 * T + W + 2) / 2 * 2;  // float2 per record (even)
};

// TwoSum (Knuth) on both lanes of a float2: s + d = s' + e exactly, e added to the error sum
// err.  Differences are fused multiply-adds with -1, which round exactly like a subtraction.
__device__ __forceinline__ void two_sum2(float2 &s, float2 &err, const float2 d) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  const float2 s2 = __fadd2_rn(s, d);
  const float2 bb = __ffma2_rn(s, m1, s2);   // s2 - s
  const float2 sb = __ffma2_rn(bb, m1, s2);  // s2 - bb
  const float2 e1 = __ffma2_rn(sb, m1, s);   // s - (s2 - bb)
  const float2 e2 = __ffma2_rn(bb, m1, d);   // d - bb
  err = __fadd2_rn(err, __fadd2_rn(e1, e2));
  s = s2;
}

// Lane layout of the row tasks: lane = g * T + c owns tile column c (T = 8 + W - 1 columns)
// and the channel pairs g, g + G, ..., G = 32 / T lane groups.
template <int W>
struct SpreadLanes {
  static constexpr int T = kBin + W - 1;
  static constexpr int G = 32 / T;
};

template <int W>
__host__ __device__ constexpr int spread_pairs(int cpl) { return SpreadLanes<W>::G * cpl; }

// One block per subproblem (a bin of 8^3 cells and at most max_sub of its points); the cells
// it can reach form a tile of the bin and a (W-1)-cell halo, T^3 cells.
//  1. the block counting-sorts its points by the (axis-1, axis-0) corner (l1, l0) of their
//     window and stages, in that order, each point's record (packed corner, 3W weights) and
//     its CTF-scaled channel pairs (im_backward's prologue folded in);
//  2. a task is one tile row: plane a, row b.  The points whose window covers it are the W
//     contiguous ranges {l1 = b - o1, l0 in [a - W + 1, a]}, o1 = 0 .. W-1, of the sorted
//     order.  Lane (g, c) keeps the sums of cell (a, b, c) for its channel pairs in registers:
//     each group of kFoldRanges ranges is summed in FP32 and, with COMP, added to the cell's
//     (hi, lo) pair by a TwoSum, so the error of the cell's accumulation is that of one short
//     FP32 sum per group.
//     The finished row goes to the global grid with one complex atomic per cell and channel.
//     Warps take tasks from a shared counter, so the heavy middle rows spread over all warps.
//  The block needs no shared-memory tile: its shared memory is the staged points only, and
//  several blocks share an SM.
template <int KT, int W, int CPL, bool COMP, bool RP>
__global__ void __launch_bounds__(kSpreadWarps * 32, RP ? 1 : 2) spread_kernel(const SpreadParams a) {
  constexpr int T = SpreadLanes<W>::T;
  constexpr int G = RP ? 1 : SpreadLanes<W>::G;  // lane groups over channel pairs
  constexpr int NP = G * CPL;                     // channel pairs staged per group
  constexpr int TP = (T + 1) / 2;                 // row pairs per plane (RP)
  static_assert(!RP || 2 * T <= 32, "two rows of lanes per warp");
  using Rec = PointRec<W>;
  constexpr int F2 = Rec::F2;
  extern __shared__ float4 smem4[];
  float4 *s_val = smem4;                                                         // max_sub * NP
  long long *s_rowoff = reinterpret_cast<long long *>(s_val + a.max_sub * NP);  // T * T
  float2 *s_rec = reinterpret_cast<float2 *>(s_rowoff + T * T);                // max_sub * F2
  int *s_key = reinterpret_cast<int *>(s_rec + a.max_sub * F2);                // max_sub
  int *s_pid = s_key + a.max_sub;                                              // max_sub
  float *s_sc = reinterpret_cast<float *>(s_pid + a.max_sub);                  // max_sub
  int *s_cnt = reinterpret_cast<int *>(s_sc + a.max_sub);                      // kKeys
  int *s_off = s_cnt + kKeys;                                                  // kKeys + 1
  int *s_coloff = s_off + kKeys + 1;                                           // T
  int *s_task = s_coloff + T;                                                  // 1

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
  // 1b. records, point ids and prologue factors in sorted order
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
    (void)c1;
    float2 *rec = s_rec + slot * F2;
    const int l0 = c0 - ts0, l2 = c2 - ts2;  // bin-local corners, >= 1 - W (zero padding below)
#pragma unroll
    for (int e = 0; e < T; ++e) {
      rec[e] = make_float2(0.f, 0.f);
      rec[Rec::W2 + e] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int r = 0; r < W; ++r) {
      if (l0 + r >= 0 && l0 + r < T) rec[l0 + r] = make_float2(w0[r], w0[r]);
      if (l2 + r >= 0 && l2 + r < T) rec[Rec::W2 + l2 + r] = make_float2(w2[r], w2[r]);
      rec[Rec::W1 + r] = make_float2(w1[r], w1[r]);
    }
    rec[Rec::W1 + W] = make_float2(0.f, 0.f);
    const int id = sp_id(sp.idf);
    float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
    if (a.ctf) sc *= __ldg(a.ctf + id);
    s_pid[slot] = id;
    s_sc[slot] = sc;
  }
  // global offsets of the tile's rows (axes 0, 1) and columns (axis 2)
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

  const int lane = tid & 31;
  // RP: lane = (row of the pair, column), every lane all NP pairs; else lane = (pair group, column)
  const int g = lane / T, c = lane - (lane / T) * T;
  const bool lane_live = RP ? g < 2 : g < G;
  const int gv = (RP || !lane_live) ? 0 : g;  // idle lanes compute pair 0 and drop it
  const int npairs = (a.nch + 1) / 2;
  for (int p0 = 0; p0 < npairs; p0 += NP) {  // channel groups of NP pairs
    __syncthreads();
    // 1c. this group's scaled channel pairs, in sorted order
    for (int e = tid; e < cnt * NP; e += blockDim.x) {
      const int slot = e / NP, pp = p0 + (e - (e / NP) * NP);
      const float sc = s_sc[slot];
      const float2 *src = a.vals + (int64_t)s_pid[slot] * a.ips + (int64_t)(a.ch0 + 2 * pp) * a.ics;
      const float2 v0 = 2 * pp < a.nch ? __ldg(src) : make_float2(0.f, 0.f);
      const float2 v1 = 2 * pp + 1 < a.nch ? __ldg(src + a.ics) : make_float2(0.f, 0.f);
      s_val[e] = make_float4(v0.x * sc, v0.y * sc, v1.x * sc, v1.y * sc);
    }
    if (tid == 0) *s_task = 0;
    __syncthreads();

    // 2. row tasks (RP: row-pair tasks)
    constexpr int ntasks = RP ? T * TP : T * T;
    for (;;) {
      int task = 0;
      if (lane == 0) task = atomicAdd(s_task, 1);
      task = __shfl_sync(0xffffffffu, task, 0);
      if (task >= ntasks) break;
      const int pa = RP ? task / TP : task / T;
      const int rb = RP ? (task - pa * TP) * 2 : task - pa * T;  // first row of the task
      const int r1 = RP ? rb + g : rb;                            // this lane's row
      const bool row_live = lane_live && r1 < T;
      const int b0lo = max(pa - W + 1 - kLMin, 0), b0hi = min(pa - kLMin, 15);
      // cell sums of channel pairs (0, 1) and (2, 3) of each pair group, and their TwoSum errors
      float2 hi01[CPL], hi23[CPL], lo01[CPL], lo23[CPL];
#pragma unroll
      for (int u = 0; u < CPL; ++u) {
        hi01[u] = hi23[u] = lo01[u] = lo23[u] = make_float2(0.f, 0.f);
      }
      bool any = false;
      const int lhi = RP ? rb + 1 : rb;
      const float2 *w2c = s_rec + Rec::W2 + c;  // this lane's column weight, record 0
      // points with window corner l1 cover row l1 + o1; the ranges of kFoldRanges consecutive
      // l1 are summed in FP32 before one compensated fold
      for (int l1g = lhi; l1g > rb - W; l1g -= kFoldRanges) {
        float2 part01[CPL], part23[CPL];  // packed FP32 (FFMA2), same rounding as fmaf
#pragma unroll
        for (int u = 0; u < CPL; ++u) {
          part01[u] = make_float2(0.f, 0.f);
          part23[u] = make_float2(0.f, 0.f);
        }
        bool in = false;
#pragma unroll
        for (int sr = 0; sr < kFoldRanges; ++sr) {
          const int l1 = l1g - sr;
          const int b1 = l1 - kLMin;
          if (l1 <= rb - W || b1 < 0 || b1 > 15 || b0lo > b0hi) continue;
          const int ibeg = s_off[(b1 << 4) | b0lo], iend = s_off[((b1 << 4) | b0hi) + 1];
          const int o1 = r1 - l1;
          const bool in1 = row_live && o1 >= 0 && o1 < W;
          in |= in1 && ibeg < iend;
          const int k1 = Rec::W1 + (in1 ? o1 : W);  // the zero slot for rows the range misses
          // two points per iteration; a lane whose column or row is outside a point's window
          // multiplies by a zero weight
          int i = ibeg;
          for (; i + 1 < iend; i += 2) {
            const float2 *ra = s_rec + i * F2, *rb2 = ra + F2;
            const float2 wa = __fmul2_rn(__fmul2_rn(ra[pa], ra[k1]), w2c[i * F2]);
            const float2 wb = __fmul2_rn(__fmul2_rn(rb2[pa], rb2[k1]), w2c[(i + 1) * F2]);
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
              const float4 xa = s_val[i * NP + gv + G * u];
              const float4 xb = s_val[(i + 1) * NP + gv + G * u];
              part01[u] = __ffma2_rn(wa, make_float2(xa.x, xa.y), part01[u]);
              part23[u] = __ffma2_rn(wa, make_float2(xa.z, xa.w), part23[u]);
              part01[u] = __ffma2_rn(wb, make_float2(xb.x, xb.y), part01[u]);
              part23[u] = __ffma2_rn(wb, make_float2(xb.z, xb.w), part23[u]);
            }
          }
          if (i < iend) {
            const float2 *ra = s_rec + i * F2;
            const float2 wa = __fmul2_rn(__fmul2_rn(ra[pa], ra[k1]), w2c[i * F2]);
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
              const float4 xa = s_val[i * NP + gv + G * u];
              part01[u] = __ffma2_rn(wa, make_float2(xa.x, xa.y), part01[u]);
              part23[u] = __ffma2_rn(wa, make_float2(xa.z, xa.w), part23[u]);
            }
          }
        }
        if (!in) continue;
        any = true;
#pragma unroll
        for (int u = 0; u < CPL; ++u) {
          if (!COMP) {
            hi01[u] = __fadd2_rn(hi01[u], part01[u]);
            hi23[u] = __fadd2_rn(hi23[u], part23[u]);
          } else {
            two_sum2(hi01[u], lo01[u], part01[u]);
            two_sum2(hi23[u], lo23[u], part23[u]);
          }
        }
      }
      // 3. the finished cell goes to the global grid
      if (!any || !row_live) continue;
      const long long ro = s_rowoff[pa * T + r1];
      const int co = s_coloff[c];
      if (ro < 0 || co < 0) continue;
#pragma unroll
      for (int u = 0; u < CPL; ++u) {
        const int pp = p0 + gv + G * u;
        const float2 x01 = COMP ? __fadd2_rn(hi01[u], lo01[u]) : hi01[u];
        const float2 x23 = COMP ? __fadd2_rn(hi23[u], lo23[u]) : hi23[u];
        float2 *dst = a.grid + (ro + co) * a.cs + (int64_t)(a.ch0 + 2 * pp) * a.chs;
        if (2 * pp < a.nch && (x01.x != 0.0f || x01.y != 0.0f)) atomicAdd(dst, x01);
        if (2 * pp + 1 < a.nch && (x23.x != 0.0f || x23.y != 0.0f)) atomicAdd(dst + a.chs, x23);
      }
    }
  }
}

template <int KT, int W, int CPL, bool COMP, bool RP>
int launch_one(const SpreadParams &a, int64_t max_blocks, cudaStream_t st) {
  constexpr int T = SpreadLanes<W>::T;
  constexpr int NP = (RP ? 1 : SpreadLanes<W>::G) * CPL;
  const size_t smem = (size_t)a.max_sub * (NP * sizeof(float4) + PointRec<W>::F2 * sizeof(float2) + 3 * sizeof(int)) +
                      (size_t)T * T * sizeof(long long) + (2 * kKeys + 2 + T) * sizeof(int);
  if (smem > 227 * 1024) {
    set_error("spreading stage of %zu bytes exceeds shared memory", smem);
    return COV3D_EINVAL;
  }
  if (smem > 32 * 1024) {  // static shared arrays come on top of the dynamic size
    cudaError_t e = cudaFuncSetAttribute(spread_kernel<KT, W, CPL, COMP, RP>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(spread_kernel)");
  }
  spread_kernel<KT, W, CPL, COMP, RP><<<(unsigned)max_blocks, kSpreadWarps * 32, smem, st>>>(a);
  return launched("spread_kernel");
}

// One launch for all channels: the block sorts and stages its points once.  With three or more
// channel pairs, row-pair tasks with every lane holding kRowPairCPL pairs (groups of that many);
// otherwise row tasks with the pairs spread over lane groups.
template <int KT, int W, bool COMP>
int launch_wc(SpreadParams a, int nchan, int64_t max_blocks, cudaStream_t st) {
  constexpr int G = SpreadLanes<W>::G;
  a.ch0 = 0;
  a.nch = nchan;
  const int npairs = (nchan + 1) / 2;
  if (npairs >= 3 && 2 * SpreadLanes<W>::T <= 32) return launch_one<KT, W, kRowPairCPL, COMP, true>(a, max_blocks, st);
  const int cpl = (npairs + G - 1) / G;
  if (cpl <= 1) return launch_one<KT, W, 1, COMP, false>(a, max_blocks, st);
  if (cpl == 2) return launch_one<KT, W, 2, COMP, false>(a, max_blocks, st);
  return launch_one<KT, W, kMaxCPL, COMP, false>(a, max_blocks, st);
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
