// Spreading ("type-1" half of the NUFFT; exact adjoint of interp.cu, replacing the
// reference's grid_sample backward with FP32 global atomics, nufft_plan.py:171-242), over the
// bin-sorted point records of points_sort.cu.  See spread_kernel for the decomposition.

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

constexpr int kBin = 8;
constexpr int kSpreadWarps = 16;
// Row-group kernel: two blocks of 8 warps per SM (128 registers), so one block's staging
// (sort, records, values) overlaps the other's tasks; one block of 16 warps measured 20.1
// against 18.0 ms at the cov-SGD workload
constexpr int kRowsWarps = 8;
constexpr int kRowsBlocks = 2;

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
  const CtfCoef *ctfc;
  int nyquist;
  float scale;
  float2 *grid;
  int64_t cs, chs;
  int shift;
  int max_sub;
};

// Prologue factor of im_backward: CTF multiply, Nyquist zeroing, scale (projection_funcs.py:385-399).
__device__ __forceinline__ float prologue(const PointGeom &g, int64_t id, const float *ctf, const CtfCoef *ctfc,
                                          int nyquist, float scale) {
  float sc = scale;
  if (nyquist && on_nyquist(g, id)) sc = 0.0f;
  return sc * ctf_factor(ctf, ctfc, g, id);
}

constexpr int kLMin = -8;   // window corners relative to the bin lie in [kLMin, kLMin + 16)
constexpr int kKeys = 256;  // sort key (l1 - kLMin) * 16 + (l0 - kLMin)
constexpr int kFoldRanges = 3;  // window-corner rows l1 summed in FP32 between compensated folds
// spread_rows_kernel: a task's W + ROWS - 1 = 8 ranges (w = 6) in two groups of four, two
// compensated folds instead of three (16.3 against 16.6 ms per cov-SGD step)
constexpr int kRowsFold = 4;

// Per-point record staged once per block, in elements of float2 (each weight twice, the operand
// of a packed multiply: spread_kernel) or float (each weight once, splatted in a register:
// spread_rows_kernel, where the bytes shared memory returns per visit are the bound): the
// axis-0 weights by tile plane and the axis-2 weights by tile column, zero
// outside the point's window (the column slot T is always zero, for idle lanes), and the W
// axis-1 weights with ROWS - 1 zeros before them and max(ROWS - 1, 1) after.  A lane's weight
// for tile row b of a point with window corner l1 is then
// rec[plane] * rec[W1 + b - l1] * rec[W2 + column], with no corner arithmetic and no select:
// lanes outside the window read zeros.
template <int W, int ROWS>
struct PointRec {
  static constexpr int T = kBin + W - 1;
  static constexpr int W1 = T + ROWS - 1;            // axis-1 weight o1 at W1 + o1
  static constexpr int Z1 = ROWS > 1 ? ROWS - 1 : 1;  // zeros after the axis-1 weights
  static constexpr int W2 = W1 + W + Z1;             // axis-2 weights by column
  static constexpr int F2 = (W2 + T + 2) / 2 * 2;    // float2 per record (even)
};

// Shared memory after the staged channel values: tile row offsets, point records, sort keys,
// point ids, prologue factors, key counters and offsets, column offsets, the task counter.
struct StageSmem {
  long long *rowoff;  // T * T
  void *rec;          // max_sub * F2 record elements (float2, or float for scalar weights)
  int *key, *pid;     // max_sub each
  float *sc;          // max_sub
  int *cnt, *off;     // kKeys, kKeys + 1
  int *coloff;        // T
  int *task;          // 1
};

__host__ __device__ constexpr size_t stage_bytes(int max_sub, int T, int F2, size_t esize) {
  return (size_t)T * T * sizeof(long long) + (size_t)max_sub * (F2 * esize + 3 * sizeof(int)) +
         (size_t)(2 * kKeys + 2 + T) * sizeof(int);
}

__device__ __forceinline__ StageSmem carve(void *base, int max_sub, int T, int F2, int esize) {
  StageSmem s;
  s.rowoff = static_cast<long long *>(base);
  s.rec = s.rowoff + T * T;
  s.key = reinterpret_cast<int *>(static_cast<char *>(s.rec) + (size_t)max_sub * F2 * esize);
  s.pid = s.key + max_sub;
  s.sc = reinterpret_cast<float *>(s.pid + max_sub);
  s.cnt = reinterpret_cast<int *>(s.sc + max_sub);
  s.off = s.cnt + kKeys;
  s.coloff = s.off + kKeys + 1;
  s.task = s.coloff + T;
  return s;
}

// A subproblem: its points [first, first + cnt) of the sorted order and the tile origin.
struct SubTile {
  int first, cnt, ts0, ts1, ts2;
};

__device__ __forceinline__ SubTile sub_tile(const SpreadParams &a, int sub) {
  const int bin = a.sub_bin[sub];
  const int nb12 = a.bins.nb[1] * a.bins.nb[2];
  SubTile t;
  t.first = a.sub_first[sub];
  t.cnt = a.sub_count[sub];
  t.ts0 = (bin / nb12) * kBin;
  t.ts1 = ((bin / a.bins.nb[2]) % a.bins.nb[1]) * kBin;
  t.ts2 = (bin % a.bins.nb[2]) * kBin;
  return t;
}

// Stage 1 of both spreading kernels: the block counting-sorts its points by the (axis-1,
// axis-0) corner (l1, l0) of their window and stages, in that order, each point's record, id
// and prologue factor (im_backward's Nyquist zeroing, CTF and scale), then the global offsets
// of the tile's rows and columns.  The caller synchronises before reading them.
// a weight as a record element: twice (a packed-multiply operand) or once
__device__ __forceinline__ void put_weight(float2 *e, float x) { *e = make_float2(x, x); }
__device__ __forceinline__ void put_weight(float *e, float x) { *e = x; }

template <int KT, int W, int ROWS, typename E>
__device__ __forceinline__ void stage_subproblem(const SpreadParams &a, const StageSmem &s, const SubTile &st) {
  using Rec = PointRec<W, ROWS>;
  constexpr int T = Rec::T;
  constexpr int F2 = Rec::F2;
  const int n = a.g.n;
  const int tid = threadIdx.x;
  for (int e = tid; e < kKeys; e += blockDim.x) s.cnt[e] = 0;
  __syncthreads();
  // sort keys and ranks
  for (int k = tid; k < st.cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[st.first + k];
    int c0 = first_cell<KT, W>(sp.t0), c1 = first_cell<KT, W>(sp.t1);
    if (KT == COV3D_KERNEL_ES) {
      c0 = wrap1(c0, n);
      c1 = wrap1(c1, n);
    }
    const int key = (min(max(c1 - st.ts1 - kLMin, 0), 15) << 4) | min(max(c0 - st.ts0 - kLMin, 0), 15);
    s.key[k] = key | (atomicAdd(s.cnt + key, 1) << 8);
  }
  __syncthreads();
  if (tid < 32) {  // exclusive scan of the 256 counters by one warp, 8 per lane
    int v[kKeys / 32], sum = 0;
#pragma unroll
    for (int u = 0; u < kKeys / 32; ++u) {
      v[u] = s.cnt[tid * (kKeys / 32) + u];
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
      s.off[tid * (kKeys / 32) + u] = base;
      base += v[u];
    }
    if (tid == 31) s.off[kKeys] = incl;
  }
  __syncthreads();
  // records, point ids and prologue factors in sorted order
  for (int k = tid; k < st.cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[st.first + k];
    const int kr = s.key[k];
    const int slot = s.off[kr & 255] + (kr >> 8);
    float w0[W], w1[W], w2[W];
    int c0 = taps<KT, W>(sp.t0, a.k.beta, w0);
    taps<KT, W>(sp.t1, a.k.beta, w1);
    int c2 = taps<KT, W>(sp.t2, a.k.beta, w2);
    if (KT == COV3D_KERNEL_ES) {
      c0 = wrap1(c0, n);
      c2 = wrap1(c2, n);
    }
    E *rec = static_cast<E *>(s.rec) + slot * F2;
    const int l0 = c0 - st.ts0, l2 = c2 - st.ts2;  // bin-local corners, >= 1 - W (zero padding below)
    const float z = 0.0f;
#pragma unroll
    for (int e = 0; e < T; ++e) {
      put_weight(rec + e, z);
      put_weight(rec + Rec::W2 + e, z);
    }
    put_weight(rec + Rec::W2 + T, z);
#pragma unroll
    for (int e = T; e < Rec::W1; ++e) put_weight(rec + e, z);
#pragma unroll
    for (int e = Rec::W1 + W; e < Rec::W2; ++e) put_weight(rec + e, z);
#pragma unroll
    for (int r = 0; r < W; ++r) {
      if (l0 + r >= 0 && l0 + r < T) put_weight(rec + l0 + r, w0[r]);
      if (l2 + r >= 0 && l2 + r < T) put_weight(rec + Rec::W2 + l2 + r, w2[r]);
      put_weight(rec + Rec::W1 + r, w1[r]);
    }
    const int id = sp_id(sp.idf);
    float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
    sc *= ctf_factor(a.ctf, a.ctfc, a.g, id);
    s.pid[slot] = id;
    s.sc[slot] = sc;
  }
  // global offsets of the tile's rows (axes 0, 1) and columns (axis 2)
  for (int e = tid; e < T * T; e += blockDim.x) {
    const int ra = e / T, rb = e - (e / T) * T;
    int m0 = st.ts0 + ra, m1 = st.ts1 + rb;
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
    s.rowoff[e] = ok ? ((int64_t)m0 * n + m1) * n : -1;
  }
  for (int e = tid; e < T; e += blockDim.x) {
    int m2 = st.ts2 + e;
    bool ok = true;
    if (KT == COV3D_KERNEL_ES) {
      m2 = m2 >= n ? m2 - n : m2;
    } else {
      ok = m2 < n;
    }
    m2 += a.shift;
    m2 = m2 >= n ? m2 - n : m2;
    s.coloff[e] = ok ? m2 : -1;
  }
}

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

// Row tasks, for few channels.  One block per subproblem (a bin of 8^3 cells and at most
// max_sub of its points); the cells it can reach form a tile of the bin and a (W-1)-cell halo,
// T^3 cells.  After stage_subproblem, a task is one tile row: plane a, row b.  The points whose
// window covers it are the W contiguous ranges {l1 = b - o1, l0 in [a - W + 1, a]},
// o1 = 0 .. W-1, of the sorted order.  Lane (g, c) keeps the sums of cell (a, b, c) for its
// channel pairs in registers: each group of kFoldRanges ranges is summed in FP32 and, with COMP,
// added to the cell's (hi, lo) pair by a TwoSum, so the error of the cell's accumulation is that
// of one short FP32 sum per group.  The finished row goes to the global grid with one complex
// atomic per cell and channel.  Warps take tasks from a shared counter.  The block needs no
// shared-memory tile: its shared memory is the staged points only.
template <int KT, int W, int CPL, bool COMP>
__global__ void __launch_bounds__(kSpreadWarps * 32, W < 8 ? 2 : 1) spread_kernel(const SpreadParams a) {
  constexpr int T = SpreadLanes<W>::T;
  constexpr int G = SpreadLanes<W>::G;  // lane groups over channel pairs
  constexpr int NP = G * CPL;           // channel pairs staged per group
  using Rec = PointRec<W, 1>;
  constexpr int F2 = Rec::F2;
  extern __shared__ float4 smem4[];
  float4 *s_val = smem4;  // max_sub * NP
  const StageSmem s = carve(s_val + a.max_sub * NP, a.max_sub, T, F2, sizeof(float2));
  const float2 *recs = static_cast<const float2 *>(s.rec);
  const int sub = blockIdx.x;
  if (sub >= *a.nsub) return;
  const SubTile st = sub_tile(a, sub);
  stage_subproblem<KT, W, 1, float2>(a, s, st);

  const int tid = threadIdx.x, lane = tid & 31;
  const int g = lane / T, c = lane - (lane / T) * T;
  const bool lane_live = g < G;
  const int gv = lane_live ? g : 0;  // idle lanes compute pair 0 and drop it
  const int npairs = (a.nch + 1) / 2;
  for (int p0 = 0; p0 < npairs; p0 += NP) {  // channel groups of NP pairs
    __syncthreads();
    // this group's scaled channel pairs, in sorted order
    for (int e = tid; e < st.cnt * NP; e += blockDim.x) {
      const int slot = e / NP, pp = p0 + (e - (e / NP) * NP);
      const float sc = s.sc[slot];
      const float2 *src = a.vals + (int64_t)s.pid[slot] * a.ips + (int64_t)(a.ch0 + 2 * pp) * a.ics;
      const float2 v0 = 2 * pp < a.nch ? __ldg(src) : make_float2(0.f, 0.f);
      const float2 v1 = 2 * pp + 1 < a.nch ? __ldg(src + a.ics) : make_float2(0.f, 0.f);
      s_val[e] = make_float4(v0.x * sc, v0.y * sc, v1.x * sc, v1.y * sc);
    }
    if (tid == 0) *s.task = 0;
    __syncthreads();

    for (;;) {
      int task = 0;
      if (lane == 0) task = atomicAdd(s.task, 1);
      task = __shfl_sync(0xffffffffu, task, 0);
      if (task >= T * T) break;
      const int pa = task / T;
      const int rb = task - pa * T;  // the task's row
      const int b0lo = max(pa - W + 1 - kLMin, 0), b0hi = min(pa - kLMin, 15);
      // cell sums of channel pairs (0, 1) and (2, 3) of each pair group, and their TwoSum errors
      float2 hi01[CPL], hi23[CPL], lo01[CPL], lo23[CPL];
#pragma unroll
      for (int u = 0; u < CPL; ++u) {
        hi01[u] = hi23[u] = lo01[u] = lo23[u] = make_float2(0.f, 0.f);
      }
      bool any = false;
      const float2 *w2c = recs + Rec::W2 + c;  // this lane's column weight, record 0
      for (int l1g = rb; l1g > rb - W; l1g -= kFoldRanges) {
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
          const int ibeg = s.off[(b1 << 4) | b0lo], iend = s.off[((b1 << 4) | b0hi) + 1];
          in |= lane_live && ibeg < iend;
          const int k1 = Rec::W1 + (lane_live ? rb - l1 : W);  // a zero slot for idle lanes
          // two points per iteration; a lane whose column is outside a point's window
          // multiplies by a zero weight
          int i = ibeg;
          for (; i + 1 < iend; i += 2) {
            const float2 *ra = recs + i * F2, *rb2 = ra + F2;
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
            const float2 *ra = recs + i * F2;
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
        if (!any) {  // the first group: its fold, TwoSum(0, sum), is (sum, 0) exactly
#pragma unroll
          for (int u = 0; u < CPL; ++u) {
            hi01[u] = part01[u];
            hi23[u] = part23[u];
          }
        } else {
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
        any = true;
      }
      // the finished cell goes to the global grid
      if (!any) continue;
      const long long ro = s.rowoff[pa * T + rb];
      const int co = s.coloff[c];
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

// Row-group tasks with the channels split over two lane halves, for many channels (the
// covariance gradient's r eigenvolumes).  Stage 1 as in spread_kernel; the channel values of a
// group of 2 * CH channels are staged per point as two 16-byte-aligned halves of CH.  A task is
// ROWS consecutive tile rows of one plane: lane (h, c) owns tile column c of those rows for the
// channels of half h (26 of 32 lanes at W = 6), so every point of the task's ranges costs a lane
// CH values, ROWS + 2 weight loads and ROWS * CH packed multiply-adds, and a point is visited by
// the tasks of its W planes and the row groups its W rows meet (W = 6, ROWS = 3: 16 on
// average).  Shared memory returns per point and lane 40 bytes of values where lanes owning all
// channels of one cell would take 80: the loads, not the multiply-adds, bound this kernel.  The
// task's ranges are those of the corners l1 in [b - W + 1, b + ROWS - 1]; the summation (FP32
// groups of kRowsFold ranges, TwoSum folds with COMP) and the atomics are those of
// spread_kernel.
template <int KT, int W, int CH, int ROWS, bool COMP>
__global__ void __launch_bounds__(kRowsWarps * 32, kRowsBlocks) spread_rows_kernel(const SpreadParams a) {
  constexpr int T = kBin + W - 1;
  static_assert(2 * T <= 32, "two lane halves of T columns per warp");
  constexpr int HS = (CH + 1) / 2 * 2;       // float2 per half of a point's values (even)
  constexpr int PS = 2 * HS;                 // float2 of values per point
  constexpr int RG = (T + ROWS - 1) / ROWS;  // row groups per plane
  using Rec = PointRec<W, ROWS>;
  constexpr int F2 = Rec::F2;
  extern __shared__ float4 smem4[];
  float2 *s_val = reinterpret_cast<float2 *>(smem4);  // max_sub * PS
  const StageSmem s = carve(s_val + a.max_sub * PS, a.max_sub, T, F2, sizeof(float));
  const float *recs = static_cast<const float *>(s.rec);  // weights once each (scalar records)
  const int sub = blockIdx.x;
  if (sub >= *a.nsub) return;
  const SubTile st = sub_tile(a, sub);
  stage_subproblem<KT, W, ROWS, float>(a, s, st);

  const int tid = threadIdx.x, lane = tid & 31;
  const int h = lane / T;
  const bool lane_live = h < 2;
  const int hv = lane_live ? h : 0;             // idle lanes read half 0 ...
  const int c = lane_live ? lane - h * T : T;   // ... and the zero column weight
  const float *w2c = recs + Rec::W2 + c;        // this lane's column weight, record 0
  for (int p0 = 0; p0 < a.nch; p0 += 2 * CH) {  // channel groups of 2 * CH
    __syncthreads();
    // this group's scaled channel values, in sorted order: half hh holds p0 + hh * CH + ch
    for (int e = tid; e < st.cnt * 2 * CH; e += blockDim.x) {
      const int slot = e / (2 * CH), r = e - slot * (2 * CH);
      const int hh = r / CH, ch = r - hh * CH;
      const float sc = s.sc[slot];
      float2 v = make_float2(0.f, 0.f);
      if (p0 + r < a.nch) {
        const float2 x = __ldg(a.vals + (int64_t)s.pid[slot] * a.ips + (int64_t)(a.ch0 + p0 + r) * a.ics);
        v = make_float2(x.x * sc, x.y * sc);
      }
      s_val[slot * PS + hh * HS + ch] = v;
    }
    if (tid == 0) *s.task = 0;
    __syncthreads();

    for (;;) {
      int task = 0;
      if (lane == 0) task = atomicAdd(s.task, 1);
      task = __shfl_sync(0xffffffffu, task, 0);
      if (task >= T * RG) break;
      const int pa = task / RG;
      const int rb = (task - pa * RG) * ROWS;  // first row of the task
      const int b0lo = max(pa - W + 1 - kLMin, 0), b0hi = min(pa - kLMin, 15);
      float2 hi[ROWS][CH], lo[ROWS][CH];  // cell sums and their TwoSum errors
#pragma unroll
      for (int q = 0; q < ROWS; ++q)
#pragma unroll
        for (int ch = 0; ch < CH; ++ch) hi[q][ch] = lo[q][ch] = make_float2(0.f, 0.f);
      // the points of the task's ranges l1g, l1g - 1, ... (kRowsFold of them) multiplied into acc
      // (packed FP32, FFMA2: the same rounding as fmaf); true if any range held a point
      auto group = [&](const int l1g, float2(&acc)[ROWS][CH]) {
        bool got = false;
#pragma unroll  // 128 registers, 8 bytes of spills; not unrolled (126, none): 16.5 against 16.3 ms
        for (int sr = 0; sr < kRowsFold; ++sr) {
          const int l1 = l1g - sr;
          const int b1 = l1 - kLMin;
          if (l1 <= rb - W || b1 < 0 || b1 > 15 || b0lo > b0hi) continue;
          const int ibeg = s.off[(b1 << 4) | b0lo], iend = s.off[((b1 << 4) | b0hi) + 1];
          got |= ibeg < iend;
          const int k1 = Rec::W1 + rb - l1;  // row rb + q reads the axis-1 weight k1 + q
#pragma unroll 2  // two points' loads in flight (17.5 against 18.0 ms; four: no further gain)
          for (int i = ibeg; i < iend; ++i) {
            const float *rec = recs + i * F2;
            const float w02 = rec[pa] * w2c[i * F2];
            float2 w[ROWS];
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
              const float wq = w02 * rec[k1 + q];
              w[q] = make_float2(wq, wq);
            }
            const float2 *vp = s_val + i * PS + hv * HS;
            float2 v[CH];
#pragma unroll
            for (int ch = 0; ch + 1 < CH; ch += 2) {
              const float4 x = *reinterpret_cast<const float4 *>(vp + ch);
              v[ch] = make_float2(x.x, x.y);
              v[ch + 1] = make_float2(x.z, x.w);
            }
            if (CH & 1) v[CH - 1] = vp[CH - 1];
#pragma unroll
            for (int q = 0; q < ROWS; ++q)
#pragma unroll
              for (int ch = 0; ch < CH; ++ch) acc[q][ch] = __ffma2_rn(w[q], v[ch], acc[q][ch]);
          }
        }
        return got;
      };
      // the first group straight into the cell sums (its fold, TwoSum(0, sum), is (sum, 0)
      // exactly), each later one summed apart and folded in
      bool any = group(rb + ROWS - 1, hi);
      for (int l1g = rb + ROWS - 1 - kRowsFold; l1g > rb - W; l1g -= kRowsFold) {
        float2 part[ROWS][CH];
#pragma unroll
        for (int q = 0; q < ROWS; ++q)
#pragma unroll
          for (int ch = 0; ch < CH; ++ch) part[q][ch] = make_float2(0.f, 0.f);
        if (!group(l1g, part)) continue;
        any = true;
#pragma unroll
        for (int q = 0; q < ROWS; ++q)
#pragma unroll
          for (int ch = 0; ch < CH; ++ch) {
            if (!COMP) hi[q][ch] = __fadd2_rn(hi[q][ch], part[q][ch]);
            else two_sum2(hi[q][ch], lo[q][ch], part[q][ch]);
          }
      }
      // the finished cells go to the global grid
      if (!any || !lane_live) continue;
      const int co = s.coloff[c];
      if (co < 0) continue;
#pragma unroll
      for (int q = 0; q < ROWS; ++q) {
        if (rb + q >= T) break;
        const long long ro = s.rowoff[pa * T + rb + q];
        if (ro < 0) continue;
        float2 *dst = a.grid + (ro + co) * a.cs + (int64_t)(a.ch0 + p0 + hv * CH) * a.chs;
#pragma unroll
        for (int ch = 0; ch < CH; ++ch) {
          const float2 x = COMP ? __fadd2_rn(hi[q][ch], lo[q][ch]) : hi[q][ch];
          if (p0 + hv * CH + ch < a.nch && (x.x != 0.0f || x.y != 0.0f)) atomicAdd(dst + ch * a.chs, x);
        }
      }
    }
  }
}

constexpr int kRowGroupCH = 5;  // channels per lane half (row-group tasks)
constexpr int kRows = 3;        // tile rows per lane (row-group tasks; 2 measured 12 % slower)

template <typename Kernel>
int launch_spread_kernel(Kernel kernel, const char *name, size_t smem, const SpreadParams &a, int64_t max_blocks,
                         cudaStream_t st, int warps = kSpreadWarps) {
  if (smem > 227 * 1024) {
    set_error("spreading stage of %zu bytes exceeds shared memory", smem);
    return COV3D_EINVAL;
  }
  if (smem > 32 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(spread)");
  }
  kernel<<<(unsigned)max_blocks, warps * 32, smem, st>>>(a);
  return launched(name);
}

// One launch for all channels: the block sorts and stages its points once.  With three or more
// channel pairs, narrow windows (W <= 2) take row tasks with two channel pairs per lane group
// and wider ones take row-group tasks over two lane halves of kRowGroupCH channels (groups of
// 2 * kRowGroupCH channels), otherwise row tasks with the (at most two, G >= 2) pairs spread
// over the lane groups.
template <int KT, int W, bool COMP>
int launch_wc(SpreadParams a, int nchan, int64_t max_blocks, cudaStream_t st) {
  constexpr int T = kBin + W - 1;
  constexpr int G = SpreadLanes<W>::G;
  a.ch0 = 0;
  a.nch = nchan;
  const int npairs = (nchan + 1) / 2;
  if constexpr (W <= 2) {
    // narrow windows: one-row tasks with two pairs per lane group (G * 2 pairs per channel group),
    // small registers and shared memory, two blocks per SM; the row-group kernel's three-row
    // tasks multiply by zero for all but two of a lane's columns (bilinear step: 4.6 against
    // 7.4 ms)
    if (npairs >= 3) {
      constexpr int CPL = 2;
      const size_t smem = (size_t)a.max_sub * G * CPL * sizeof(float4) +
                          stage_bytes(a.max_sub, T, PointRec<W, 1>::F2, sizeof(float2));
      return launch_spread_kernel(spread_kernel<KT, W, CPL, COMP>, "spread_kernel", smem, a, max_blocks, st);
    }
  }
  if constexpr (W > 2) {
    if (npairs >= 3) {
      constexpr int PS = 2 * ((kRowGroupCH + 1) / 2 * 2);
      const size_t smem = (size_t)a.max_sub * PS * sizeof(float2) +
                          stage_bytes(a.max_sub, T, PointRec<W, kRows>::F2, sizeof(float));
      return launch_spread_kernel(spread_rows_kernel<KT, W, kRowGroupCH, kRows, COMP>, "spread_rows_kernel", smem,
                                  a, max_blocks, st, kRowsWarps);
    }
  }
  static_assert(2 * G >= 2, "at most two channel pairs spread over the lane groups");
  const size_t smem =
      (size_t)a.max_sub * G * sizeof(float4) + stage_bytes(a.max_sub, T, PointRec<W, 1>::F2, sizeof(float2));
  return launch_spread_kernel(spread_kernel<KT, W, 1, COMP>, "spread_kernel", smem, a, max_blocks, st);
}

template <int KT, int W>
int launch_w(SpreadParams a, int nchan, bool comp, int64_t max_blocks, cudaStream_t st) {
  return comp ? launch_wc<KT, W, true>(a, nchan, max_blocks, st) : launch_wc<KT, W, false>(a, nchan, max_blocks, st);
}

// Per-image adjoint (no sum over images): direct global atomics, one thread per point.
template <int KT, int W>
__global__ void spread_unagg_kernel(PointGeom g, KernelSpec k, int64_t M, const float2 *__restrict__ vals,
                                    int64_t ips, const float *ctf, const CtfCoef *ctfc, int nyquist, float scale,
                                    float2 *grids) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= M) return;
  const float sc = prologue(g, id, ctf, ctfc, nyquist, scale);
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
  a.ctfc = e.ctfc;
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
          <<<blocks, 256, 0, p->stream>>>(g, k, p->n_points, v, in_ps, e.ctf, e.ctfc, e.nyquist, e.scale, out);
      break;
    case COV3D_KERNEL_LINEAR:
      spread_unagg_kernel<COV3D_KERNEL_LINEAR, 2>
          <<<blocks, 256, 0, p->stream>>>(g, k, p->n_points, v, in_ps, e.ctf, e.ctfc, e.nyquist, e.scale, out);
      break;
    default:
      switch (p->width) {
#define COV3D_UW(Wv)                                                                                     \
  case Wv:                                                                                             \
    spread_unagg_kernel<COV3D_KERNEL_ES, Wv>                                                           \
        <<<blocks, 256, 0, p->stream>>>(g, k, p->n_points, v, in_ps, e.ctf, e.ctfc, e.nyquist, e.scale, out); \
    break;
        COV3D_UW(4) COV3D_UW(5) COV3D_UW(6) COV3D_UW(7) COV3D_UW(8)
#undef COV3D_UW
        default: set_error("unsupported ES width %d", p->width); return COV3D_EINVAL;
      }
  }
  return launched("spread_unagg_kernel");
}

}  // namespace cov3d
