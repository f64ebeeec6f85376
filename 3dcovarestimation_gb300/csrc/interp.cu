// Interpolation ("type-2" half of the NUFFT, and the reference's grid_sample forward) over
// bin-sorted points: each subproblem's tile of the fine grid is read from HBM once into shared
// memory and reused by all its points; the projection epilogue (Nyquist zeroing, CTF
// multiply, 1/L) is fused.
#include <cstdlib>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

struct InterpParams {
  PointGeom g;
  KernelSpec k;
  Bins bins;
  const SortedPoint *pts;
  const int *sub_bin;
  const int *sub_first;
  const int *sub_count;
  const int *nsub;
  const float2 *grid;
  int64_t cs, chs;
  int shift;
  int ch0;
  int nch;  // channels in this pass (<= 2 * CP)
  int max_sub;
  float2 *out;
  int64_t ops, ocs;
  const float *ctf;
  const CtfCoef *ctfc;
  int nyquist;
  float scale;
};

constexpr int kBin = 8;
constexpr int kInterpWarps = 24;  // 56 registers: 24 warps next to the one 190 KB tile per SM

// Channel pairs per pass: lanes are (window cell, channel pair) pairs, so W * CP <= 32, and the
// tile (bin + halo) of 2*CP complex channels must fit in shared memory.
template <int W>
struct InterpCP {
  static constexpr int value = W <= 2 ? 16 : 32 / W;
};

// One block per subproblem.  The block stages the bin's tile (bin + (W-1)-cell halo) of 2*CP
// channels in shared memory as [cell][channel] complex, then each warp takes one point at a
// time: lane (j, q) reads the two channels 2q, 2q+1 of tile[row][corner2 + j] for the W*W
// window rows -- W*CP contiguous 16-byte values per row, no bank conflicts -- and accumulates
// weight * value; the W partial sums of each pair are combined through shared memory and the
// epilogue (Nyquist zeroing, CTF, scale) is applied.
template <int KT, int W, int CP>
__global__ void __launch_bounds__(kInterpWarps * 32) interp_kernel(const InterpParams a) {
  constexpr int T = kBin + W - 1;
  constexpr int CH = 2 * CP;
  constexpr int LANES = W * CP;
  extern __shared__ float4 tile4[];  // T^3 * CP float4 (= 2 complex), then kInterpWarps * 32 float4
  float2 *tile = reinterpret_cast<float2 *>(tile4);
  float4 *red = tile4 + T * T * T * CP;
  SortedPoint *s_sp = reinterpret_cast<SortedPoint *>(red + kInterpWarps * 32);  // max_sub
  float *s_sc = reinterpret_cast<float *>(s_sp + a.max_sub);                     // epilogue factor
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

  // stage the tile: per-row global offsets and per-cell axis-2 offsets are tabulated first, then
  // (channel, row, cell) elements are copied with cell fastest for coalesced global reads
  __shared__ long long s_rowoff[T * T];
  __shared__ int s_coloff[T];
  for (int e = tid; e < T * T; e += blockDim.x) {
    const int c0 = e / T, c1 = e - (e / T) * T;
    int m0 = ts0 + c0, m1 = ts1 + c1;
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
    s_rowoff[e] = ok ? ((int64_t)m0 * n + m1) * n * a.cs : -1;
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
  // the subproblem's point records and epilogue factors (Nyquist zeroing, CTF, scale)
  for (int k = tid; k < cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[first + k];
    s_sp[k] = sp;
    float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
    sc *= ctf_factor(a.ctf, a.ctfc, a.g, sp_id(sp.idf));
    s_sc[k] = sc;
  }
  const float2 *gbase = a.grid + (int64_t)a.ch0 * a.chs;
  // asynchronous copies global -> shared (8 bytes each, zero-filled outside the grid / past the
  // pass's channels), all in flight before one wait
  for (int e = tid; e < CH * T * T * T; e += blockDim.x) {
    const int c2 = e % T;
    const int rowi = (e / T) % (T * T);
    const int ch = e / (T * T * T);
    const long long ro = s_rowoff[rowi];
    const int co = s_coloff[c2];
    const bool ok = ch < a.nch && ro >= 0 && co >= 0;
    const float2 *src = ok ? gbase + ro + (int64_t)co * a.cs + (int64_t)ch * a.chs : gbase;
    const unsigned dst = (unsigned)__cvta_generic_to_shared(tile + (rowi * T + c2) * CH + ch);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(ok ? 8 : 0) : "memory");
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int j = lane / CP, q = lane - (lane / CP) * CP;  // window cell along axis 2, channel pair
  float4 *wred = red + warp * 32;
  for (int k = warp; k < cnt; k += kInterpWarps) {
    const SortedPoint sp = s_sp[k];
    int c0[3];
    c0[0] = first_cell<KT, W>(sp.t0);
    c0[1] = first_cell<KT, W>(sp.t1);
    c0[2] = first_cell<KT, W>(sp.t2);
    // one kernel weight per lane < 3W, then shared through the warp
    float myw = 0.0f;
    if (lane < 3 * W) {
      const int d = lane / W, tq = lane - (lane / W) * W;
      const float td = d == 0 ? sp.t0 : d == 1 ? sp.t1 : sp.t2;
      myw = tap_weight<KT, W>(td, tq, a.k.beta);
    }
    float w0[W], w1[W];
#pragma unroll
    for (int r = 0; r < W; ++r) {
      w0[r] = __shfl_sync(0xffffffffu, myw, r);
      w1[r] = __shfl_sync(0xffffffffu, myw, W + r);
    }
    const float wj = __shfl_sync(0xffffffffu, myw, 2 * W + (j < W ? j : 0));
    int l0 = c0[0], l1 = c0[1], l2 = c0[2];
    if (KT == COV3D_KERNEL_ES) {
      l0 = wrap1(l0, n);
      l1 = wrap1(l1, n);
      l2 = wrap1(l2, n);
    }
    l0 -= ts0;
    l1 -= ts1;
    l2 -= ts2;
    const int cell2 = l2 + j;
    const bool lane_ok = lane < LANES && cell2 >= 0;
    const float4 *base = tile4 + cell2 * CP + q;
    // two packed FP32 accumulators (FFMA2: one instruction per channel pair of values; the
    // same rounding as two fmaf); each window plane is summed over its rows with the axis-1
    // weights first, then added with its axis-0 weight times this lane's axis-2 weight
    float2 a01 = make_float2(0.f, 0.f), a23 = make_float2(0.f, 0.f);
    if (lane_ok) {
      float2 ww1[W];
#pragma unroll
      for (int i1 = 0; i1 < W; ++i1) ww1[i1] = make_float2(w1[i1], w1[i1]);
#pragma unroll
      for (int i0 = 0; i0 < W; ++i0) {
        const int r0 = l0 + i0;
        if (KT != COV3D_KERNEL_ES && r0 < 0) continue;
        float2 p01 = make_float2(0.f, 0.f), p23 = make_float2(0.f, 0.f);
#pragma unroll
        for (int i1 = 0; i1 < W; ++i1) {
          const int r1 = l1 + i1;
          if (KT != COV3D_KERNEL_ES && r1 < 0) continue;
          const float4 v = base[(r0 * T + r1) * T * CP];
          p01 = __ffma2_rn(ww1[i1], make_float2(v.x, v.y), p01);
          p23 = __ffma2_rn(ww1[i1], make_float2(v.z, v.w), p23);
        }
        const float w0j = w0[i0] * wj;
        const float2 ww0 = make_float2(w0j, w0j);
        a01 = __ffma2_rn(ww0, p01, a01);
        a23 = __ffma2_rn(ww0, p23, a23);
      }
    }
    wred[lane] = make_float4(a01.x, a01.y, a23.x, a23.y);
    __syncwarp();
    if (lane < CP) {
      float4 s = wred[lane];
#pragma unroll
      for (int r = 1; r < W; ++r) {
        const float4 x = wred[r * CP + lane];
        s.x += x.x;
        s.y += x.y;
        s.z += x.z;
        s.w += x.w;
      }
      // epilogue: vol_forward's Nyquist zeroing, CTF multiply and 1/L (projection_funcs.py:355-370)
      const int64_t id = sp_id(sp.idf);
      const float sc = s_sc[k];
      float2 *o = a.out + id * a.ops + (int64_t)(a.ch0 + 2 * lane) * a.ocs;
      if (2 * lane < a.nch) o[0] = make_float2(s.x * sc, s.y * sc);
      if (2 * lane + 1 < a.nch) o[a.ocs] = make_float2(s.z * sc, s.w * sc);
    }
    __syncwarp();
  }
}

// ----------------------------------------------------------------------------- grouped points
// Register-blocked ES interpolation for many channels (the covariance step's r eigenvolumes).
//
// The points of a subproblem are counting-sorted by the 2x2x2 block of their window corner
// (64 blocks per 8^3 bin); the points of one block all lie in the union window of W + 1 cells
// per axis that starts at the block's smallest corner (W along an axis where they share the
// corner).  A warp task is up to Q * kGroupP points of one block: lane (g, c) owns channel c of
// kGroupP points (group g), so every row of the union is read once per task -- the same
// addresses for the Q groups, a shared-memory broadcast -- and each loaded value feeds
// kGroupP points: per row and point, the row is reduced with the point's axis-2 weights
// (zero outside its window) and added with its axis-0 x axis-1 weight.  The work per point is
// (W + 1)^2 (W + 2) multiply-adds per channel against W^3 (1.8x at W = 6), in exchange for
// four times fewer shared loads per multiply-add than one point per lane; the tile staging and
// the epilogue (Nyquist zeroing, CTF, scale) are those of interp_kernel.
constexpr int kGroupWarps = 16;
// COV3D_INTERP_GROUP=0 selects the one-point-per-warp kernel for every channel count
// (comparison runs); read once per process.
inline bool interp_group_disabled() {
  static const bool off = [] {
    const char *v = getenv("COV3D_INTERP_GROUP");
    return v && v[0] == '0';
  }();
  return off;
}
constexpr int kGroupP = 4;  // points per lane
constexpr int kGroupKeys = 64;

// Complex channels per pass: the T^3 tile of CH channels and the per-point weight records must
// fit in shared memory next to each other.
template <int W>
struct GroupCH {
  static constexpr int value = W <= 6 ? 10 : (W == 7 ? 8 : 6);
};

__host__ __device__ constexpr size_t group_smem_bytes(int T, int CH, int max_sub) {
  return (size_t)T * T * T * CH * 8 + (size_t)max_sub * (24 * 4 + 6 * 4) + (size_t)(kGroupKeys * 3 + 4) * 4;
}

// One task of a warp: the union window rows [u0, u0 + e0) x [u1, u1 + e1) x [u2, u2 + E2) of the
// tile; acc[p] += sum over the window of w0 w1 w2 * value for this lane's kGroupP points.
template <int W, int CH, int E2>
__device__ __forceinline__ void group_rows(const float2 *__restrict__ tile, int u0, int u1, int u2, int e0, int e1,
                                           int cl, const float (&w1r)[kGroupP][W + 1],
                                           const float (&w2r)[kGroupP][W + 1], const int (&o0)[kGroupP],
                                           const int (&slot)[kGroupP], const bool (&valid)[kGroupP],
                                           const float *__restrict__ wts, float2 (&acc)[kGroupP]) {
  constexpr int T = kBin + W - 1;
  for (int i0 = 0; i0 < e0; ++i0) {
    float w0c[kGroupP];
#pragma unroll
    for (int p = 0; p < kGroupP; ++p) {
      const int j = i0 - o0[p];
      w0c[p] = (valid[p] && j >= 0 && j < W) ? wts[slot[p] * 24 + j] : 0.0f;
    }
    const float2 *row = tile + (((u0 + i0) * T + u1) * T + u2) * CH + cl;
#pragma unroll
    for (int i1 = 0; i1 < W + 1; ++i1) {
      if (i1 < e1) {
        float2 v[E2];
#pragma unroll
        for (int k = 0; k < E2; ++k) v[k] = row[(i1 * T + k) * CH];
#pragma unroll
        for (int p = 0; p < kGroupP; ++p) {
          float2 t = __fmul2_rn(make_float2(w2r[p][0], w2r[p][0]), v[0]);
#pragma unroll
          for (int k = 1; k < E2; ++k) t = __ffma2_rn(make_float2(w2r[p][k], w2r[p][k]), v[k], t);
          const float rw = w0c[p] * w1r[p][i1];
          acc[p] = __ffma2_rn(make_float2(rw, rw), t, acc[p]);
        }
      }
    }
  }
}

template <int W, int CH>
__global__ void __launch_bounds__(kGroupWarps * 32, 1) interp_group_kernel(const InterpParams a) {
  constexpr int T = kBin + W - 1;
  constexpr int Q = 32 / CH;
  constexpr int TP = Q * kGroupP;  // points per task (<= 32)
  constexpr int U = W + 1;
  static_assert(TP <= 32, "a task's points are read by one lane each");
  extern __shared__ float4 smem4[];
  float2 *tile = reinterpret_cast<float2 *>(smem4);                 // T^3 * CH, [cell][channel]
  float *wts = reinterpret_cast<float *>(tile + T * T * T * CH);     // max_sub * 24: w0[8] w1[8] w2[8]
  int *pid = reinterpret_cast<int *>(wts + a.max_sub * 24);          // point id, sorted order
  float *psc = reinterpret_cast<float *>(pid + a.max_sub);           // epilogue factor
  int *pcor = reinterpret_cast<int *>(psc + a.max_sub);              // corners l0 | l1 << 8 | l2 << 16
  int *pkey = pcor + a.max_sub;                                      // key | rank << 8, input order
  int *tfirst = pkey + a.max_sub;                                    // task -> first sorted slot
  int *tcount = tfirst + a.max_sub;                                  // task -> points
  int *kcnt = tcount + a.max_sub;                                    // kGroupKeys
  int *koff = kcnt + kGroupKeys;                                     // kGroupKeys + 1
  int *ktoff = koff + kGroupKeys + 1;                                // kGroupKeys + 1
  int *tcounter = ktoff + kGroupKeys + 1;
  __shared__ long long s_rowoff[T * T];
  __shared__ int s_coloff[T];
  __shared__ int s_lo[3], s_hi[3];  // corner extents of the subproblem's points
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

  for (int e = tid; e < T * T; e += blockDim.x) {
    const int c0 = e / T, c1 = e - (e / T) * T;
    int m0 = ts0 + c0, m1 = ts1 + c1;
    m0 = m0 >= n ? m0 - n : m0;
    m1 = m1 >= n ? m1 - n : m1;
    m0 += a.shift;
    m1 += a.shift;
    m0 = m0 >= n ? m0 - n : m0;
    m1 = m1 >= n ? m1 - n : m1;
    s_rowoff[e] = ((int64_t)m0 * n + m1) * n * a.cs;
  }
  for (int e = tid; e < T; e += blockDim.x) {
    int m2 = ts2 + e;
    m2 = m2 >= n ? m2 - n : m2;
    m2 += a.shift;
    s_coloff[e] = m2 >= n ? m2 - n : m2;
  }
  for (int e = tid; e < kGroupKeys; e += blockDim.x) kcnt[e] = 0;
  if (tid < 3) {
    s_lo[tid] = kBin;
    s_hi[tid] = -1;
  }
  if (tid == 0) *tcounter = 0;
  __syncthreads();
  // block keys of the window corners, ranks within a key, and the corners' extents
  {
    int lo0 = kBin, lo1 = kBin, lo2 = kBin, hi0 = -1, hi1 = -1, hi2 = -1;
    for (int k = tid; k < cnt; k += blockDim.x) {
      const SortedPoint sp = a.pts[first + k];
      const int l0 = wrap1(first_cell<COV3D_KERNEL_ES, W>(sp.t0), n) - ts0;
      const int l1 = wrap1(first_cell<COV3D_KERNEL_ES, W>(sp.t1), n) - ts1;
      const int l2 = wrap1(first_cell<COV3D_KERNEL_ES, W>(sp.t2), n) - ts2;
      const int key = ((l0 >> 1) * 4 + (l1 >> 1)) * 4 + (l2 >> 1);
      pkey[k] = key | (atomicAdd(kcnt + key, 1) << 8);
      lo0 = min(lo0, l0), lo1 = min(lo1, l1), lo2 = min(lo2, l2);
      hi0 = max(hi0, l0), hi1 = max(hi1, l1), hi2 = max(hi2, l2);
    }
    lo0 = __reduce_min_sync(0xffffffffu, lo0), lo1 = __reduce_min_sync(0xffffffffu, lo1);
    lo2 = __reduce_min_sync(0xffffffffu, lo2);
    hi0 = __reduce_max_sync(0xffffffffu, hi0), hi1 = __reduce_max_sync(0xffffffffu, hi1);
    hi2 = __reduce_max_sync(0xffffffffu, hi2);
    if ((tid & 31) == 0 && hi0 >= 0) {
      atomicMin(s_lo + 0, lo0), atomicMin(s_lo + 1, lo1), atomicMin(s_lo + 2, lo2);
      atomicMax(s_hi + 0, hi0), atomicMax(s_hi + 1, hi1), atomicMax(s_hi + 2, hi2);
    }
  }
  __syncthreads();
  // the tile cells the points' windows reach ([lo, hi + W) per axis), asynchronously: in flight
  // while the points are sorted
  const float2 *gbase = a.grid + (int64_t)a.ch0 * a.chs;
  {
    const int b0 = s_lo[0], b1 = s_lo[1], b2 = s_lo[2];
    const int x0 = s_hi[0] - b0 + W, x1 = s_hi[1] - b1 + W, x2 = s_hi[2] - b2 + W;
    const int box = x0 * x1 * x2;
    for (int e = tid; e < CH * box; e += blockDim.x) {
      const int ch = e / box;
      const int rem = e - ch * box;
      const int c2 = b2 + rem % x2;
      const int r01 = rem / x2;
      const int c1 = b1 + r01 % x1, c0 = b0 + r01 / x1;
      const int rowi = c0 * T + c1;
      const bool ok = ch < a.nch;
      const float2 *src = ok ? gbase + s_rowoff[rowi] + (int64_t)s_coloff[c2] * a.cs + (int64_t)ch * a.chs : gbase;
      const unsigned dst = (unsigned)__cvta_generic_to_shared(tile + (rowi * T + c2) * CH + ch);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(ok ? 8 : 0) : "memory");
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  if (tid < 32) {  // point offsets and task offsets per key (two keys per lane), and the task list
    const int k0 = 2 * tid;
    const int c0 = kcnt[k0], c1 = kcnt[k0 + 1];
    const int t0 = (c0 + TP - 1) / TP, t1 = (c1 + TP - 1) / TP;
    int ip = c0 + c1, it = t0 + t1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int xp = __shfl_up_sync(0xffffffffu, ip, o), xt = __shfl_up_sync(0xffffffffu, it, o);
      if (tid >= o) {
        ip += xp;
        it += xt;
      }
    }
    const int bp = ip - (c0 + c1), bt = it - (t0 + t1);
    koff[k0] = bp;
    koff[k0 + 1] = bp + c0;
    ktoff[k0] = bt;
    ktoff[k0 + 1] = bt + t0;
    for (int j = 0; j < t0; ++j) {
      tfirst[bt + j] = bp + j * TP;
      tcount[bt + j] = min(TP, c0 - j * TP);
    }
    for (int j = 0; j < t1; ++j) {
      tfirst[bt + t0 + j] = bp + c0 + j * TP;
      tcount[bt + t0 + j] = min(TP, c1 - j * TP);
    }
    if (tid == 31) {
      koff[kGroupKeys] = ip;
      ktoff[kGroupKeys] = it;
    }
  }
  __syncthreads();
  // per point, in sorted order: the axis weights, the id, the epilogue factor, the corners
  for (int k = tid; k < cnt; k += blockDim.x) {
    const SortedPoint sp = a.pts[first + k];
    const int kr = pkey[k];
    const int slot = koff[kr & 255] + (kr >> 8);
    float w[3][W];
    const int c0 = wrap1(taps<COV3D_KERNEL_ES, W>(sp.t0, a.k.beta, w[0]), n) - ts0;
    const int c1 = wrap1(taps<COV3D_KERNEL_ES, W>(sp.t1, a.k.beta, w[1]), n) - ts1;
    const int c2 = wrap1(taps<COV3D_KERNEL_ES, W>(sp.t2, a.k.beta, w[2]), n) - ts2;
    float *ws = wts + slot * 24;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int j = 0; j < 8; ++j) ws[d * 8 + j] = j < W ? w[d][j] : 0.0f;
    pid[slot] = sp_id(sp.idf);
    float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
    sc *= ctf_factor(a.ctf, a.ctfc, a.g, sp_id(sp.idf));
    psc[slot] = sc;
    pcor[slot] = c0 | (c1 << 8) | (c2 << 16);
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();

  const int ntasks = ktoff[kGroupKeys];
  const int lane = tid & 31;
  const int g = lane / CH;
  const bool live = g < Q;
  const int gl = live ? g : 0;
  const int cl = live ? lane - g * CH : 0;
  for (;;) {
    int task = 0;
    if (lane == 0) task = atomicAdd(tcounter, 1);
    task = __shfl_sync(0xffffffffu, task, 0);
    if (task >= ntasks) break;
    const int tf = tfirst[task], tn = tcount[task];
    // union window of the task's points: smallest corner and extent (W, or W + 1 where the
    // corners differ) per axis
    const int cor = pcor[tf + (lane < tn ? lane : 0)];
    const int l0 = cor & 255, l1 = (cor >> 8) & 255, l2 = cor >> 16;
    const int u0 = __reduce_min_sync(0xffffffffu, l0), u1 = __reduce_min_sync(0xffffffffu, l1);
    const int u2 = __reduce_min_sync(0xffffffffu, l2);
    const int e0 = __reduce_max_sync(0xffffffffu, l0) - u0 + W;
    const int e1 = __reduce_max_sync(0xffffffffu, l1) - u1 + W;
    const int e2 = __reduce_max_sync(0xffffffffu, l2) - u2 + W;
    float w1r[kGroupP][U], w2r[kGroupP][U];
    int o0[kGroupP], slot[kGroupP];
    bool valid[kGroupP];
#pragma unroll
    for (int p = 0; p < kGroupP; ++p) {
      const int idx = gl * kGroupP + p;
      valid[p] = live && idx < tn;
      slot[p] = tf + (valid[p] ? idx : 0);
      const int cp = pcor[slot[p]];
      o0[p] = (cp & 255) - u0;
      const int o1 = ((cp >> 8) & 255) - u1, o2 = (cp >> 16) - u2;
      const float4 *wp = reinterpret_cast<const float4 *>(wts + slot[p] * 24);
      const float4 a1 = wp[2], b1 = wp[3], a2 = wp[4], b2 = wp[5];
      const float x1[8] = {a1.x, a1.y, a1.z, a1.w, b1.x, b1.y, b1.z, b1.w};
      const float x2[8] = {a2.x, a2.y, a2.z, a2.w, b2.x, b2.y, b2.z, b2.w};
#pragma unroll
      for (int k = 0; k < U; ++k) {
        // tap k - o of the point (o = 0 or 1), zero outside its window
        const float y1 = o1 ? (k > 0 ? x1[k - 1] : 0.0f) : (k < W ? x1[k] : 0.0f);
        const float y2 = o2 ? (k > 0 ? x2[k - 1] : 0.0f) : (k < W ? x2[k] : 0.0f);
        w1r[p][k] = valid[p] ? y1 : 0.0f;
        w2r[p][k] = valid[p] ? y2 : 0.0f;
      }
    }
    float2 acc[kGroupP];
#pragma unroll
    for (int p = 0; p < kGroupP; ++p) acc[p] = make_float2(0.f, 0.f);
    if (e2 == W) {
      group_rows<W, CH, W>(tile, u0, u1, u2, e0, e1, cl, w1r, w2r, o0, slot, valid, wts, acc);
    } else {
      group_rows<W, CH, W + 1>(tile, u0, u1, u2, e0, e1, cl, w1r, w2r, o0, slot, valid, wts, acc);
    }
    // epilogue: vol_forward's Nyquist zeroing, CTF multiply and 1/L (projection_funcs.py:355-370)
    if (live && cl < a.nch) {
#pragma unroll
      for (int p = 0; p < kGroupP; ++p) {
        if (!valid[p]) continue;
        const float sc = psc[slot[p]];
        a.out[(int64_t)pid[slot[p]] * a.ops + (int64_t)(a.ch0 + cl) * a.ocs] = make_float2(acc[p].x * sc, acc[p].y * sc);
      }
    }
  }
}

template <int W>
int launch_group(InterpParams a, int nchan, int64_t max_blocks, cudaStream_t st) {
  constexpr int T = kBin + W - 1;
  constexpr int CH = GroupCH<W>::value;
  const size_t smem = group_smem_bytes(T, CH, a.max_sub);
  cudaError_t e = cudaFuncSetAttribute(interp_group_kernel<W, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(interp_group_kernel)");
  for (int done = 0; done < nchan; done += CH) {
    a.ch0 = done;
    a.nch = min(CH, nchan - done);
    interp_group_kernel<W, CH><<<(unsigned)max_blocks, kGroupWarps * 32, smem, st>>>(a);
    COV3D_TRY(launched("interp_group_kernel"));
  }
  return COV3D_OK;
}

// Points whose window lies entirely outside the grid (zero padding) get zero outputs.
__global__ void interp_dead_kernel(const SortedPoint *__restrict__ pts, const int *__restrict__ off, int64_t nbins,
                                   int nchan, float2 *__restrict__ out, int64_t ops, int64_t ocs) {
  const int lo = off[nbins], hi = off[nbins + 1];
  for (int k = lo + blockIdx.x * blockDim.x + threadIdx.x; k < hi; k += gridDim.x * blockDim.x) {
    const int64_t id = sp_id(pts[k].idf);
    for (int c = 0; c < nchan; ++c) out[id * ops + c * ocs] = make_float2(0.f, 0.f);
  }
}

template <int KT, int W, int CP>
int launch_cp(const InterpParams &a, int64_t max_blocks, cudaStream_t st) {
  constexpr int T = kBin + W - 1;
  const size_t smem =
      ((size_t)T * T * T * CP + kInterpWarps * 32) * sizeof(float4) + (size_t)a.max_sub * (sizeof(SortedPoint) + 4);
  if (smem > 32 * 1024) {  // static shared arrays come on top of the dynamic size
    cudaError_t e = cudaFuncSetAttribute(interp_kernel<KT, W, CP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(interp_kernel)");
  }
  interp_kernel<KT, W, CP><<<(unsigned)max_blocks, kInterpWarps * 32, smem, st>>>(a);
  return launched("interp_kernel");
}

// Channel passes of at most 2*InterpCP<W> channels; a short last pass uses a smaller tile.
template <int KT, int W>
int launch_w(InterpParams a, int nchan, int64_t max_blocks, cudaStream_t st) {
  constexpr int CPMAX = InterpCP<W>::value;
  if (KT == COV3D_KERNEL_ES && W >= 4 && nchan >= 8 && a.max_sub <= 288 && !interp_group_disabled())
    return launch_group<W < 4 ? 4 : W>(a, nchan, max_blocks, st);
  int done = 0;
  while (done < nchan) {
    const int left = nchan - done;
    a.ch0 = done;
    int s = COV3D_OK, ch = 0;
    if (left >= 2 * CPMAX) {
      ch = 2 * CPMAX;
      a.nch = ch;
      s = launch_cp<KT, W, CPMAX>(a, max_blocks, st);
    } else if (left > 4) {
      ch = left;  // up to 2*CPMAX - 1 channels in the full-size tile
      a.nch = ch;
      s = launch_cp<KT, W, CPMAX>(a, max_blocks, st);
    } else if (left > 2) {
      ch = left;
      a.nch = ch;
      s = launch_cp<KT, W, (CPMAX > 2 ? 2 : CPMAX)>(a, max_blocks, st);
    } else {
      ch = left;
      a.nch = ch;
      s = launch_cp<KT, W, 1>(a, max_blocks, st);
    }
    if (s != COV3D_OK) return s;
    done += ch;
  }
  return COV3D_OK;
}

}  // namespace

int launch_interp(cov3d_plan *p, const GridArgs &ga, int nchan, void *out, int64_t out_ps, int64_t out_cs,
                  const EpilogueArgs &e) {
  if (p->point_kind == kPointsNone || p->n_points == 0) {
    set_error("no points set");
    return COV3D_ESTATE;
  }
  InterpParams a{};
  a.g = make_geom(p);
  a.k = make_kernel(p);
  a.bins = p->bins;
  a.pts = p->sorted.as<SortedPoint>();
  a.max_sub = p->max_sub;
  a.sub_bin = p->sub_bin.as<int>();
  a.sub_first = p->sub_first.as<int>();
  a.sub_count = p->sub_count.as<int>();
  a.nsub = p->nsub.as<int>();
  a.grid = static_cast<const float2 *>(ga.grid);
  a.cs = ga.cell_stride;
  a.chs = ga.chan_stride;
  a.shift = ga.shift;
  a.out = static_cast<float2 *>(out);
  a.ops = out_ps;
  a.ocs = out_cs;
  a.ctf = e.ctf;
  a.ctfc = e.ctfc;
  a.nyquist = e.nyquist;
  a.scale = e.scale;
  const int64_t mb = p->bins.nbins + p->n_points / p->max_sub + 1;
  if (p->kernel != COV3D_KERNEL_ES) {
    interp_dead_kernel<<<64, 256, 0, p->stream>>>(a.pts, p->bin_off.as<int>(), p->bins.nbins, nchan, a.out, out_ps,
                                                  out_cs);
    COV3D_LAUNCHED("interp_dead_kernel");
  }
  switch (p->kernel) {
    case COV3D_KERNEL_NEAREST: return launch_w<COV3D_KERNEL_NEAREST, 1>(a, nchan, mb, p->stream);
    case COV3D_KERNEL_LINEAR: return launch_w<COV3D_KERNEL_LINEAR, 2>(a, nchan, mb, p->stream);
    default:
      switch (p->width) {
        case 4: return launch_w<COV3D_KERNEL_ES, 4>(a, nchan, mb, p->stream);
        case 5: return launch_w<COV3D_KERNEL_ES, 5>(a, nchan, mb, p->stream);
        case 6: return launch_w<COV3D_KERNEL_ES, 6>(a, nchan, mb, p->stream);
        case 7: return launch_w<COV3D_KERNEL_ES, 7>(a, nchan, mb, p->stream);
        case 8: return launch_w<COV3D_KERNEL_ES, 8>(a, nchan, mb, p->stream);
        default: set_error("unsupported ES width %d (supported: 4..8)", p->width); return COV3D_EINVAL;
      }
  }
}

}  // namespace cov3d
