// Interpolation ("type-2" half of the NUFFT, and the reference's grid_sample forward) over
// bin-sorted points: each bin's tile of the fine grid is read from HBM once into shared memory
// and reused by all its points; the projection epilogue (Nyquist zeroing, CTF multiply, 1/L)
// is fused.
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
  const int *bin_off;  // first sorted point of each bin (exclusive scan of the bin counts)
  const int *nsub;
  const float2 *grid;
  int64_t cs, chs;
  int shift;
  int ch0;
  int nch;  // channels in this pass (<= 2 * CP)
  float2 *out;
  int64_t ops, ocs;
  const float *ctf;
  const CtfCoef *ctfc;
  int nyquist;
  float scale;
};

constexpr int kBin = 8;
constexpr int kInterpWarps = 24;    // warps per block of the small tiles (two blocks per SM)
// Warps per block: 32 next to the wide windows' large tiles, one block per SM (ES, 10 channels:
// 11.9 against 12.0 ms with 24; the narrow tiles measured slower with 32)
template <int W, int CP>
struct InterpWarps {
  static constexpr int value = (W > 2 && CP >= 3) ? 32 : kInterpWarps;
};
constexpr int kInterpChunk = 1024;  // points staged at a time (20 KB; 2048 measured slightly slower)

// Channel pairs per pass: lanes are (window cell, channel pair) pairs, so W * CP <= 32, and the
// tile (bin + halo) of 2*CP complex channels must fit in shared memory.
template <int W>
struct InterpCP {
  static constexpr int value = W <= 2 ? 16 : 32 / W;
};

// One block per bin (see the kernel's first lines).  The block stages the bin's tile (bin +
// (W-1)-cell halo) of 2*CP channels in shared memory as [cell][channel] complex, then each warp
// takes one point at a time (32 / (W*CP) points for the narrow bilinear and nearest windows):
// lane (j, q) reads the two channels 2q, 2q+1 of tile[row][corner2 + j] for the W*W window
// rows -- W*CP contiguous 16-byte values per row, no bank conflicts -- and accumulates
// weight * value; the W partial sums of each pair are combined by a warp-shuffle tree and the
// epilogue (Nyquist zeroing, CTF, scale) is applied.
template <int KT, int W, int CP>
__global__ void __launch_bounds__(InterpWarps<W, CP>::value * 32) interp_kernel(const InterpParams a) {
  constexpr int T = kBin + W - 1;
  constexpr int CH = 2 * CP;
  constexpr int LANES = W * CP;
  // points per warp iteration: several when a point's W*CP lanes (and its 3W weights) fit more
  // than once into the warp, as for the bilinear and nearest kernels
  constexpr int PPW = (LANES >= 3 * W && 32 / LANES > 1) ? 32 / LANES : 1;
  extern __shared__ float4 tile4[];  // T^3 * CP float4 (= 2 complex), then the point records
  float2 *tile = reinterpret_cast<float2 *>(tile4);
  SortedPoint *s_sp = reinterpret_cast<SortedPoint *>(tile4 + T * T * T * CP);  // kInterpChunk
  float *s_sc = reinterpret_cast<float *>(s_sp + kInterpChunk);                  // epilogue factor
  const int sub = blockIdx.x;
  if (sub >= *a.nsub) return;
  const int bin = a.sub_bin[sub];
  const int first = a.sub_first[sub];
  // one block per bin: the block of the bin's first subproblem takes all of the bin's points,
  // kInterpChunk at a time, so the tile is staged once per bin (512 points per bin on average
  // at the cov-SGD workload, which 288-point subproblems split 2.8 ways; 14.1 -> 12.6 ms)
  if (first != a.bin_off[bin]) return;
  const int last = a.bin_off[bin + 1];
  int cnt = min(kInterpChunk, last - first);
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
  // pass's channels), all in flight before one wait.  A warp copies RPW tile rows (channel,
  // plane, row) at a time, lane (s, c2) cell c2 of its row s: the column offset is fixed per
  // lane, and only the row index is decomposed per copy
  {
    constexpr int RPW = 32 / T;
    const int lane = tid & 31, s = lane / T, c2 = lane - (lane / T) * T;
    if (s < RPW) {
      const int co = s_coloff[c2];
      const int64_t co_cs = co >= 0 ? (int64_t)co * a.cs : 0;
      const float2 *src0 = gbase + co_cs;
      const unsigned dst0 = (unsigned)__cvta_generic_to_shared(tile + c2 * CH);
      const int step = (int)(blockDim.x >> 5) * RPW;
      for (int row = (tid >> 5) * RPW + s; row < CH * T * T; row += step) {
        const int ch = row / (T * T);
        const int rowi = row - ch * (T * T);
        const long long ro = s_rowoff[rowi];
        const bool ok = ch < a.nch && ro >= 0 && co >= 0;
        const float2 *src = ok ? src0 + ro + (int64_t)ch * a.chs : gbase;
        const unsigned dst = dst0 + (unsigned)((rowi * T * CH + ch) * sizeof(float2));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(ok ? 8 : 0) : "memory");
      }
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  // lane = (point slot pp, window cell j along axis 2, channel pair q)
  const int pp = lane / LANES, sl = lane - (lane / LANES) * LANES;
  const int j = sl / CP, q = sl - (sl / CP) * CP;
  const int lane0 = (pp < PPW ? pp : 0) * LANES;  // first lane of this lane's point slot
  const int wl = PPW == 1 ? lane : sl;             // this lane's tap among the point's 3W weights
  // the point slots' taps, per warp and double-buffered by iteration (see below)
  __shared__ __align__(16) float s_w[InterpWarps<W, CP>::value * 2 * PPW * 24];
  int wbuf = 0;
  for (int base = first;;) {
    for (int k0 = warp * PPW; k0 < cnt; k0 += InterpWarps<W, CP>::value * PPW) {
      const int k = k0 + pp;
      const bool pt_ok = pp < PPW && k < cnt;
      const SortedPoint sp = s_sp[pt_ok ? k : k0];
      int c0[3];
      c0[0] = first_cell<KT, W>(sp.t0);
      c0[1] = first_cell<KT, W>(sp.t1);
      c0[2] = first_cell<KT, W>(sp.t2);
      // one kernel weight per lane wl < 3W, then shared through the warp
      float myw = 0.0f;
      if (wl < 3 * W) {
        const int d = wl / W, tq = wl - (wl / W) * W;
        const float td = d == 0 ? sp.t0 : d == 1 ? sp.t1 : sp.t2;
        myw = tap_weight<KT, W>(td, tq, a.k.beta);
      }
      // through the warp's slot in shared memory (double-buffered by iteration): axis-0 taps at
      // 0, axis-1 at 8, axis-2 at 16, read back as broadcast 16-byte loads -- five loads and a
      // store instead of 13 shuffles in the queue the tile loads use (11.9 -> 11.5 ms)
      float *ws = s_w + ((warp * 2 + wbuf) * PPW + lane0 / LANES) * 24;
      if (wl < 3 * W) ws[(wl / W) * 8 + wl - (wl / W) * W] = myw;
      __syncwarp();
      float w0[8], w1[8];
      {
        const float4 a0 = *reinterpret_cast<const float4 *>(ws), a1 = *reinterpret_cast<const float4 *>(ws + 4);
        const float4 b0 = *reinterpret_cast<const float4 *>(ws + 8), b1 = *reinterpret_cast<const float4 *>(ws + 12);
        w0[0] = a0.x; w0[1] = a0.y; w0[2] = a0.z; w0[3] = a0.w; w0[4] = a1.x; w0[5] = a1.y; w0[6] = a1.z; w0[7] = a1.w;
        w1[0] = b0.x; w1[1] = b0.y; w1[2] = b0.z; w1[3] = b0.w; w1[4] = b1.x; w1[5] = b1.y; w1[6] = b1.z; w1[7] = b1.w;
      }
      const float wj = ws[16 + (j < W ? j : 0)];
      wbuf ^= 1;
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
      const bool lane_ok = pt_ok && cell2 >= 0;
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
      // the W partial sums of each pair by a shuffle tree over the window cells j (lanes j*CP + q
      // of the slot): at each level cell j adds cell j + h, h = ceil(width / 2)
      float4 s = make_float4(a01.x, a01.y, a23.x, a23.y);
  #pragma unroll
      for (int lvl = 0; lvl < 3; ++lvl) {
        const int wc = lvl == 0 ? W : lvl == 1 ? (W + 1) / 2 : ((W + 1) / 2 + 1) / 2;
        if (wc <= 1) break;
        const int h = (wc + 1) / 2;
        float4 t;
        t.x = __shfl_down_sync(0xffffffffu, s.x, h * CP);
        t.y = __shfl_down_sync(0xffffffffu, s.y, h * CP);
        t.z = __shfl_down_sync(0xffffffffu, s.z, h * CP);
        t.w = __shfl_down_sync(0xffffffffu, s.w, h * CP);
        if (j + h < wc) {
          s.x += t.x;
          s.y += t.y;
          s.z += t.z;
          s.w += t.w;
        }
      }
      if (pt_ok && sl < CP) {
        // epilogue: vol_forward's Nyquist zeroing, CTF multiply and 1/L (projection_funcs.py:355-370)
        const int64_t id = sp_id(sp.idf);
        const float sc = s_sc[k];
        float2 *o = a.out + id * a.ops + (int64_t)(a.ch0 + 2 * sl) * a.ocs;
        if (2 * sl < a.nch) o[0] = make_float2(s.x * sc, s.y * sc);
        if (2 * sl + 1 < a.nch) o[a.ocs] = make_float2(s.z * sc, s.w * sc);
      }
    }
    base += kInterpChunk;
    if (base >= last) break;
    cnt = min(kInterpChunk, last - base);
    __syncthreads();  // every warp is done with the previous points
    for (int k = tid; k < cnt; k += blockDim.x) {
      const SortedPoint sp = a.pts[base + k];
      s_sp[k] = sp;
      float sc = (a.nyquist && sp_nyquist(sp.idf)) ? 0.0f : a.scale;
      sc *= ctf_factor(a.ctf, a.ctfc, a.g, sp_id(sp.idf));
      s_sc[k] = sc;
    }
    __syncthreads();
  }
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
      (size_t)T * T * T * CP * sizeof(float4) + (size_t)kInterpChunk * (sizeof(SortedPoint) + 4);
  if (smem > 32 * 1024) {  // static shared arrays come on top of the dynamic size
    cudaError_t e = cudaFuncSetAttribute(interp_kernel<KT, W, CP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(interp_kernel)");
  }
  interp_kernel<KT, W, CP><<<(unsigned)max_blocks, InterpWarps<W, CP>::value * 32, smem, st>>>(a);
  return launched("interp_kernel");
}

// Channel passes of at most 2*InterpCP<W> channels; a short last pass uses a smaller tile.
template <int KT, int W>
int launch_w(InterpParams a, int nchan, int64_t max_blocks, cudaStream_t st) {
  constexpr int CPMAX = InterpCP<W>::value;
  int done = 0;
  while (done < nchan) {
    const int left = nchan - done;
    a.ch0 = done;
    int s = COV3D_OK, ch = 0;
    if (left >= 2 * CPMAX) {
      ch = 2 * CPMAX;
      a.nch = ch;
      s = launch_cp<KT, W, CPMAX>(a, max_blocks, st);
    } else {
      ch = left;
      a.nch = ch;
      if constexpr (W <= 2) {
        // narrow windows: the smallest tile that holds the pass, with several points per warp
        const int need = (left + 1) / 2;
        if (need <= 3) s = launch_cp<KT, W, 3>(a, max_blocks, st);
        else if (need <= 4) s = launch_cp<KT, W, 4>(a, max_blocks, st);
        else if (need <= 5) s = launch_cp<KT, W, 5>(a, max_blocks, st);
        else if (need <= 8) s = launch_cp<KT, W, 8>(a, max_blocks, st);
        else s = launch_cp<KT, W, CPMAX>(a, max_blocks, st);
      } else {
        // up to 2*CPMAX - 1 channels in the full-size tile; 3-4 and 1-2 channels in smaller ones
        if (left > 4) s = launch_cp<KT, W, CPMAX>(a, max_blocks, st);
        else if (left > 2) s = launch_cp<KT, W, (CPMAX > 2 ? 2 : CPMAX)>(a, max_blocks, st);
        else s = launch_cp<KT, W, 1>(a, max_blocks, st);
      }
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
  a.sub_bin = p->sub_bin.as<int>();
  a.sub_first = p->sub_first.as<int>();
  a.bin_off = p->bin_off.as<int>();
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
