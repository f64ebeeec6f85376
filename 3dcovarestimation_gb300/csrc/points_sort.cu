// Spatial binning of nonuniform points (counting sort by the first cell of each point's
// kernel window) and the subproblem table used by the spreading kernel.
//
// The reference hands unsorted points to cuFINUFFT with gpu_sort=0 (nufft_plan.py:297) or to
// grid_sample; here every point set is sorted once per setpts/setrot so that interpolation
// reads the grid with spatial locality and spreading can accumulate per-bin tiles in shared
// memory.
#include "cov3d_device.cuh"

namespace cov3d {

namespace {

// Bin of every point (dead points, whose window misses the grid, go to bin nbins) and its
// rank in the bin.  The lanes of a warp that share a bin (neighbouring pixels mostly do) take
// their ranks from one atomic on the bin's counter, in lane order.
template <int KT, int W>
__global__ void bin_count_kernel(PointGeom g, KernelSpec k, Bins bins, int64_t M, int *__restrict__ count,
                                 int *__restrict__ pt_bin, int *__restrict__ pt_rank) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = id < M;
  int bin = -1;
  if (valid) {
    float t[3];
    point_index(g, id, t);
    int b[3];
    bool dead = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int c0 = first_cell<KT, W>(t[d]);
      if (!(t[d] == t[d])) {  // NaN coordinate: no contribution
        dead = true;
        c0 = 0;
      }
      if (k.periodic) {
        c0 = pmod(c0, g.n);
      } else {
        if (c0 + W - 1 < 0 || c0 > g.n - 1) dead = true;
        c0 = min(max(c0, 0), g.n - 1);
      }
      b[d] = c0 / bins.bs[d];
    }
    bin = dead ? (int)bins.nbins : (b[0] * bins.nb[1] + b[1]) * bins.nb[2] + b[2];
  }
  const unsigned grp = __match_any_sync(0xffffffffu, bin);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(grp) - 1;
  int base = 0;
  if (valid && lane == leader) base = atomicAdd(count + bin, __popc(grp));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!valid) return;
  pt_bin[id] = bin;
  pt_rank[id] = base + __popc(grp & ((1u << lane) - 1u));
}

// Single-block exclusive scans over the bin counts: point offsets, and subproblem offsets
// (ceil(count / max_sub) subproblems per live bin).
__global__ void bin_scan_kernel(const int *__restrict__ count, int64_t nbins, int max_sub, int *__restrict__ off,
                                int *__restrict__ sub_off, int *__restrict__ nsub) {
  __shared__ long long s_pts[1024];
  __shared__ long long s_sub[1024];
  const int tid = threadIdx.x;
  const int64_t total = nbins + 1;  // includes the dead bin
  const int64_t per = (total + blockDim.x - 1) / blockDim.x;
  const int64_t lo = tid * per;
  const int64_t hi = min(total, lo + per);
  long long sp = 0, ss = 0;
  for (int64_t i = lo; i < hi; ++i) {
    sp += count[i];
    if (i < nbins) ss += (count[i] + max_sub - 1) / max_sub;
  }
  s_pts[tid] = sp;
  s_sub[tid] = ss;
  __syncthreads();
  for (int ofs = 1; ofs < (int)blockDim.x; ofs <<= 1) {
    long long ap = tid >= ofs ? s_pts[tid - ofs] : 0;
    long long as = tid >= ofs ? s_sub[tid - ofs] : 0;
    __syncthreads();
    s_pts[tid] += ap;
    s_sub[tid] += as;
    __syncthreads();
  }
  long long rp = s_pts[tid] - sp;
  long long rs = s_sub[tid] - ss;
  for (int64_t i = lo; i < hi; ++i) {
    off[i] = (int)rp;
    rp += count[i];
    if (i < nbins) {
      sub_off[i] = (int)rs;
      rs += (count[i] + max_sub - 1) / max_sub;
    }
  }
  if (tid == blockDim.x - 1) {
    off[total] = (int)s_pts[tid];
    *nsub = (int)s_sub[tid];
  }
}

__global__ void scatter_kernel(PointGeom g, int64_t M, const int *__restrict__ pt_bin, const int *__restrict__ pt_rank,
                               const int *__restrict__ off, SortedPoint *__restrict__ sorted) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= M) return;
  const int pos = off[pt_bin[id]] + pt_rank[id];
  float t[3];
  point_index(g, id, t);
  SortedPoint sp;
  sp.t0 = t[0];
  sp.t1 = t[1];
  sp.t2 = t[2];
  sp.idf = (int)id | (on_nyquist(g, id) ? kNyquistBit : 0);
  sorted[pos] = sp;
}

__global__ void subproblem_kernel(int64_t nbins, int max_sub, const int *__restrict__ count,
                                  const int *__restrict__ off, const int *__restrict__ sub_off,
                                  int *__restrict__ sub_bin, int *__restrict__ sub_first, int *__restrict__ sub_count) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const int c = count[b];
  const int s0 = sub_off[b];
  for (int s = 0; s * max_sub < c; ++s) {
    sub_bin[s0 + s] = (int)b;
    sub_first[s0 + s] = off[b] + s * max_sub;
    sub_count[s0 + s] = min(max_sub, c - s * max_sub);
  }
}

template <int KT, int W>
void launch_count(cov3d_plan *p, const PointGeom &g, const KernelSpec &k, int blocks) {
  bin_count_kernel<KT, W><<<blocks, 256, 0, p->stream>>>(g, k, p->bins, p->n_points, p->bin_count.as<int>(), p->pt_bin.as<int>(),
                                                        p->pt_rank.as<int>());
}

}  // namespace

// Every buffer the sort of M points uses (a no-op when they are large enough already).
int reserve_sort(cov3d_plan *p, int64_t M) {
  const int64_t nb = p->bins.nbins;
  const int64_t max_subs = nb + M / p->max_sub + 1;
  COV3D_TRY(grow(p->bin_count, (nb + 2) * 4));
  COV3D_TRY(grow(p->bin_off, (nb + 2) * 4));
  COV3D_TRY(grow(p->sub_off, (nb + 2) * 4));
  COV3D_TRY(grow(p->pt_bin, M * 4));
  COV3D_TRY(grow(p->pt_rank, M * 4));
  COV3D_TRY(grow(p->sorted, M * (int64_t)sizeof(SortedPoint)));
  COV3D_TRY(grow(p->sub_bin, max_subs * 4));
  COV3D_TRY(grow(p->sub_first, max_subs * 4));
  COV3D_TRY(grow(p->sub_count, max_subs * 4));
  COV3D_TRY(grow(p->nsub, 16));
  return COV3D_OK;
}

int sort_points(cov3d_plan *p) {
  const int64_t M = p->n_points;
  if (M <= 0) return COV3D_OK;
  if (M >= (int64_t)(1 << 30)) {
    set_error("too many points (%lld); the limit is 2^30-1 per plan", (long long)M);
    return COV3D_EINVAL;
  }
  COV3D_TRY(reserve_sort(p, M));
  const int64_t nb = p->bins.nbins;

  COV3D_CUDA(cudaMemsetAsync(p->bin_count.as<int>(), 0, (nb + 1) * sizeof(int), p->stream));
  const PointGeom g = make_geom(p);
  const KernelSpec k = make_kernel(p);
  const int blocks = (int)((M + 255) / 256);
  switch (p->kernel) {
    case COV3D_KERNEL_NEAREST: launch_count<COV3D_KERNEL_NEAREST, 1>(p, g, k, blocks); break;
    case COV3D_KERNEL_LINEAR: launch_count<COV3D_KERNEL_LINEAR, 2>(p, g, k, blocks); break;
    default:
      switch (p->width) {
#define COV3D_W(Wv) \
  case Wv: launch_count<COV3D_KERNEL_ES, Wv>(p, g, k, blocks); break;
        COV3D_W(2) COV3D_W(3) COV3D_W(4) COV3D_W(5) COV3D_W(6) COV3D_W(7) COV3D_W(8) COV3D_W(9) COV3D_W(10)
        COV3D_W(11) COV3D_W(12) COV3D_W(13) COV3D_W(14) COV3D_W(15) COV3D_W(16)
#undef COV3D_W
        default:
          set_error("unsupported ES width %d", p->width);
          return COV3D_EINVAL;
      }
  }
  COV3D_LAUNCHED("bin_count_kernel");
  bin_scan_kernel<<<1, 1024, 0, p->stream>>>(p->bin_count.as<int>(), nb, p->max_sub, p->bin_off.as<int>(), p->sub_off.as<int>(), p->nsub.as<int>());
  COV3D_LAUNCHED("bin_scan_kernel");
  scatter_kernel<<<blocks, 256, 0, p->stream>>>(g, M, p->pt_bin.as<int>(), p->pt_rank.as<int>(), p->bin_off.as<int>(),
                                                p->sorted.as<SortedPoint>());
  COV3D_LAUNCHED("scatter_kernel");
  subproblem_kernel<<<(int)((nb + 255) / 256), 256, 0, p->stream>>>(nb, p->max_sub, p->bin_count.as<int>(), p->bin_off.as<int>(),
                                                                    p->sub_off.as<int>(), p->sub_bin.as<int>(), p->sub_first.as<int>(),
                                                                    p->sub_count.as<int>());
  COV3D_LAUNCHED("subproblem_kernel");
  return COV3D_OK;
}

}  // namespace cov3d
