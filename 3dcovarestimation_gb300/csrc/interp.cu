// Interpolation ("type-2" half of the NUFFT, and the reference's grid_sample forward):
// one thread per nonuniform point, visited in bin-sorted order so that the warps of a block
// gather overlapping neighbourhoods of the fine grid through L1.  All channels of a pass are
// accumulated in registers from channels-last cells (one 16-byte vector load per two complex
// channels), and the projection epilogue (Nyquist zeroing, CTF multiply, 1/L) is fused.
#include "cov3d_device.cuh"

namespace cov3d {

namespace {

struct InterpParams {
  PointGeom g;
  KernelSpec k;
  int64_t M;
  const int *perm;
  const float2 *grid;
  int64_t cs, chs;
  int shift;
  int ch0;
  float2 *out;
  int64_t ops, ocs;
  const float *ctf;
  int nyquist;
  float scale;
};

template <int KT, int W, int CH, bool CONTIG>
__global__ void __launch_bounds__(256) interp_kernel(const InterpParams a) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.M) return;
  const int64_t id = a.perm ? (int64_t)__ldg(a.perm + k) : k;
  const int n = a.g.n;
  float t[3];
  point_index(a.g, id, t);
  float wt[3][W];
  int s[3][W];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int c0 = taps<KT, W>(t[d], a.k.beta, wt[d]);
#pragma unroll
    for (int j = 0; j < W; ++j) {
      int m = c0 + j;
      if (KT == COV3D_KERNEL_ES) {
        m = pmod(m, n);
      } else if (m < 0 || m >= n) {
        wt[d][j] = 0.0f;
        m = 0;
      }
      m += a.shift;
      s[d][j] = m >= n ? m - n : m;
    }
  }
  float2 acc[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) acc[c] = make_float2(0.f, 0.f);
  const float2 *gbase = a.grid + a.ch0 * a.chs;
#pragma unroll 1
  for (int i0 = 0; i0 < W; ++i0) {
#pragma unroll
    for (int i1 = 0; i1 < W; ++i1) {
      const float wab = wt[0][i0] * wt[1][i1];
      if (KT != COV3D_KERNEL_ES && wab == 0.0f) continue;
      const int64_t row = ((int64_t)s[0][i0] * n + s[1][i1]) * n;
#pragma unroll
      for (int i2 = 0; i2 < W; ++i2) {
        const float w = wab * wt[2][i2];
        if (KT != COV3D_KERNEL_ES && w == 0.0f) continue;
        const float2 *cell = gbase + (row + s[2][i2]) * a.cs;
        if (CONTIG) {
          const float4 *c4 = reinterpret_cast<const float4 *>(cell);
#pragma unroll
          for (int c = 0; c < CH / 2; ++c) {
            const float4 v = __ldg(c4 + c);
            acc[2 * c].x = fmaf(w, v.x, acc[2 * c].x);
            acc[2 * c].y = fmaf(w, v.y, acc[2 * c].y);
            acc[2 * c + 1].x = fmaf(w, v.z, acc[2 * c + 1].x);
            acc[2 * c + 1].y = fmaf(w, v.w, acc[2 * c + 1].y);
          }
        } else {
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            const float2 v = __ldg(cell + c * a.chs);
            acc[c].x = fmaf(w, v.x, acc[c].x);
            acc[c].y = fmaf(w, v.y, acc[c].y);
          }
        }
      }
    }
  }
  // epilogue: vol_forward's Nyquist zeroing, CTF multiply and 1/L (projection_funcs.py:355-370)
  const int64_t b = id / a.g.P;
  const int p = (int)(id - b * a.g.P);
  float sc = a.scale;
  if (a.nyquist && (a.g.Lp % 2 == 0)) {
    const int row = p / a.g.Lp;
    const int col = p - row * a.g.Lp;
    if (row == 0 || col == 0) sc = 0.0f;
  }
  if (a.ctf) sc *= __ldg(a.ctf + id);
  float2 *o = a.out + id * a.ops + (int64_t)a.ch0 * a.ocs;
#pragma unroll
  for (int c = 0; c < CH; ++c) o[c * a.ocs] = make_float2(acc[c].x * sc, acc[c].y * sc);
}

template <int KT, int W, int CH>
int launch_ch(const InterpParams &a, bool contig, cudaStream_t st) {
  const int blocks = (int)((a.M + 255) / 256);
  if (CH % 2 == 0 && contig) {
    interp_kernel<KT, W, CH, (CH % 2 == 0)><<<blocks, 256, 0, st>>>(a);
  } else {
    interp_kernel<KT, W, CH, false><<<blocks, 256, 0, st>>>(a);
  }
  return launched("interp_kernel");
}

template <int KT, int W>
int launch_w(InterpParams a, int nchan, cudaStream_t st) {
  int done = 0;
  while (done < nchan) {
    const int left = nchan - done;
    const int ch = left >= 16 ? 16 : left >= 10 ? 10 : left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
    a.ch0 = done;
    const bool contig = a.chs == 1 && (a.cs % 2 == 0) && (done % 2 == 0) &&
                        ((reinterpret_cast<uintptr_t>(a.grid) & 15) == 0);
    int st_ = COV3D_OK;
    switch (ch) {
      case 16: st_ = launch_ch<KT, W, 16>(a, contig, st); break;
      case 10: st_ = launch_ch<KT, W, 10>(a, contig, st); break;
      case 8: st_ = launch_ch<KT, W, 8>(a, contig, st); break;
      case 4: st_ = launch_ch<KT, W, 4>(a, contig, st); break;
      case 2: st_ = launch_ch<KT, W, 2>(a, contig, st); break;
      default: st_ = launch_ch<KT, W, 1>(a, contig, st); break;
    }
    if (st_ != COV3D_OK) return st_;
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
  a.M = p->n_points;
  a.perm = p->perm.as<int>();
  a.grid = static_cast<const float2 *>(ga.grid);
  a.cs = ga.cell_stride;
  a.chs = ga.chan_stride;
  a.shift = ga.shift;
  a.out = static_cast<float2 *>(out);
  a.ops = out_ps;
  a.ocs = out_cs;
  a.ctf = e.ctf;
  a.nyquist = e.nyquist;
  a.scale = e.scale;
  switch (p->kernel) {
    case COV3D_KERNEL_NEAREST: return launch_w<COV3D_KERNEL_NEAREST, 1>(a, nchan, p->stream);
    case COV3D_KERNEL_LINEAR: return launch_w<COV3D_KERNEL_LINEAR, 2>(a, nchan, p->stream);
    default:
      switch (p->width) {
        case 4: return launch_w<COV3D_KERNEL_ES, 4>(a, nchan, p->stream);
        case 5: return launch_w<COV3D_KERNEL_ES, 5>(a, nchan, p->stream);
        case 6: return launch_w<COV3D_KERNEL_ES, 6>(a, nchan, p->stream);
        case 7: return launch_w<COV3D_KERNEL_ES, 7>(a, nchan, p->stream);
        case 8: return launch_w<COV3D_KERNEL_ES, 8>(a, nchan, p->stream);
        default: set_error("unsupported ES width %d (supported: 4..8)", p->width); return COV3D_EINVAL;
      }
  }
}

}  // namespace cov3d
