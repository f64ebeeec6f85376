// Per-image r x r contractions of the covariance cost and its hand-written adjoint.
//
// For image b with projections Q_b (P x r, the CTF-weighted central-slice samples of the r
// Fourier-domain eigenvolumes, projection_funcs.py:321-370) and Fourier image y_b:
//   gram_ij = sum_p conj(Q_pi) Q_pj,  h_i = sum_p conj(Q_pi) y_p
// ML objective (raw_cost_maximum_liklihood_fourier_domain, covar_sgd.py:1381-1399, through
// compute_latentMAP_batch, wiener_coords.py:168-203):
//   m = gram / s2 + I,  b = h / s2,  z = m^-1 b,  cost_b = (-Re(b^H z) + logdet m) / 2
//   dcost_b / d conj(Q_pi) = sum_j C_ij Q_pj + u_i y_p,
//   C = (conj(m^-1) + conj(z) z^T) / (2 s2),  u = -conj(z) / (2 s2)
// LS objective (raw_cost_fourier_domain, covar_sgd.py:1320-1347), M = conj(gram), t = conj(h):
//   cost_b = -2 |t|^2 + ||M||_F^2 + 2 s2 tr M,  C = 2 M + 2 s2 I,  u = -2 t
// The r x r factorisations run in FP64 (one thread per image).
#include "cov3d_device.cuh"

namespace cov3d {

namespace {

constexpr int kMaxRank = 32;
constexpr int kGramChunk = 128;

// One block per image: chunks of pixels are staged in shared memory; every thread owns one
// (job, pixel-group) pair where a job is one entry of the upper triangle of gram, one h_i,
// or |y|^2.  Partial sums per chunk are added to a Kahan-compensated running total.
__global__ void __launch_bounds__(1024) gram_kernel(const float2 *__restrict__ Q, int64_t q_is, int64_t q_ps,
                                                    int64_t q_cs, const float2 *__restrict__ Y, int P, int r,
                                                    float2 *__restrict__ gram, float2 *__restrict__ h,
                                                    float *__restrict__ yy) {
  extern __shared__ float2 sq[];  // kGramChunk * (r + 1)
  const int b = blockIdx.x;
  const int ntri = r * (r + 1) / 2;
  const int J = ntri + r + 1;
  const int groups = max(1, (int)blockDim.x / J);
  const int tid = threadIdx.x;
  const int job = tid % J;
  const int grp = tid / J;
  const bool active = grp < groups;
  int ji = 0, jj = 0, kind = 0;
  if (job < ntri) {
    int q = job, i = 0;
    while (q >= r - i) {
      q -= r - i;
      ++i;
    }
    ji = i;
    jj = i + q;
    kind = 0;
  } else if (job < ntri + r) {
    ji = job - ntri;
    kind = 1;
  } else {
    kind = 2;
  }
  float2 sum = make_float2(0.f, 0.f), comp = make_float2(0.f, 0.f);
  const float2 *Qb = Q + (int64_t)b * q_is;
  const float2 *Yb = Y + (int64_t)b * P;
  float2 *sy = sq + kGramChunk * r;
  for (int p0 = 0; p0 < P; p0 += kGramChunk) {
    const int np = min(kGramChunk, P - p0);
    __syncthreads();
    if (q_cs == 1) {
      for (int e = tid; e < np * r; e += blockDim.x) {
        const int pp = e / r, i = e - pp * r;
        sq[e] = Qb[(int64_t)(p0 + pp) * q_ps + i];
      }
    } else {
      for (int e = tid; e < np * r; e += blockDim.x) {
        const int i = e / np, pp = e - i * np;
        sq[pp * r + i] = Qb[(int64_t)(p0 + pp) * q_ps + (int64_t)i * q_cs];
      }
    }
    for (int e = tid; e < np; e += blockDim.x) sy[e] = Yb[p0 + e];
    __syncthreads();
    if (!active) continue;
    float2 part = make_float2(0.f, 0.f);
    for (int p = grp; p < np; p += groups) {
      float2 a, c;
      if (kind == 2) {
        a = sy[p];
        c = a;
      } else {
        a = sq[p * r + ji];
        c = kind == 0 ? sq[p * r + jj] : sy[p];
      }
      // conj(a) * c
      part.x = fmaf(a.x, c.x, fmaf(a.y, c.y, part.x));
      part.y = fmaf(a.x, c.y, fmaf(-a.y, c.x, part.y));
    }
    // Kahan update of the running total
    float yx = part.x - comp.x, tx = sum.x + yx;
    comp.x = (tx - sum.x) - yx;
    sum.x = tx;
    float yyv = part.y - comp.y, ty = sum.y + yyv;
    comp.y = (ty - sum.y) - yyv;
    sum.y = ty;
  }
  __syncthreads();
  // reduce over pixel groups
  float2 *red = sq;
  if (active) red[grp * J + job] = sum;
  __syncthreads();
  if (active && grp == 0) {
    float2 tot = sum;
    for (int g = 1; g < groups; ++g) {
      tot.x += red[g * J + job].x;
      tot.y += red[g * J + job].y;
    }
    if (kind == 0) {
      gram[((int64_t)b * r + ji) * r + jj] = tot;
      if (ji != jj) gram[((int64_t)b * r + jj) * r + ji] = make_float2(tot.x, -tot.y);
    } else if (kind == 1) {
      h[(int64_t)b * r + ji] = tot;
    } else {
      yy[b] = tot.x;
    }
  }
}

// (i, j) of product k of the upper triangle (0 <= i <= j < R1), row-major
template <int R1>
__host__ __device__ constexpr int tri_i(int k) {
  int i = 0;
  while (k >= R1 - i) {
    k -= R1 - i;
    ++i;
  }
  return i;
}
template <int R1>
__host__ __device__ constexpr int tri_j(int k) {
  int i = 0;
  while (k >= R1 - i) {
    k -= R1 - i;
    ++i;
  }
  return i + k;
}

constexpr int kGramSubsets = 8;   // product subsets per image (2 warps each)
constexpr int kGramLanes = 64;    // threads per subset, striding over the pixels

// part[KK] += conj(v[i]) * v[j] for product k = S + kGramSubsets * KK, indices fixed at
// compile time so the pixel stays in registers
template <int R1, int S, int KK, int PER>
struct GramAcc {
  __device__ __forceinline__ static void run(const float2 (&v)[R1], float2 (&part)[PER]) {
    constexpr int k = S + kGramSubsets * KK;
    if constexpr (k < R1 * (R1 + 1) / 2) {
      constexpr int i = tri_i<R1>(k), j = tri_j<R1>(k);
      const float2 a = v[i], c = v[j];
      part[KK].x = fmaf(a.x, c.x, fmaf(a.y, c.y, part[KK].x));
      part[KK].y = fmaf(a.x, c.y, fmaf(-a.y, c.x, part[KK].y));
    }
    if constexpr (KK + 1 < PER) GramAcc<R1, S, KK + 1, PER>::run(v, part);
  }
};

// One staged chunk of pixels for the products k = S, S + kGramSubsets, ... of this subset:
// part[kk] += conj(v[i]) * v[j] with v a pixel's r projections and y (row of R + 1 in shared
// memory, read into registers)
template <int R, int S, int PER>
__device__ __forceinline__ void gram_chunk(const float2 *rows, int np, int lane, float2 (&part)[PER]) {
  constexpr int R1 = R + 1;
  for (int p = lane; p < np; p += kGramLanes) {
    float2 v[R1];
#pragma unroll
    for (int i = 0; i < R1; ++i) v[i] = rows[p * R1 + i];
    GramAcc<R1, S, 0, PER>::run(v, part);
  }
}

constexpr int kGramChunkPx = kGramSubsets * kGramLanes;  // pixels staged per chunk
constexpr int kGramBufs = 2;  // staging buffers (a third measured no faster)

// Per-image Gram for the fused step's layout (point-major Q with r contiguous projections per
// pixel): one block per image, eight product subsets of two warps.  Chunks of kGramChunkPx
// pixels are staged in shared memory by coalesced 8-byte asynchronous copies (double-buffered)
// as rows of r projections and y, 88 bytes apart at r = 10 so the subsets' 8-byte reads are
// free of bank conflicts; every subset reads every pixel of the chunk from there, and each
// thread adds its chunk sums to Kahan-compensated totals.
template <int R>
__global__ void __launch_bounds__(kGramSubsets * kGramLanes, 1) gram_pixel_kernel(
    const float2 *__restrict__ Q, int64_t q_is, const float2 *__restrict__ Y, int P, float2 *__restrict__ gram,
    float2 *__restrict__ h, float *__restrict__ yy) {
  constexpr int R1 = R + 1, NPR = R1 * (R1 + 1) / 2, PER = (NPR + kGramSubsets - 1) / kGramSubsets;
  constexpr int NT = kGramSubsets * kGramLanes;
  extern __shared__ float2 srows[];  // kGramBufs * kGramChunkPx * R1
  const int b = blockIdx.x;
  const int sub = threadIdx.x / kGramLanes, lane = threadIdx.x % kGramLanes;
  float2 sum[PER], comp[PER];
#pragma unroll
  for (int kk = 0; kk < PER; ++kk) {
    sum[kk] = make_float2(0.f, 0.f);
    comp[kk] = make_float2(0.f, 0.f);
  }
  const float2 *Qb = Q + (int64_t)b * q_is;
  const float2 *Yb = Y + (int64_t)b * P;
  auto stage = [&](int c, float2 *dst) {
    const int p0 = c * kGramChunkPx, np = min(kGramChunkPx, P - p0);
    const float2 *src = Qb + (int64_t)p0 * R;
    for (int e = threadIdx.x; e < np * R; e += NT) {
      const int p = e / R, i = e - p * R;
      const unsigned d = (unsigned)__cvta_generic_to_shared(dst + p * R1 + i);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src + e) : "memory");
    }
    for (int p = threadIdx.x; p < np; p += NT) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(dst + p * R1 + R);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(Yb + p0 + p) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  const int nchunks = (P + kGramChunkPx - 1) / kGramChunkPx;
  // kGramBufs - 1 chunks in flight ahead of the one being summed; a buffer is refilled after the
  // barrier that ends the iteration which read it
  for (int c = 0; c < kGramBufs - 1; ++c) {
    if (c < nchunks) stage(c, srows + c * kGramChunkPx * R1);
    else asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  for (int c = 0; c < nchunks; ++c) {
    const float2 *cur = srows + (c % kGramBufs) * kGramChunkPx * R1;
    const int cn = c + kGramBufs - 1;
    if (cn < nchunks) stage(cn, srows + (cn % kGramBufs) * kGramChunkPx * R1);
    else asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group %0;\n" ::"n"(kGramBufs - 1) : "memory");
    __syncthreads();
    const int np = min(kGramChunkPx, P - c * kGramChunkPx);
    float2 part[PER];
#pragma unroll
    for (int kk = 0; kk < PER; ++kk) part[kk] = make_float2(0.f, 0.f);
    switch (sub) {
      case 0: gram_chunk<R, 0, PER>(cur, np, lane, part); break;
      case 1: gram_chunk<R, 1, PER>(cur, np, lane, part); break;
      case 2: gram_chunk<R, 2, PER>(cur, np, lane, part); break;
      case 3: gram_chunk<R, 3, PER>(cur, np, lane, part); break;
      case 4: gram_chunk<R, 4, PER>(cur, np, lane, part); break;
      case 5: gram_chunk<R, 5, PER>(cur, np, lane, part); break;
      case 6: gram_chunk<R, 6, PER>(cur, np, lane, part); break;
      default: gram_chunk<R, 7, PER>(cur, np, lane, part); break;
    }
#pragma unroll
    for (int kk = 0; kk < PER; ++kk) {  // Kahan update of the running totals
      float yx = part[kk].x - comp[kk].x, tx = sum[kk].x + yx;
      comp[kk].x = (tx - sum[kk].x) - yx;
      sum[kk].x = tx;
      float yv = part[kk].y - comp[kk].y, ty = sum[kk].y + yv;
      comp[kk].y = (ty - sum[kk].y) - yv;
      sum[kk].y = ty;
    }
    __syncthreads();  // the buffer is refilled next
  }
  // reduce over the 64 lanes of the subset: shuffles within each warp, then the two warps
  __shared__ float2 red[kGramSubsets][2][PER];
  const int w = lane >> 5;
#pragma unroll
  for (int kk = 0; kk < PER; ++kk) {
    float x = sum[kk].x, y = sum[kk].y;
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if ((lane & 31) == 0) red[sub][w][kk] = make_float2(x, y);
  }
  __syncthreads();
  if (lane < PER) {
    const int kk = lane;
    const int k = sub + kGramSubsets * kk;
    if (k < NPR) {
      const float2 t = make_float2(red[sub][0][kk].x + red[sub][1][kk].x, red[sub][0][kk].y + red[sub][1][kk].y);
      int i = 0, kr = k;
      while (kr >= R1 - i) {
        kr -= R1 - i;
        ++i;
      }
      const int j = i + kr;
      if (j < R) {
        gram[((int64_t)b * R + i) * R + j] = t;
        if (i != j) gram[((int64_t)b * R + j) * R + i] = make_float2(t.x, -t.y);
      } else if (i < R) {
        h[(int64_t)b * R + i] = t;
      } else {
        yy[b] = t.x;
      }
    }
  }
}

struct cd {
  double x, y;
};
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd cconj(cd a) { return {a.x, -a.y}; }
__device__ __forceinline__ cd csub(cd a, cd b) { return {a.x - b.x, a.y - b.y}; }

// In-place Cholesky m = L L^H (lower triangle); returns log det m, NaN if m is not positive
// definite.  The diagonal entry (k, k) holds {L_kk, 1 / L_kk}, so the triangular solves
// multiply instead of dividing.
__device__ double chol_logdet(cd *m, int r) {
  double logdet = 0.0;
  for (int k = 0; k < r; ++k) {
    double d = m[k * r + k].x;
    for (int j = 0; j < k; ++j) d -= m[k * r + j].x * m[k * r + j].x + m[k * r + j].y * m[k * r + j].y;
    if (!(d > 0.0)) return __longlong_as_double(0x7ff8000000000000ULL);
    const double lkk = sqrt(d), inv = 1.0 / lkk;
    m[k * r + k] = {lkk, inv};
    logdet += 2.0 * log(lkk);
    for (int i = k + 1; i < r; ++i) {
      cd s = m[i * r + k];
      for (int j = 0; j < k; ++j) s = csub(s, cmul(m[i * r + j], cconj(m[k * r + j])));
      m[i * r + k] = {s.x * inv, s.y * inv};
    }
  }
  return logdet;
}

// Solve (L L^H) x = rhs in place, L from chol_logdet.
__device__ void chol_solve(const cd *Lm, int r, cd *x) {
  for (int i = 0; i < r; ++i) {
    cd s = x[i];
    for (int j = 0; j < i; ++j) s = csub(s, cmul(Lm[i * r + j], x[j]));
    const double inv = Lm[i * r + i].y;
    x[i] = {s.x * inv, s.y * inv};
  }
  for (int i = r - 1; i >= 0; --i) {
    cd s = x[i];
    for (int j = i + 1; j < r; ++j) s = csub(s, cmul(cconj(Lm[j * r + i]), x[j]));
    const double inv = Lm[i * r + i].y;
    x[i] = {s.x * inv, s.y * inv};
  }
}

struct SolveArgs {
  int B, r, objective;
  const float2 *gram;
  const float2 *h;
  const float *yy;
  double s2;
  const double *linv;  // (r, r) real symmetric added to gram/s2, or null (identity)
  double wscale;       // scale of C and u (1/B for ML, 1/(B L^4) for LS)
  double cscale;       // scale of the per-image cost
  float2 *C;           // (B, r, r)
  float2 *u;           // (B, r)
  double *cost_b;      // (B) or null
  double *cost_sum;    // scalar accumulator
  float2 *z_out;       // (B, r) latent coordinates or null
  float2 *m_out;       // (B, r, r) m or null
  int *bad;            // set to 1 if a factorisation failed
};

// Thread kc of image b.  Every one of the image's r threads factors m (the same arithmetic,
// so the same bits) and solves for z; thread kc then writes column kc of C from column kc of
// m^-1, and thread 0 the per-image outputs (cost, z, m, u).  RMAX sizes the per-thread
// working arrays (local memory): the smallest class that holds r keeps them in L1.
template <int RMAX>
__device__ double solve_one(const SolveArgs &a, const int b, const int kc) {
  const int r = a.r;
  cd m[RMAX * RMAX];
  cd z[RMAX];
  cd bb[RMAX];
  const float2 *G = a.gram + (int64_t)b * r * r;
  const float2 *hb = a.h + (int64_t)b * r;
  double cost = 0.0;
  if (a.objective == 0) {
    for (int i = 0; i < r; ++i) {
      for (int j = 0; j < r; ++j) {
        const float2 g = G[i * r + j];
        double add = a.linv ? a.linv[i * r + j] : (i == j ? 1.0 : 0.0);
        m[i * r + j] = {g.x / a.s2 + add, g.y / a.s2};
      }
      bb[i] = {hb[i].x / a.s2, hb[i].y / a.s2};
    }
    if (a.m_out && kc == 0) {
      for (int i = 0; i < r * r; ++i) a.m_out[(int64_t)b * r * r + i] = make_float2((float)m[i].x, (float)m[i].y);
    }
    const double logdet = chol_logdet(m, r);
    if (!(logdet == logdet)) {
      atomicExch(a.bad, 1);
      return 0.0;
    }
    for (int i = 0; i < r; ++i) z[i] = bb[i];
    chol_solve(m, r, z);
    double bz = 0.0;
    for (int i = 0; i < r; ++i) bz += bb[i].x * z[i].x + bb[i].y * z[i].y;
    cost = 0.5 * (-bz + logdet);
    if (a.z_out && kc == 0) {
      for (int i = 0; i < r; ++i) a.z_out[(int64_t)b * r + i] = make_float2((float)z[i].x, (float)z[i].y);
    }
    if (a.C) {
      // column kc of m^-1: solve m x = e_kc; C_ij = (conj(minv_ij) + conj(z_i) z_j) / (2 s2)
      const double f = a.wscale / (2.0 * a.s2);
      cd col[RMAX];
      for (int i = 0; i < r; ++i) col[i] = {i == kc ? 1.0 : 0.0, 0.0};
      chol_solve(m, r, col);
      for (int i = 0; i < r; ++i) {
        const cd zz = cmul(cconj(z[i]), z[kc]);
        a.C[((int64_t)b * r + i) * r + kc] = make_float2((float)((col[i].x + zz.x) * f), (float)((-col[i].y + zz.y) * f));
      }
      if (kc == 0) {
        for (int i = 0; i < r; ++i) a.u[(int64_t)b * r + i] = make_float2((float)(-z[i].x * f), (float)(z[i].y * f));
      }
    }
  } else {
    // least squares (thread 0 of the image)
    if (kc != 0) return 0.0;
    double t2 = 0.0, fro = 0.0, tr = 0.0;
    for (int i = 0; i < r; ++i) {
      t2 += (double)hb[i].x * hb[i].x + (double)hb[i].y * hb[i].y;
      tr += G[i * r + i].x;
      for (int j = 0; j < r; ++j) fro += (double)G[i * r + j].x * G[i * r + j].x + (double)G[i * r + j].y * G[i * r + j].y;
    }
    cost = -2.0 * t2 + fro + 2.0 * a.s2 * tr;
    if (a.C) {
      const double f = a.wscale;
      for (int i = 0; i < r; ++i) {
        for (int j = 0; j < r; ++j) {
          const float2 g = G[i * r + j];  // M_ij = conj(gram_ij)
          a.C[((int64_t)b * r + i) * r + j] =
              make_float2((float)((2.0 * g.x + (i == j ? 2.0 * a.s2 : 0.0)) * f), (float)(-2.0 * g.y * f));
        }
        // u_i = -2 t_i = -2 conj(h_i)
        a.u[(int64_t)b * r + i] = make_float2((float)(-2.0 * hb[i].x * f), (float)(2.0 * hb[i].y * f));
      }
    }
  }
  if (kc != 0) return 0.0;
  cost *= a.cscale;
  if (a.cost_b) a.cost_b[b] = cost;
  return cost;
}

constexpr int kSolveThreads = 128;

// r threads per image, kSolveThreads / r images per block; the images' costs are summed per
// block (one FP64 atomic per block instead of one per image on the same address)
template <int RMAX>
__global__ void __launch_bounds__(kSolveThreads) solve_kernel(const SolveArgs a) {
  const int ipb = kSolveThreads / a.r;
  const int b = blockIdx.x * ipb + threadIdx.x / a.r;
  const int kc = threadIdx.x - (threadIdx.x / a.r) * a.r;
  double cost = (threadIdx.x < ipb * a.r && b < a.B) ? solve_one<RMAX>(a, b, kc) : 0.0;
  if (!a.cost_sum) return;
  for (int o = 16; o > 0; o >>= 1) cost += __shfl_xor_sync(0xffffffffu, cost, o);
  __shared__ double wsum[kSolveThreads / 32];
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cost;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < kSolveThreads / 32; ++i) t += wsum[i];
    atomicAdd(a.cost_sum, t);
  }
}

// W = C Q + u y on chunks of pixels of one image (Q element (p, i) at
// Q[b*q_is + p*q_ps + i*q_cs], W likewise with its own strides; W may alias Q).
__global__ void __launch_bounds__(256) wpass_kernel(const float2 *Q, int64_t q_is, int64_t q_ps, int64_t q_cs,
                                                    const float2 *__restrict__ Y, const float2 *__restrict__ C,
                                                    const float2 *__restrict__ u, int P, int r, float2 *W,
                                                    int64_t w_is, int64_t w_ps, int64_t w_cs) {
  extern __shared__ float2 sw[];
  float2 *sC = sw;                    // r*r
  float2 *su = sC + r * r;            // r
  float2 *sq = su + r;                // kGramChunk * r
  float2 *sy = sq + kGramChunk * r;   // kGramChunk
  const int b = blockIdx.y;
  const int p0 = blockIdx.x * kGramChunk;
  const int np = min(kGramChunk, P - p0);
  const int tid = threadIdx.x;
  for (int e = tid; e < r * r; e += blockDim.x) sC[e] = C[(int64_t)b * r * r + e];
  for (int e = tid; e < r; e += blockDim.x) su[e] = u[(int64_t)b * r + e];
  const float2 *Qb = Q + (int64_t)b * q_is;
  for (int e = tid; e < np * r; e += blockDim.x) {
    const int pp = e / r, i = e - pp * r;
    sq[e] = Qb[(int64_t)(p0 + pp) * q_ps + (int64_t)i * q_cs];
  }
  for (int e = tid; e < np; e += blockDim.x) sy[e] = Y[(int64_t)b * P + p0 + e];
  __syncthreads();
  float2 *Wb = W + (int64_t)b * w_is;
  for (int e = tid; e < np * r; e += blockDim.x) {
    const int p = e / r, i = e - p * r;
    const float2 yv = sy[p];
    const float2 ui = su[i];
    float2 acc = make_float2(ui.x * yv.x - ui.y * yv.y, ui.x * yv.y + ui.y * yv.x);
    const float2 *crow = sC + i * r;
    const float2 *qp = sq + p * r;
    for (int j = 0; j < r; ++j) {
      const float2 c = crow[j], q = qp[j];
      acc.x = fmaf(c.x, q.x, fmaf(-c.y, q.y, acc.x));
      acc.y = fmaf(c.x, q.y, fmaf(c.y, q.x, acc.y));
    }
    Wb[(int64_t)(p0 + p) * w_ps + (int64_t)i * w_cs] = acc;
  }
}

// wpass for the fused step's layout (point-major, channel stride 1, W over Q in place): one
// thread per pixel holds its r projections and y in registers (16-byte loads), C and u are
// broadcast from shared memory, the r outputs are written back over the pixel's Q (16-byte
// stores).
template <int R>
__global__ void __launch_bounds__(256) wpass_pixel_kernel(float2 *QW, int64_t q_is, int64_t q_ps,
                                                          const float2 *__restrict__ Y, const float2 *__restrict__ C,
                                                          const float2 *__restrict__ u, int P) {
  __shared__ float2 sC[R * R], su[R];
  const int b = blockIdx.y;
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) sC[e] = C[(int64_t)b * R * R + e];
  for (int e = threadIdx.x; e < R; e += blockDim.x) su[e] = u[(int64_t)b * R + e];
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  float2 *qp = QW + (int64_t)b * q_is + (int64_t)p * q_ps;
  float2 q[R];
  // the pixel's R complex values as R/2 16-byte loads (R even, rows 16-byte aligned: checked
  // by the launcher; 0.69 -> 0.56 ms against 8-byte loads)
  float4 *qp4 = reinterpret_cast<float4 *>(qp);
#pragma unroll
  for (int j = 0; j < R / 2; ++j) {
    const float4 v = qp4[j];
    q[2 * j] = make_float2(v.x, v.y);
    q[2 * j + 1] = make_float2(v.z, v.w);
  }
  const float2 yv = Y[(int64_t)b * P + p];
  float2 w[R];
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const float2 ui = su[i];
    float2 acc = make_float2(ui.x * yv.x - ui.y * yv.y, ui.x * yv.y + ui.y * yv.x);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 c = sC[i * R + j];
      acc.x = fmaf(c.x, q[j].x, fmaf(-c.y, q[j].y, acc.x));
      acc.y = fmaf(c.x, q[j].y, fmaf(c.y, q[j].x, acc.y));
    }
    w[i] = acc;
  }
#pragma unroll
  for (int i = 0; i < R / 2; ++i) qp4[i] = make_float4(w[2 * i].x, w[2 * i].y, w[2 * i + 1].x, w[2 * i + 1].y);
}

__global__ void finalize_kernel(const double *acc, int r, double inv_count, double *d_cost, float *glog) {
  const int i = threadIdx.x;
  if (i == 0 && d_cost) *d_cost = acc[0] * inv_count + acc[1];
  if (i < r && glog) glog[i] = (float)acc[8 + i];
}

}  // namespace

int launch_gram(cudaStream_t st, int B, int P, int r, const void *q, int64_t is, int64_t ps, int64_t cs,
                const void *images, void *gram, void *h, float *yy) {
  if (r < 1 || r > kMaxRank) {
    set_error("rank %d out of range (1..%d)", r, kMaxRank);
    return COV3D_EINVAL;
  }
  if (cs == 1 && ps == r && r == 10) {
    const size_t smem = kGramBufs * (size_t)kGramChunkPx * (10 + 1) * sizeof(float2);
    cudaError_t e = cudaFuncSetAttribute(gram_pixel_kernel<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(gram_pixel_kernel)");
    gram_pixel_kernel<10><<<B, kGramSubsets * kGramLanes, smem, st>>>(
        static_cast<const float2 *>(q), is, static_cast<const float2 *>(images), P, static_cast<float2 *>(gram),
        static_cast<float2 *>(h), yy);
    return launched("gram_pixel_kernel");
  }
  const int J = r * (r + 1) / 2 + r + 1;
  const int threads = J > 256 ? ((J + 31) / 32) * 32 : 256;
  const size_t smem = (size_t)kGramChunk * (r + 1) * sizeof(float2);
  gram_kernel<<<B, threads, smem, st>>>(static_cast<const float2 *>(q), is, ps, cs, static_cast<const float2 *>(images),
                                        P, r, static_cast<float2 *>(gram), static_cast<float2 *>(h), yy);
  return launched("gram_kernel");
}

int launch_wpass(cudaStream_t st, int B, int P, int r, const void *q, int64_t is, int64_t ps, int64_t cs,
                 const void *images, const void *C, const void *u, void *w, int64_t wis, int64_t wps, int64_t wcs) {
  if (q == w && is == wis && ps == wps && cs == 1 && wcs == 1 && ps == r && (r == 10 || r == 20) &&
      (reinterpret_cast<uintptr_t>(w) & 15) == 0 && (is & 1) == 0) {
    dim3 g((P + 255) / 256, B);
    float2 *qw = static_cast<float2 *>(w);
    const float2 *y = static_cast<const float2 *>(images);
    const float2 *cc = static_cast<const float2 *>(C), *uu = static_cast<const float2 *>(u);
    if (r == 10) {
      wpass_pixel_kernel<10><<<g, 256, 0, st>>>(qw, is, ps, y, cc, uu, P);
    } else {
      wpass_pixel_kernel<20><<<g, 256, 0, st>>>(qw, is, ps, y, cc, uu, P);
    }
    return launched("wpass_pixel_kernel");
  }
  const size_t smem = (size_t)(r * r + r + kGramChunk * (r + 1)) * sizeof(float2);
  dim3 grid((P + kGramChunk - 1) / kGramChunk, B);
  wpass_kernel<<<grid, 256, smem, st>>>(static_cast<const float2 *>(q), is, ps, cs,
                                        static_cast<const float2 *>(images), static_cast<const float2 *>(C),
                                        static_cast<const float2 *>(u), P, r, static_cast<float2 *>(w), wis, wps,
                                        wcs);
  return launched("wpass_kernel");
}

int launch_solve(cudaStream_t st, int B, int r, int objective, const void *gram, const void *h, double s2,
                 const double *linv, double wscale, double cscale, void *C, void *u, double *cost_b, double *cost_sum,
                 void *z, void *m, int *bad) {
  if (r < 1 || r > kMaxRank) {
    set_error("rank %d out of range (1..%d)", r, kMaxRank);
    return COV3D_EINVAL;
  }
  SolveArgs sa{};
  sa.B = B;
  sa.r = r;
  sa.objective = objective;
  sa.gram = static_cast<const float2 *>(gram);
  sa.h = static_cast<const float2 *>(h);
  sa.s2 = s2;
  sa.linv = linv;
  sa.wscale = wscale;
  sa.cscale = cscale;
  sa.C = static_cast<float2 *>(C);
  sa.u = static_cast<float2 *>(u);
  sa.cost_b = cost_b;
  sa.cost_sum = cost_sum;
  sa.z_out = static_cast<float2 *>(z);
  sa.m_out = static_cast<float2 *>(m);
  sa.bad = bad;
  static_assert(kMaxRank <= kSolveThreads, "one thread per column of every image");
  const int ipb = kSolveThreads / r;
  const unsigned blocks = (unsigned)((B + ipb - 1) / ipb);
  if (r <= 10) {
    solve_kernel<10><<<blocks, kSolveThreads, 0, st>>>(sa);
  } else if (r <= 16) {
    solve_kernel<16><<<blocks, kSolveThreads, 0, st>>>(sa);
  } else if (r <= 20) {
    solve_kernel<20><<<blocks, kSolveThreads, 0, st>>>(sa);
  } else {
    solve_kernel<kMaxRank><<<blocks, kSolveThreads, 0, st>>>(sa);
  }
  return launched("solve_kernel");
}

int covar_cost_grad(cov3d_plan *p, const cov3d_cost_args *a, double *h_cost, double *d_cost, float *d_grad_vectors,
                    float *d_grad_log_sqrt, double *d_per_image_cost) {
  const int r = a->rank;
  if (r < 1 || r > kMaxRank || r > p->n_trans) {
    set_error("rank %d out of range (1..min(32, n_trans=%d))", r, p->n_trans);
    return COV3D_EINVAL;
  }
  if (!a->d_vectors || !a->d_log_sqrt || !a->d_images || !d_grad_vectors || !d_grad_log_sqrt) {
    set_error("null pointer argument");
    return COV3D_EINVAL;
  }
  if (p->point_kind == kPointsNone || p->points_L != p->L) {
    set_error("points for L=%d images must be set before the cost", p->L);
    return COV3D_ESTATE;
  }
  if (!(a->noise_var > 0.0)) {
    set_error("noise_var must be positive");
    return COV3D_EINVAL;
  }
  const int B = (int)p->n_images;
  const int L = p->L;
  const int P = L * L;
  const int64_t n3 = (int64_t)p->n * p->n * p->n;
  const int64_t M = p->n_points;

  COV3D_TRY(grow(p->fine, n3 * r * 8));
  COV3D_TRY(grow(p->fine2, n3 * r * 8));
  COV3D_TRY(grow(p->q, M * r * 8));
  const int64_t small_bytes = (int64_t)B * (r * r * 8 * 2 + r * 8 * 2 + 8 + 8) + 64;
  COV3D_TRY(grow(p->small, small_bytes));
  float2 *gram = p->small.as<float2>();
  float2 *h = gram + (int64_t)B * r * r;
  float2 *C = h + (int64_t)B * r;
  float2 *u = C + (int64_t)B * r * r;
  float *yy = reinterpret_cast<float *>(u + (int64_t)B * r);
  int *bad = reinterpret_cast<int *>(yy + B);
  double *acc = p->acc.as<double>();

  COV3D_CUDA(cudaMemsetAsync(acc, 0, 64 * sizeof(double), p->stream));
  COV3D_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), p->stream));

  // 1. pack the deapodised, scaled eigenvolumes into the fine grid; 2. forward FFT.  Even L:
  // pruned transforms, staged in fine2 (zeroed before the spread anyway): 2D FFTs over each
  // channel's L support planes, then the axis-0 FFT out of place into fine.
  const bool pruned = prunable(p);
  // fine grids of n = 128 .. 512: hand-written line transforms with the pack, the regulariser
  // (value, and the gradient grid's initial coef * fr * G or zero) and the unpack fused in.  The
  // forward one up to n = 256: at 512 its 32 x 16 split idles half the threads in one stage and
  // measured slower than pack + cuFFT + regulariser (19.0 against 15.4 ms at L = 256, r = 10);
  // the inverse is faster at every size (8.8 against 11.1 ms there).
  const bool lines_inv = pruned && line_transforms_apply(p);
  const bool lines_fwd = lines_inv && p->n <= 256;
  const bool with_reg = a->d_fourier_reg && a->reg_scale != 0.0;
  const bool ml_reg = with_reg && a->objective == 0;  // sum fr |G|^2: fused into the transforms
  const bool ls_reg = with_reg && a->objective != 0;  // |X X^H|^2: GEMMs before the spread (ls_reg.cu)
  const int64_t fr_stride = a->fourier_reg_per_channel ? n3 : 0;
  const float *gcp = a->use_grid_correction ? p->gc1d.as<float>() : nullptr;
  cufftHandle fft = 0, fplanes = 0, faxis0 = 0;
  if (pruned) {
    COV3D_TRY(grow(p->fine2, n3 * r * 8));
    if (!lines_fwd) {  // the forward transform on cuFFT
      COV3D_TRY(get_fft_planes(p, &fplanes));
      COV3D_TRY(get_fft_axis0(p, &faxis0));
    }
  } else {
    COV3D_TRY(get_fft(p, r, &fft));
  }
  const int64_t half_off = (int64_t)(p->n - L / 2) * p->n * p->n;
  if (lines_fwd) {
    PhaseScope ps(p, kPhaseFftFwd);
    COV3D_TRY(step_forward_lines(p, a->d_vectors, a->d_log_sqrt, gcp, r, p->fine2.as<float2>(), p->fine.as<float2>(),
                                 ml_reg ? a->d_fourier_reg : nullptr, fr_stride, a->reg_scale / (2.0 * a->noise_var),
                                 acc + 1));
  } else {
    PhaseScope ps(p, kPhasePack);
    COV3D_TRY(launch_pack(p, a->d_vectors, nullptr, a->d_log_sqrt, a->use_grid_correction, r,
                          pruned ? p->fine2.ptr : p->fine.ptr));
  }
  if (!lines_fwd) {
    PhaseScope ps(p, kPhaseFftFwd);
    if (pruned) {
      for (int c = 0; c < r; ++c) {
        float2 *src = p->fine2.as<float2>() + c * n3;
        COV3D_TRY(fft2(fplanes, src, src, CUFFT_FORWARD));
        COV3D_TRY(fft2(fplanes, src + half_off, src + half_off, CUFFT_FORWARD));
        COV3D_TRY(fft2(faxis0, src, p->fine.as<float2>() + c * n3, CUFFT_FORWARD));
      }
    } else {
      COV3D_TRY(check_cufft(cufftExecC2C(fft, p->fine.as<cufftComplex>(), p->fine.as<cufftComplex>(), CUFFT_FORWARD),
                            "cufftExecC2C(forward)"));
    }
  }
  // 3. interpolate at the central slices with the fused projection epilogue -> Q (B*P, r)
  const int shift = p->n - p->n / 2;
  GridArgs ga{p->fine.ptr, 1, n3, shift};
  EpilogueArgs ep{a->ctf_params ? nullptr : a->d_ctf, 1, 1.0f / (float)L};
  if (a->ctf_params && a->d_ctf) COV3D_TRY(prepare_ctf_coef(p, a->d_ctf, B, L, &ep.ctfc));
  {
    PhaseScope ps(p, kPhaseInterp);
    COV3D_TRY(launch_interp(p, ga, r, p->q.ptr, r, 1, ep));
  }
  // 4. per-image Gram, 5. FP64 solve -> cost, C, u
  {
    PhaseScope ps(p, kPhaseGram);
    if (a->gram_bf16) {
      COV3D_TRY(launch_gram_bf16(p, p->stream, B, P, r, p->q.ptr, (int64_t)P * r, r, 1, a->d_images, gram, h, yy));
    } else {
      COV3D_TRY(launch_gram(p->stream, B, P, r, p->q.ptr, (int64_t)P * r, r, 1, a->d_images, gram, h, yy));
    }
  }
  const double L4 = (double)L * L * L * L;
  {
    PhaseScope ps(p, kPhaseSolve);
    COV3D_TRY(launch_solve(p->stream, B, r, a->objective, gram, h, a->noise_var, nullptr,
                           a->objective == 0 ? 1.0 / B : 1.0 / (B * L4), a->objective == 0 ? 1.0 : 1.0 / L4, C, u,
                           d_per_image_cost, acc, nullptr, nullptr, bad));
  }
  // 6. dcost/dconj(Q) in place, 7. spread through the exact adjoint (CTF, Nyquist, 1/L prologue)
  {
    PhaseScope ps(p, kPhaseWpass);
    COV3D_TRY(launch_wpass(p->stream, B, P, r, p->q.ptr, (int64_t)P * r, r, 1, a->d_images, C, u, p->q.ptr,
                           (int64_t)P * r, r, 1));
  }
  // 7'. the regulariser (value and gradient coef * fr * G) initialises the gradient grid, so the
  // spread adds onto it and no zeroing pass is needed; without one, the grid is zeroed
  if (ml_reg && !lines_fwd) {
    PhaseScope ps(p, kPhaseReg);
    COV3D_TRY(launch_ml_reg(p, p->fine.ptr, p->fine2.ptr, a->d_fourier_reg, fr_stride, r,
                            a->reg_scale / (2.0 * a->noise_var), acc + 1, 1));
  }
  if (ls_reg) {  // value and derivative, onto the gradient grid (zero after the line transforms)
    PhaseScope ps(p, kPhaseReg);
    if (!lines_fwd) COV3D_TRY(launch_zero(p, p->fine2.ptr, n3 * r * 8));
    COV3D_TRY(launch_ls_reg(p, p->fine.ptr, p->fine2.ptr, a->d_fourier_reg, fr_stride, r, a->reg_scale / L4,
                            acc + 1));
  }
  {
    PhaseScope ps(p, kPhaseSpread);
    if (!with_reg && !lines_fwd) COV3D_TRY(launch_zero(p, p->fine2.ptr, n3 * r * 8));
    COV3D_TRY(launch_spread(p, p->q.ptr, r, 1, r, ep, p->fine2.ptr, 1, n3, shift));
  }
  // 9. adjoint FFT, 10. crop + deapodise + chain rule to the Covar parameters
  if (lines_inv) {
    PhaseScope ps(p, kPhaseFftInv);
    COV3D_TRY(step_inverse_lines(p, p->fine2.as<float2>(), a->d_vectors, a->d_log_sqrt, gcp, r, d_grad_vectors,
                                 acc + 8));
  } else {
    PhaseScope ps(p, kPhaseFftInv);
    if (pruned) {  // axis 0 over all lines, then 2D only on the support planes the crop reads
      for (int c = 0; c < r; ++c) {
        float2 *g = p->fine2.as<float2>() + c * n3;
        COV3D_TRY(fft2(faxis0, g, g, CUFFT_INVERSE));
        COV3D_TRY(fft2(fplanes, g, g, CUFFT_INVERSE));
        COV3D_TRY(fft2(fplanes, g + half_off, g + half_off, CUFFT_INVERSE));
      }
    } else {
      COV3D_TRY(check_cufft(cufftExecC2C(fft, p->fine2.as<cufftComplex>(), p->fine2.as<cufftComplex>(), CUFFT_INVERSE),
                            "cufftExecC2C(inverse)"));
    }
  }
  if (!lines_inv) {
    PhaseScope ps(p, kPhaseUnpack);
    COV3D_TRY(launch_unpack_grad(p, p->fine2.ptr, a->d_vectors, a->d_log_sqrt, a->use_grid_correction, r,
                                 d_grad_vectors, acc + 8));
  }
  finalize_kernel<<<1, 64, 0, p->stream>>>(acc, r, 1.0 / B, d_cost, d_grad_log_sqrt);
  COV3D_LAUNCHED("finalize_kernel");
  if (h_cost) {
    COV3D_CUDA(cudaMemcpyAsync(p->h_acc, acc, 8 * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    int h_bad = 0;
    COV3D_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    COV3D_CUDA(cudaStreamSynchronize(p->stream));
    if (h_bad) {
      set_error("a per-image matrix m was not positive definite");
      return COV3D_ENONFINITE;
    }
    *h_cost = p->h_acc[0] / B + p->h_acc[1];
  }
  return COV3D_OK;
}

}  // namespace cov3d
