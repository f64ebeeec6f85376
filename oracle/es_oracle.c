/*
 * CPU oracle (test infrastructure only): exponential-of-semicircle interpolation and
 * spreading on a centered, channels-last complex fine grid, in plain C with OpenMP.
 *
 * Restates the published ES-kernel NUFFT spreading step (Barnett, Magland & af Klinteberg,
 * SIAM J. Sci. Comput. 2019) that the reference reaches through cuFINUFFT / FINUFFT
 * (reference nufft_plan.py:288-316, :359, :387), with the same conventions as
 * oracle/nufft_oracle.py (es_interp / es_spread): a point at fractional index t touches cells
 * c0 .. c0+w-1 with c0 = ceil(t - w/2), weight exp(beta*(sqrt(1-(2x/w)^2)-1)), x = t - cell,
 * cells wrapped periodically mod n.
 *
 * Compiled twice: -DREAL=double (the oracle) and -DREAL=float (the timed CPU baseline).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL double
#endif

#define MAXW 16

static int es_taps(REAL t, int w, REAL beta, REAL *wt) {
  const int c0 = (int)ceil((double)t - 0.5 * w);
  for (int j = 0; j < w; ++j) {
    const REAL x = (t - (REAL)(c0 + j)) * ((REAL)2 / (REAL)w);
    const REAL u = (REAL)1 - x * x;
    wt[j] = u > 0 ? (REAL)exp((double)(beta * ((REAL)sqrt((double)u) - (REAL)1))) : (REAL)0;
  }
  return c0;
}

static inline int pmod(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}

/* out[m*nchan + c] (complex) = sum over the window of grid[cell*nchan + c] * weight */
void oracle_es_interp(int n, int w, double beta, int nchan, const REAL *grid, int64_t M, const REAL *t, REAL *out,
                      int nthreads) {
  if (w > MAXW) return;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t m = 0; m < M; ++m) {
    REAL wt[3][MAXW];
    int c0[3];
    for (int d = 0; d < 3; ++d) c0[d] = es_taps(t[3 * m + d], w, (REAL)beta, wt[d]);
    REAL *o = out + 2 * m * nchan;
    for (int c = 0; c < 2 * nchan; ++c) o[c] = 0;
    for (int a = 0; a < w; ++a) {
      const int i0 = pmod(c0[0] + a, n);
      for (int b = 0; b < w; ++b) {
        const int i1 = pmod(c0[1] + b, n);
        const REAL wab = wt[0][a] * wt[1][b];
        const int64_t row = ((int64_t)i0 * n + i1) * n;
        for (int e = 0; e < w; ++e) {
          const REAL ww = wab * wt[2][e];
          const REAL *g = grid + 2 * (row + pmod(c0[2] + e, n)) * nchan;
          for (int c = 0; c < nchan; ++c) {
            o[2 * c] += ww * g[2 * c];
            o[2 * c + 1] += ww * g[2 * c + 1];
          }
        }
      }
    }
  }
}

/* grid[cell*nchan + c] += sum over points of vals[m*nchan + c] * weight; the axis-0 slabs of
 * the grid are split between threads, every thread visiting all points (deterministic). */
void oracle_es_spread(int n, int w, double beta, int nchan, REAL *grid, int64_t M, const REAL *t, const REAL *vals,
                      int nthreads) {
  if (w > MAXW) return;
  int *first = (int *)malloc(sizeof(int) * (size_t)M);
  if (!first) return;
  for (int64_t m = 0; m < M; ++m) first[m] = (int)ceil((double)t[3 * m] - 0.5 * w);
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0, nt = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    nt = omp_get_num_threads();
#endif
    const int lo = (int)((int64_t)n * tid / nt), hi = (int)((int64_t)n * (tid + 1) / nt);
    for (int64_t m = 0; m < M; ++m) {
      int hit = 0;
      for (int a = 0; a < w; ++a) {
        const int i0 = pmod(first[m] + a, n);
        if (i0 >= lo && i0 < hi) hit = 1;
      }
      if (!hit) continue;
      REAL wt[3][MAXW];
      int c0[3];
      for (int d = 0; d < 3; ++d) c0[d] = es_taps(t[3 * m + d], w, (REAL)beta, wt[d]);
      const REAL *v = vals + 2 * m * nchan;
      for (int a = 0; a < w; ++a) {
        const int i0 = pmod(c0[0] + a, n);
        if (i0 < lo || i0 >= hi) continue;
        for (int b = 0; b < w; ++b) {
          const int i1 = pmod(c0[1] + b, n);
          const REAL wab = wt[0][a] * wt[1][b];
          const int64_t row = ((int64_t)i0 * n + i1) * n;
          for (int e = 0; e < w; ++e) {
            const REAL ww = wab * wt[2][e];
            REAL *g = grid + 2 * (row + pmod(c0[2] + e, n)) * nchan;
            for (int c = 0; c < nchan; ++c) {
              g[2 * c] += ww * v[2 * c];
              g[2 * c + 1] += ww * v[2 * c + 1];
            }
          }
        }
      }
    }
  }
  free(first);
}

int oracle_real_size(void) { return (int)sizeof(REAL); }
