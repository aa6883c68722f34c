/*
 * oracle/fft64.c -- CPU FP64 oracle for the batched complex-to-complex FFT.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the tcfft_gb300 product links, loads
 * or calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, as the checker.
 *
 * What it restates (reference = rox906/tcFFT):
 *   - oracle_fft_1d: the reference's accuracy oracle, FFTW's forward DFT in
 *     FP64, unnormalised, sign -1, one plan per batch item
 *     (accuracy.cpp:11-23, fftw_plan_dft_1d(..., FFTW_FORWARD, ...)).
 *     FFTW 3.3.8 (README.md:2) is not vendored and not installed here, so the
 *     published algorithm (the DFT X[k] = sum_n x[n] exp(-2 pi i n k / N)) is
 *     computed by an own iterative radix-2 FFT with an exactly reduced
 *     twiddle table.  sign=+1 gives the conjugate-direction (adjoint) DFT.
 *   - oracle_fft_2d: accuracy_2d.cpp:11-23 (fftw_plan_dft_2d(nx, ny),
 *     row-major [nx][ny], forward, unnormalised).
 *   - oracle_gen_rev: the mixed-radix digit-reversal permutation the reference
 *     applies to the input on the host (tcfft_doit_half.cpp:6-29).
 *   - oracle_clipped_error: the reference's error metric, the mean over all
 *     real and imaginary components of min(1, |(t - s) / s|)
 *     (accuracy.cpp:25-41).
 *   - oracle_dft_naive: an O(N^2) long-double DFT used to cross-check the FFT.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PI 3.14159265358979323846264338327950288

/* cos/sin of -sign*2*pi*j/n for j in [0, n), computed from the first octant
 * with exact symmetry so that table entries are accurate to ~1 ulp. */
static void twiddle_table(int64_t n, int sign, double *wr, double *wi) {
  for (int64_t j = 0; j < n; ++j) {
    /* reduce j/n to an angle in [0, 1/8] turn using symmetries */
    int64_t a = j;             /* angle = 2*pi*a/n */
    int64_t q8 = a * 8 / n;    /* octant */
    double c, s;
    int64_t r;
    /* use exact integer arithmetic for the reduction: theta = 2 pi a / n */
    switch (q8) {
      case 0: r = a; c = cos(2.0 * ORACLE_PI * r / n); s = sin(2.0 * ORACLE_PI * r / n); break;
      case 1: r = n / 4 - a; c = sin(2.0 * ORACLE_PI * r / n); s = cos(2.0 * ORACLE_PI * r / n); break;
      case 2: r = a - n / 4; c = -sin(2.0 * ORACLE_PI * r / n); s = cos(2.0 * ORACLE_PI * r / n); break;
      case 3: r = n / 2 - a; c = -cos(2.0 * ORACLE_PI * r / n); s = sin(2.0 * ORACLE_PI * r / n); break;
      case 4: r = a - n / 2; c = -cos(2.0 * ORACLE_PI * r / n); s = -sin(2.0 * ORACLE_PI * r / n); break;
      case 5: r = 3 * n / 4 - a; c = -sin(2.0 * ORACLE_PI * r / n); s = -cos(2.0 * ORACLE_PI * r / n); break;
      case 6: r = a - 3 * n / 4; c = sin(2.0 * ORACLE_PI * r / n); s = -cos(2.0 * ORACLE_PI * r / n); break;
      default: r = n - a; c = cos(2.0 * ORACLE_PI * r / n); s = -sin(2.0 * ORACLE_PI * r / n); break;
    }
    /* (c, s) = (cos theta, sin theta); the DFT kernel is exp(sign * i * theta) */
    wr[j] = c;
    wi[j] = sign < 0 ? -s : s;
  }
}

/* In-place iterative radix-2 DIT FFT of one length-n (power of two) vector of
 * interleaved complex doubles, using a precomputed length-n table. */
static void fft_one(double *x, int64_t n, const double *wr, const double *wi) {
  /* bit reversal */
  for (int64_t i = 1, j = 0; i < n; ++i) {
    int64_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double tr = x[2 * i], ti = x[2 * i + 1];
      x[2 * i] = x[2 * j]; x[2 * i + 1] = x[2 * j + 1];
      x[2 * j] = tr; x[2 * j + 1] = ti;
    }
  }
  for (int64_t len = 2; len <= n; len <<= 1) {
    int64_t half = len >> 1, step = n / len;
    for (int64_t base = 0; base < n; base += len) {
      for (int64_t k = 0; k < half; ++k) {
        double cr = wr[k * step], ci = wi[k * step];
        double *u = x + 2 * (base + k), *v = x + 2 * (base + k + half);
        double vr = v[0] * cr - v[1] * ci;
        double vi = v[0] * ci + v[1] * cr;
        v[0] = u[0] - vr; v[1] = u[1] - vi;
        u[0] += vr; u[1] += vi;
      }
    }
  }
}

static int is_pow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

/* Number of OpenMP threads the oracle uses (1 without OpenMP). */
int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

/* Batched 1D DFT, in place on [batch][n] interleaved complex doubles.
 * sign = -1: forward (the reference's FFTW_FORWARD); sign = +1: conjugate
 * direction.  Returns 0 on success, -1 on bad arguments. */
int oracle_fft_1d(double *data, int64_t n, int64_t batch, int sign) {
  if (!is_pow2(n) || batch < 0 || (sign != -1 && sign != 1)) return -1;
  double *wr = (double *)malloc(sizeof(double) * n);
  double *wi = (double *)malloc(sizeof(double) * n);
  if (!wr || !wi) { free(wr); free(wi); return -1; }
  twiddle_table(n, sign, wr, wi);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t b = 0; b < batch; ++b) fft_one(data + 2 * n * b, n, wr, wi);
  free(wr); free(wi);
  return 0;
}

/* Batched 2D DFT, in place on [batch][nx][ny] interleaved complex doubles
 * (row-major, as fftw_plan_dft_2d(nx, ny) in accuracy_2d.cpp:11-23). */
int oracle_fft_2d(double *data, int64_t nx, int64_t ny, int64_t batch, int sign) {
  if (!is_pow2(nx) || !is_pow2(ny) || batch < 0 || (sign != -1 && sign != 1)) return -1;
  if (oracle_fft_1d(data, ny, batch * nx, sign) != 0) return -1;
  double *wr = (double *)malloc(sizeof(double) * nx);
  double *wi = (double *)malloc(sizeof(double) * nx);
  if (!wr || !wi) { free(wr); free(wi); return -1; }
  twiddle_table(nx, sign, wr, wi);
#pragma omp parallel
  {
    double *col = (double *)malloc(sizeof(double) * 2 * nx);
#pragma omp for schedule(dynamic, 16)
    for (int64_t bc = 0; bc < batch * ny; ++bc) {
      int64_t b = bc / ny, c = bc % ny;
      double *base = data + 2 * (b * nx * ny + c);
      for (int64_t r = 0; r < nx; ++r) {
        col[2 * r] = base[2 * r * ny];
        col[2 * r + 1] = base[2 * r * ny + 1];
      }
      fft_one(col, nx, wr, wi);
      for (int64_t r = 0; r < nx; ++r) {
        base[2 * r * ny] = col[2 * r];
        base[2 * r * ny + 1] = col[2 * r + 1];
      }
    }
    free(col);
  }
  free(wr); free(wi);
  return 0;
}

/* O(n^2) long-double DFT of one vector (out of place), for cross-checks. */
int oracle_dft_naive(const double *in, double *out, int64_t n, int sign) {
  if (n <= 0 || (sign != -1 && sign != 1)) return -1;
  for (int64_t k = 0; k < n; ++k) {
    long double sr = 0.0L, si = 0.0L;
    for (int64_t j = 0; j < n; ++j) {
      int64_t m = (j * k) % n;
      long double th = 2.0L * (long double)ORACLE_PI * (long double)m / (long double)n;
      long double c = cosl(th), s = sinl(th) * (long double)sign;
      sr += (long double)in[2 * j] * c - (long double)in[2 * j + 1] * s;
      si += (long double)in[2 * j] * s + (long double)in[2 * j + 1] * c;
    }
    out[2 * k] = (double)sr;
    out[2 * k + 1] = (double)si;
  }
  return 0;
}

/* Mixed-radix digit-reversal permutation, restating the reference's host-side
 * input reordering gen_rev (tcfft_doit_half.cpp:6-29): starting from the
 * identity, for each radix from the last to the first, every block of the
 * current length is split into `radix` interleaved sub-sequences that are
 * laid out one after the other; the block length then shrinks by that radix.
 * The caller feeds data[rev[i]] at position i.  Returns 0, or -1 when the
 * radices do not multiply to n. */
int oracle_gen_rev(int64_t n, const int *radices, int n_radices, int64_t *rev) {
  int64_t prod = 1;
  for (int i = 0; i < n_radices; ++i) {
    if (radices[i] <= 0) return -1;
    prod *= radices[i];
  }
  if (prod != n) return -1;
  int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * n);
  int64_t *nxt = (int64_t *)malloc(sizeof(int64_t) * n);
  if (!cur || !nxt) { free(cur); free(nxt); return -1; }
  for (int64_t i = 0; i < n; ++i) cur[i] = i;
  int64_t len = n;
  for (int d = n_radices - 1; d >= 0; --d) {
    int64_t r = radices[d], sub = len / r;
    for (int64_t blk = 0; blk < n; blk += len)
      for (int64_t k = 0; k < r; ++k)
        for (int64_t l = 0; l < sub; ++l) nxt[blk + k * sub + l] = cur[blk + l * r + k];
    len = sub;
    int64_t *t = cur; cur = nxt; nxt = t;
  }
  memcpy(rev, cur, sizeof(int64_t) * n);
  free(cur); free(nxt);
  return 0;
}

/* The reference's accuracy metric (accuracy.cpp:25-41): mean over all 2*count
 * real components of min(1, |(tested - standard) / standard|).  A zero
 * standard component gives an infinite or NaN ratio; min(1, inf) is 1 and
 * std::min(1.0, NaN) returns 1.0 as well, which is reproduced here. */
double oracle_clipped_error(const double *tested, const double *standard, int64_t count) {
  double err = 0.0;
#pragma omp parallel for reduction(+ : err)
  for (int64_t i = 0; i < 2 * count; ++i) {
    double r = fabs((tested[i] - standard[i]) / standard[i]);
    err += (r < 1.0) ? r : 1.0; /* NaN compares false -> 1.0, like std::min(1.0, NaN) */
  }
  return err / (double)count;
}
