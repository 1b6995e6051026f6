/*
 * sfft_oracle.c -- CPU restatement of the pcdslab/gpu-sfft pipeline (FP64).
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the CPU baseline.  Nothing
 * in the product links or calls this file.  Build (see oracle/Makefile):
 *   gcc -O2 -std=gnu11 -fopenmp -ffp-contract=off -fPIC -shared
 *
 * -ffp-contract=off is part of the specification: every floating-point
 * operation below rounds exactly as written, and the only fused operations are
 * the explicit fma() calls.  The GPU engine states the same operation
 * sequences, so stages fed identical inputs agree bit for bit.
 *
 * Citations are file:line inside the reference project.
 */
#define _GNU_SOURCE
#include "sfft_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int oc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Number theory and parameters                                              */
/* ------------------------------------------------------------------------ */

/* utils.c:180-185: largest power of two <= x (0 when x < 1). */
int oc_floor_to_pow2(double x) {
  unsigned int ans;
  for (ans = 1; ans <= x; ans <<= 1) {
  }
  return (int)(ans / 2);
}

/* utils.c:81-84 (Euclid; gcd(0, n) == n). */
int oc_gcd(int a, int b) {
  while (a % b != 0) {
    int r = a % b;
    a = b;
    b = r;
  }
  return b;
}

/* utils.c:92-105: modular inverse by the extended Euclidean algorithm. */
int oc_mod_inverse(int a, int n) {
  long long r0 = n, r1 = a, t0 = 0, t1 = 1;
  while (r1 > 0) {
    long long qt = r0 / r1, tmp;
    tmp = r0 - qt * r1; r0 = r1; r1 = tmp;
    tmp = t0 - qt * t1; t0 = t1; t1 = tmp;
  }
  t0 %= n;
  if (t0 < 0) t0 += n;
  return (int)t0;
}

/* experiment.c:54-84 and cuExperiment.cu:279-284.  The floating-point
 * expressions keep the reference's evaluation order so the integer results
 * (B, b_f, W_RLFC, w) are identical. */
int oc_derive_params(int q, int k, double Bcst, int loops_loc, int loops_thresh,
                     int loops_est, double RLFC_cst, int RLFC_loops,
                     double tolerance, oc_params *p) {
  memset(p, 0, sizeof(*p));
  if (q < 1 || q > 30 || k < 1) return OC_ERR_PARAM;
  int n = (int)pow(2, q);
  n = oc_floor_to_pow2(n);
  p->q = q; p->n = n; p->k = k; p->Bcst = Bcst; p->RLFC_cst = RLFC_cst;
  p->loops_loc = loops_loc; p->loops_thresh = loops_thresh;
  p->loops_est = loops_est; p->loops = loops_loc + loops_est;
  p->RLFC_loops = RLFC_loops; p->tolerance = tolerance;
  p->BB = (unsigned)(Bcst * sqrt((double)n * k / (log2(n))));
  p->lobefrac = 0.5 / (p->BB);
  p->b_f = (int)(1.2 * 1.1 * ((double)n / p->BB));
  p->B = oc_floor_to_pow2(p->BB);
  p->B_thresh = 2 * k;
  p->W_RLFC = oc_floor_to_pow2(RLFC_cst * n / p->B);
  int w = (int)((1 / M_PI) * (1 / p->lobefrac) * acosh(1. / tolerance));
  if (!(w % 2)) w--;
  p->w = w;
  p->t0 = cosh(acosh(1 / tolerance) / (w - 1));
  /* experiment.c:77,82-84, cuExperiment.cu:283 */
  if (!(p->b_f <= n)) return OC_ERR_PARAM;
  if (!(p->B_thresh < p->W_RLFC)) return OC_ERR_PARAM;
  if (!(p->B_thresh < p->B)) return OC_ERR_PARAM;
  if (!(loops_thresh <= loops_loc)) return OC_ERR_PARAM;
  if (!(w <= n)) return OC_ERR_PARAM;
  if (p->B < 1 || p->W_RLFC < 1 || RLFC_loops < 1 || loops_loc < 1) return OC_ERR_PARAM;
  return OC_OK;
}

/* innerLoop.cu:122-123 and outerLoop.cu:128-134. */
void oc_draw_glibc(long seed, int n, int W_RLFC, int RLFC_loops, int loops,
                   int *rlfc_offsets, int *a_out, int *ai_out) {
  if (seed >= 0) {
    srand48(seed);
    srandom((unsigned)seed);
  }
  int sigma = n / W_RLFC;
  for (int r = 0; r < RLFC_loops; r++)
    rlfc_offsets[r] = (int)(unsigned)floor(drand48() * sigma);
  for (int i = 0; i < loops; i++) {
    int a = 0;
    while (oc_gcd(a, n) != 1) a = (int)(random() % n);
    a_out[i] = a;
    ai_out[i] = oc_mod_inverse(a, n);
  }
}

/* ------------------------------------------------------------------------ */
/* FFT: radix-2 DIT (powers of two) and Bluestein (any size)                 */
/* ------------------------------------------------------------------------ */

static inline oc_complex cmul(oc_complex a, oc_complex b) {
  oc_complex c;
  c.x = a.x * b.x - a.y * b.y;
  c.y = a.x * b.y + a.y * b.x;
  return c;
}

static unsigned rev_bits(unsigned v, int bits) {
  unsigned r = 0;
  for (int i = 0; i < bits; i++) { r = (r << 1) | (v & 1u); v >>= 1; }
  return r;
}

/* Unnormalised DFT, X[k] = sum_j x[j] exp(sign*2*pi*i*j*k/N), N a power of 2.
 * Twiddles are evaluated from the exact angle, never by recurrence. */
static int fft_pow2(oc_complex *a, long N, int sign) {
  if (N <= 1) return OC_OK;
  int bits = 0;
  while ((1L << bits) < N) bits++;
  oc_complex *tw = (oc_complex *)malloc(sizeof(oc_complex) * (size_t)(N / 2));
  if (!tw) return OC_ERR_ALLOC;
#pragma omp parallel for schedule(static) if (N >= 65536)
  for (long j = 0; j < N / 2; j++) {
    double ang = 2.0 * M_PI * (double)j / (double)N;
    tw[j].x = cos(ang);
    tw[j].y = sign * sin(ang);
  }
#pragma omp parallel for schedule(static) if (N >= 65536)
  for (long i = 0; i < N; i++) {
    long r = (long)rev_bits((unsigned)i, bits);
    if (i < r) { oc_complex t = a[i]; a[i] = a[r]; a[r] = t; }
  }
  const long BLK = N < 16384 ? N : 16384;
  /* spans inside cache-sized blocks first */
#pragma omp parallel for schedule(static) if (N >= 65536)
  for (long b0 = 0; b0 < N; b0 += BLK) {
    for (long s = 1; s < BLK; s <<= 1) {
      long stride = N / (2 * s);
      for (long g = b0; g < b0 + BLK; g += 2 * s) {
        for (long j = 0; j < s; j++) {
          oc_complex t = cmul(tw[j * stride], a[g + j + s]);
          oc_complex u = a[g + j];
          a[g + j].x = u.x + t.x; a[g + j].y = u.y + t.y;
          a[g + j + s].x = u.x - t.x; a[g + j + s].y = u.y - t.y;
        }
      }
    }
  }
  for (long s = BLK; s < N; s <<= 1) {
    long stride = N / (2 * s);
#pragma omp parallel for schedule(static) if (N >= 65536)
    for (long t = 0; t < N / 2; t++) {
      long j = t % s, g = (t / s) * 2 * s;
      oc_complex tt = cmul(tw[j * stride], a[g + j + s]);
      oc_complex u = a[g + j];
      a[g + j].x = u.x + tt.x; a[g + j].y = u.y + tt.y;
      a[g + j + s].x = u.x - tt.x; a[g + j + s].y = u.y - tt.y;
    }
  }
  free(tw);
  return OC_OK;
}

/* Bluestein chirp-z: X[k] = c[k] * sum_j (x[j] c[j]) conj(c[k-j]),
 * c[m] = exp(sign*pi*i*m^2/N), with m^2 reduced mod 2N in integers. */
static int fft_bluestein(oc_complex *x, long N, int sign) {
  long M = 1;
  while (M < 2 * N - 1) M <<= 1;
  oc_complex *a = (oc_complex *)calloc((size_t)M, sizeof(oc_complex));
  oc_complex *b = (oc_complex *)calloc((size_t)M, sizeof(oc_complex));
  oc_complex *c = (oc_complex *)malloc(sizeof(oc_complex) * (size_t)N);
  if (!a || !b || !c) { free(a); free(b); free(c); return OC_ERR_ALLOC; }
#pragma omp parallel for schedule(static) if (N >= 65536)
  for (long m = 0; m < N; m++) {
    unsigned long long mm = ((unsigned long long)m * (unsigned long long)m) %
                            (unsigned long long)(2 * N);
    double ang = M_PI * (double)mm / (double)N;
    c[m].x = cos(ang);
    c[m].y = sign * sin(ang);
  }
#pragma omp parallel for schedule(static) if (N >= 65536)
  for (long m = 0; m < N; m++) {
    a[m] = cmul(x[m], c[m]);
    oc_complex cc = {c[m].x, -c[m].y};
    b[m] = cc;
    if (m > 0) b[M - m] = cc;
  }
  int st = fft_pow2(a, M, -1);
  if (st == OC_OK) st = fft_pow2(b, M, -1);
  if (st == OC_OK) {
#pragma omp parallel for schedule(static) if (M >= 65536)
    for (long m = 0; m < M; m++) a[m] = cmul(a[m], b[m]);
    st = fft_pow2(a, M, +1);
  }
  if (st == OC_OK) {
#pragma omp parallel for schedule(static) if (N >= 65536)
    for (long m = 0; m < N; m++) {
      oc_complex v = {a[m].x / (double)M, a[m].y / (double)M};
      x[m] = cmul(v, c[m]);
    }
  }
  free(a); free(b); free(c);
  return st;
}

/* Stands in for the reference's cuFFT Z2Z transforms (innerLoop.cu:144-152,
 * the W_RLFC-point RLFC FFT; :252-256, the B-point bucket FFT): unnormalised,
 * in place, sign -1 forward.  Bluestein covers the non-power-of-two lengths
 * of the filter design (cuExperiment.cu:277-448). */
int oc_fft(oc_complex *data, long N, int sign) {
  if (N <= 0) return OC_ERR_PARAM;
  if ((N & (N - 1)) == 0) return fft_pow2(data, N, sign);
  return fft_bluestein(data, N, sign);
}

/* ------------------------------------------------------------------------ */
/* A2: flat-window filter design                                             */
/* ------------------------------------------------------------------------ */

/* cuExperiment.cu:593-601 */
static double cheb(double m, double x) {
  if (fabs(x) <= 1) return cos(m * acos(x));
  return cosh(m * acosh(x));
}

static double cabs_ref(oc_complex v) { return sqrt(v.x * v.x + v.y * v.y); }

/* cuExperiment.cu:277-448.  Intended algorithm by default: the boxcar sum of
 * b_f bins is evaluated per block of 4096 outputs from a direct sum plus a
 * short recurrence, and the phase ramp exp(-2 pi i (w/2) i / n) from the exact
 * integer angle.  OC_QUIRK_FILTER_RECURRENCE replays the reference's n-step
 * sequential recurrences instead (cuExperiment.cu:389-396, :410-420). */
int oc_design_filter(const oc_params *p, unsigned quirks, oc_complex *filter_time,
                     oc_complex *filter_freq) {
  const int n = p->n, w = p->w, b_f = p->b_f;
  const double tol = p->tolerance, t0 = p->t0;
  oc_complex *win = (oc_complex *)malloc(sizeof(oc_complex) * (size_t)w);
  oc_complex *g = (oc_complex *)calloc((size_t)n, sizeof(oc_complex));
  if (!win || !g) { free(win); free(g); return OC_ERR_ALLOC; }
  /* Dolph-Chebyshev samples, NaN -> 0 (cuExperiment.cu:538-552) */
#pragma omp parallel for schedule(static) if (w >= 65536)
  for (int i = 0; i < w; i++) {
    double v = cheb(w - 1, t0 * cos(M_PI * i / (w))) * tol;
    win[i].x = isnan(v) ? 0.0 : v;
    win[i].y = 0.0;
  }
  int st = oc_fft(win, w, -1); /* cuExperiment.cu:305-308 */
  if (st != OC_OK) { free(win); free(g); return st; }
  /* rotate right by w/2 (cuShift, cuExperiment.cu:507-522) and drop the
   * imaginary part (makeDolphchebyshevKernel2, :556-564); place the two halves
   * around index 0 of g (:340-352). */
  const int h = w / 2;
  for (int j = 0; j < h; j++) {
    /* shifted[s] = win[(s - h) mod w] */
    int s_hi = h + j;            /* g[j] = shifted[h + j] */
    int s_lo = j;                /* g[n - h + j] = shifted[j] */
    g[j].x = win[(s_hi - h + w) % w].x;
    g[n - h + j].x = win[(s_lo - h + w) % w].x;
  }
  free(win);
  st = oc_fft(g, n, -1); /* :362-365 */
  if (st != OC_OK) { free(g); return st; }
  const int off = b_f / 2;
  double dmax = 0.0;
  if (quirks & OC_QUIRK_FILTER_RECURRENCE) {
    oc_complex s = {0.0, 0.0};
    for (int i = 0; i < b_f; i++) { s.x += g[i].x; s.y += g[i].y; }
    for (int i = 0; i < n; i++) {
      filter_freq[(i + n + off) & (n - 1)] = s;
      double m = cabs_ref(s);
      dmax = dmax > m ? dmax : m;
      s.x += g[(i + b_f) & (n - 1)].x - g[i].x;
      s.y += g[(i + b_f) & (n - 1)].y - g[i].y;
    }
  } else {
    const int BLKB = 4096;
    const int nblk = (n + BLKB - 1) / BLKB;
    double *bmax = (double *)calloc((size_t)nblk, sizeof(double));
    if (!bmax) { free(g); return OC_ERR_ALLOC; }
#pragma omp parallel for schedule(static)
    for (int bi = 0; bi < nblk; bi++) {
      int i0 = bi * BLKB, i1 = i0 + BLKB < n ? i0 + BLKB : n;
      oc_complex s = {0.0, 0.0};
      for (int j = 0; j < b_f; j++) {
        s.x += g[(i0 + j) & (n - 1)].x;
        s.y += g[(i0 + j) & (n - 1)].y;
      }
      double mx = 0.0;
      for (int i = i0; i < i1; i++) {
        filter_freq[(i + off) & (n - 1)] = s;
        double m = cabs_ref(s);
        mx = mx > m ? mx : m;
        s.x += g[(i + b_f) & (n - 1)].x - g[i].x;
        s.y += g[(i + b_f) & (n - 1)].y - g[i].y;
      }
      bmax[bi] = mx;
    }
    for (int bi = 0; bi < nblk; bi++) dmax = dmax > bmax[bi] ? dmax : bmax[bi];
    free(bmax);
  }
  /* makeMultipleKernel1 (:568-577) */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    filter_freq[i].x /= dmax;
    filter_freq[i].y /= dmax;
  }
  /* phase ramp (:410-420) */
  if (quirks & OC_QUIRK_FILTER_RECURRENCE) {
    oc_complex offc = {1.0, 0.0}, step;
    step.x = cos(-2 * M_PI * (w / 2) / n);
    step.y = sin(-2 * M_PI * (w / 2) / n);
    for (int i = 0; i < n; i++) {
      filter_freq[i] = cmul(filter_freq[i], offc);
      offc = cmul(offc, step);
    }
  } else {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
      long long m = ((long long)h * i) % n;
      double ang = -2.0 * M_PI * (double)m / (double)n;
      oc_complex r = {cos(ang), sin(ang)};
      filter_freq[i] = cmul(filter_freq[i], r);
    }
  }
  /* inverse FFT into g, keep the first w entries / n (:425-443) */
  memcpy(g, filter_freq, sizeof(oc_complex) * (size_t)n);
  st = oc_fft(g, n, +1);
  if (st == OC_OK) {
    for (int i = 0; i < w; i++) {
      filter_time[i].x = g[i].x / n;
      filter_time[i].y = g[i].y / n;
    }
  }
  free(g);
  return st;
}

/* ------------------------------------------------------------------------ */
/* A6: cutoff (top-num selection with the reference tie rule)                */
/* ------------------------------------------------------------------------ */

static void swap_d(double *a, double *b) { double t = *a; *a = *b; *b = t; }

/* k-th smallest (0-based) of v[0..len), destroys v (Hoare quickselect). */
static double select_kth_d(double *v, long len, long k) {
  long lo = 0, hi = len - 1;
  while (hi > lo) {
    long mid = lo + (hi - lo) / 2;
    if (v[mid] < v[lo]) swap_d(&v[mid], &v[lo]);
    if (v[hi] < v[lo]) swap_d(&v[hi], &v[lo]);
    if (v[hi] < v[mid]) swap_d(&v[hi], &v[mid]);
    double pivot = v[mid];
    long i = lo, j = hi;
    while (i <= j) {
      while (v[i] < pivot) i++;
      while (v[j] > pivot) j--;
      if (i <= j) { swap_d(&v[i], &v[j]); i++; j--; }
    }
    if (k <= j) hi = j;
    else if (k >= i) lo = i;
    else return v[k];
  }
  return v[k];
}

/* innerLoop.cu:551-616 (+ nth_element_immutable_cuda :624-642): the threshold
 * is element size-num-1 of the ascending order; every sample strictly above it
 * is taken, then samples equal to it in ascending index order until num are
 * taken; the result is sorted ascending. */
void oc_cutoff_f64(const double *samples, int size, int num, int *out) {
  double *tmp = (double *)malloc(sizeof(double) * (size_t)size);
  memcpy(tmp, samples, sizeof(double) * (size_t)size);
  double thr = select_kth_d(tmp, size, (long)size - num - 1);
  free(tmp);
  int gt = 0;
  for (int i = 0; i < size; i++) gt += samples[i] > thr;
  int need_eq = num - gt, c = 0;
  for (int i = 0; i < size; i++) {
    if (samples[i] > thr) out[c++] = i;
    else if (samples[i] == thr && need_eq > 0) { out[c++] = i; need_eq--; }
  }
}

/* oc_cutoff_f64's rule (innerLoop.cu:551-642) on FP32 samples. */
void oc_cutoff_f32(const float *samples, int size, int num, int *out) {
  double *d = (double *)malloc(sizeof(double) * (size_t)size);
  for (int i = 0; i < size; i++) d[i] = samples[i]; /* exact widening */
  oc_cutoff_f64(d, size, num, out);
  free(d);
}

/* The engine's rounding floor (not in the reference): a noiseless signal
 * leaves most RLFC bins at FFT rounding level; reading everything below
 * floor_rel * max as 0 lets those ties resolve by index (the rule above). */
void oc_cutoff_floor_f64(const double *samples, int size, int num, double floor_rel, int *out) {
  if (floor_rel <= 0.0) { oc_cutoff_f64(samples, size, num, out); return; }
  double mx = 0.0;
  for (int i = 0; i < size; i++) mx = samples[i] > mx ? samples[i] : mx;
  const double fl = mx * floor_rel;
  double *d = (double *)malloc(sizeof(double) * (size_t)size);
  for (int i = 0; i < size; i++) d[i] = samples[i] < fl ? 0.0 : samples[i];
  oc_cutoff_f64(d, size, num, out);
  free(d);
}

void oc_cutoff_floor_f32(const float *samples, int size, int num, double floor_rel, int *out) {
  float mx = 0.0f;
  for (int i = 0; i < size; i++) mx = samples[i] > mx ? samples[i] : mx;
  const float fl = floor_rel > 0.0 ? (float)((double)mx * floor_rel) : 0.0f;
  double *d = (double *)malloc(sizeof(double) * (size_t)size);
  for (int i = 0; i < size; i++) d[i] = samples[i] < fl ? 0.0 : (double)samples[i];
  oc_cutoff_f64(d, size, num, out);
  free(d);
}

/* samplesKernel (innerLoop.cu:708-718): re^2 + im^2, each product rounded. */
void oc_samples(const oc_complex *v, int size, double *s) {
#pragma omp parallel for schedule(static) if (size >= 65536)
  for (int i = 0; i < size; i++) s[i] = v[i].x * v[i].x + v[i].y * v[i].y;
}

/* ------------------------------------------------------------------------ */
/* A4: RLFC restriction                                                       */
/* ------------------------------------------------------------------------ */

/* innerLoop.cu:112-161 and restLocFreqCoeffKernel :693-703. */
int oc_rlfc(const oc_complex *x, int n, int W_RLFC, int B_thresh, int offset,
            double floor_rel, int *J2_block, oc_complex *y_f) {
  const int sigma = n / W_RLFC;
  oc_complex *y = (oc_complex *)malloc(sizeof(oc_complex) * (size_t)W_RLFC);
  double *s = (double *)malloc(sizeof(double) * (size_t)W_RLFC);
  if (!y || !s) { free(y); free(s); return OC_ERR_ALLOC; }
  for (int i = 0; i < W_RLFC; i++) y[i] = x[offset + i * sigma];
  int st = oc_fft(y, W_RLFC, -1);
  if (st == OC_OK) {
    oc_samples(y, W_RLFC, s);
    oc_cutoff_floor_f64(s, W_RLFC, B_thresh, floor_rel, J2_block);
    if (y_f) memcpy(y_f, y, sizeof(oc_complex) * (size_t)W_RLFC);
  }
  free(y); free(s);
  return st;
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* outerLoop.cu:111-121: ascending sort (radix_sort_t) then de-duplication. */
int oc_merge_j2(int *J2, int total) {
  if (total <= 0) return 0;
  qsort(J2, (size_t)total, sizeof(int), cmp_int);
  int last = 0;
  for (int i = 1; i < total; i++)
    if (J2[i] != J2[last]) J2[++last] = J2[i];
  return last + 1;
}

/* ------------------------------------------------------------------------ */
/* A5: permutation + filter                                                   */
/* ------------------------------------------------------------------------ */

/* Intended: bins_t[b] = sum_{id = b + j*B < w} x[(id*ai) mod n] * filt[id],
 * taps in ascending j, four explicit fma() per tap:
 *   re = fma(xr, fr, re); re = fma(-xi, fi, re);
 *   im = fma(xr, fi, im); im = fma(xi, fr, im);
 * The permuted index is exact: (id*ai) mod 2^32 reduced mod n (n | 2^32).
 * OC_QUIRK_RESIDUE reproduces permFilterTillKernel (innerLoop.cu:725-757):
 * the partial last tile uses tap id = b*tiles + B for b < w mod B. */
void oc_perm_filter(const oc_complex *x, int n, const oc_complex *filt, int w,
                    int B, int ai, unsigned quirks, oc_complex *bins_t) {
  const int tiles = w / B, residue = w % B;
  const unsigned mask = (unsigned)n - 1u;
#pragma omp parallel for schedule(static) if (B >= 4096)
  for (int b = 0; b < B; b++) {
    double re = 0.0, im = 0.0;
    int ntaps = tiles + (b < residue ? 1 : 0);
    for (int j = 0; j < ntaps; j++) {
      unsigned id = (unsigned)j * (unsigned)B + (unsigned)b;
      if (j == tiles && (quirks & OC_QUIRK_RESIDUE))
        id = (unsigned)b * (unsigned)tiles + (unsigned)B;
      unsigned idx = (id * (unsigned)ai) & mask;
      double xr = x[idx].x, xi = x[idx].y, fr = filt[id].x, fi = filt[id].y;
      re = fma(xr, fr, re);
      re = fma(-xi, fi, re);
      im = fma(xr, fi, im);
      im = fma(xi, fr, im);
    }
    bins_t[b].x = re;
    bins_t[b].y = im;
  }
}

/* ------------------------------------------------------------------------ */
/* A7: reverse hash + voting                                                  */
/* ------------------------------------------------------------------------ */

typedef struct { int first, second; } oc_pair;

static int cmp_pair(const void *a, const void *b) {
  int x = ((const oc_pair *)a)->first, y = ((const oc_pair *)b)->first;
  return (x > y) - (x < y);
}

/* findUpperBound (innerLoop.cu:901-920): first index with first >= val, but
 * the last index when val >= the largest key (the clamp). */
static int find_bound(const oc_pair *P, int num, int val) {
  int lo = 0, hi = num - 1;
  if (val >= P[hi].first) return hi;
  while (hi > lo) {
    int mid = (lo + hi) / 2;
    if (P[mid].first >= val) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

/* reverse_hash (innerLoop.cu:300-384) + reverseHashKernel (:783-817). */
int oc_reverse_hash(const int *J, int B_thresh, const int *J2, int num_RLFC,
                    int n, int B, int W_RLFC, int a, int ai, int loops_thresh,
                    int *vote, int *cand, int *num_cand, int cap) {
  oc_pair *P = (oc_pair *)malloc(sizeof(oc_pair) * (size_t)(num_RLFC > 0 ? num_RLFC : 1));
  if (!P) return OC_ERR_ALLOC;
  for (int m = 0; m < num_RLFC; m++) {
    int prev = (int)(((long long)J2[m] * ai) % W_RLFC);
    P[m].first = prev;
    P[m].second = (int)(((long long)prev * a) % n);
  }
  qsort(P, (size_t)num_RLFC, sizeof(oc_pair), cmp_pair);
  int status = OC_OK;
  for (int t = 0; t < B_thresh && num_RLFC > 0; t++) {
    int low = ((int)(ceil((J[t] - 0.5) * n / B)) + n) & (n - 1);
    int high = ((int)(ceil((J[t] + 0.5) * n / B)) + n) & (n - 1);
    int key = low & (W_RLFC - 1);
    int index = find_bound(P, num_RLFC, key);
    int location = low - key;
    int locinv = (int)(((long long)location * a) % n);
    for (int j = index;; j++) {
      if (j == num_RLFC) {
        j -= num_RLFC;
        location = (location + W_RLFC) & (n - 1);
        locinv = (int)(((long long)location * a) % n);
      }
      int approved = location + P[j].first;
      if ((low < high && (approved >= high || approved < low)) ||
          (low > high && (approved >= high && approved < low)))
        break;
      int loc = (locinv + P[j].second) & (n - 1);
      vote[loc]++;
      if (vote[loc] == loops_thresh) {
        if (*num_cand < cap) cand[*num_cand] = loc;
        else status = OC_ERR_CAPACITY;
        (*num_cand)++;
      }
    }
  }
  free(P);
  return status;
}

/* ------------------------------------------------------------------------ */
/* A8: estimation, A9: top-k                                                  */
/* ------------------------------------------------------------------------ */

static void sort_small(double *v, int len) { /* insertionSortDev, :924-937 */
  for (int i = 1; i < len; i++) {
    double key = v[i];
    int j = i - 1;
    while (j >= 0 && v[j] > key) { v[j + 1] = v[j]; j--; }
    v[j + 1] = key;
  }
}

/* estimateValuesKernel (innerLoop.cu:825-870).  Value per loop:
 *   p = ai*loc mod n, h = p / (n/B), d = p mod (n/B);
 *   if d > (n/B)/2 then h = (h+1) mod B, d -= n/B;
 *   H = filter_freq[(n - d) mod n];
 *   v = (bx*Hx + by*Hy, by*Hx - bx*Hy) / (Hx^2 + Hy^2)
 * every product and sum rounded separately; median of the real and of the
 * imaginary parts taken separately, element (loops-1)/2 of the sorted list. */
void oc_estimate(const int *cand, int num, const oc_complex *bins_f, int loops,
                 int n, const int *permute, int B, const oc_complex *filter_freq,
                 oc_node *out) {
  const int nb = n / B;
#pragma omp parallel for schedule(static) if (num >= 1024)
  for (int i = 0; i < num; i++) {
    double vr[64], vi[64];
    for (int j = 0; j < loops; j++) {
      int pidx = (int)(((long long)permute[j] * cand[i]) % n);
      int h = pidx / nb;
      int d = pidx & (nb - 1);
      if (d > nb / 2) { h = (h + 1) & (B - 1); d -= nb; }
      int dist = (n - d) & (n - 1);
      oc_complex H = filter_freq[dist];
      oc_complex b = bins_f[(size_t)j * B + h];
      double abs2 = H.x * H.x + H.y * H.y;
      double mr = b.x * H.x + b.y * H.y;
      double mi = b.y * H.x - b.x * H.y;
      vr[j] = mr / abs2;
      vi[j] = mi / abs2;
    }
    sort_small(vr, loops);
    sort_small(vi, loops);
    out[i].key = (unsigned)cand[i];
    out[i].value.x = vr[(loops - 1) / 2];
    out[i].value.y = vi[(loops - 1) / 2];
  }
}

static int cmp_desc_d(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x < y) - (x > y);
}

/* cuExperiment.cu:184-193 with a deterministic tie rule: the k largest
 * |value|^2 = x*x + y*y; among equal magnitudes at the threshold the earlier
 * input entries win; the selection keeps input order. */
int oc_topk(const oc_node *nodes, int num, int k, oc_node *out) {
  if (num <= 0 || k <= 0) return 0;
  if (k >= num) { memcpy(out, nodes, sizeof(oc_node) * (size_t)num); return num; }
  double *m = (double *)malloc(sizeof(double) * (size_t)num);
  for (int i = 0; i < num; i++) m[i] = nodes[i].value.x * nodes[i].value.x + nodes[i].value.y * nodes[i].value.y;
  double *srt = (double *)malloc(sizeof(double) * (size_t)num);
  memcpy(srt, m, sizeof(double) * (size_t)num);
  qsort(srt, (size_t)num, sizeof(double), cmp_desc_d);
  double thr = srt[k - 1];
  free(srt);
  int gt = 0;
  for (int i = 0; i < num; i++) gt += m[i] > thr;
  int need = k - gt, c = 0;
  for (int i = 0; i < num; i++) {
    if (m[i] > thr) out[c++] = nodes[i];
    else if (m[i] == thr && need > 0) { out[c++] = nodes[i]; need--; }
  }
  free(m);
  return c;
}

/* ------------------------------------------------------------------------ */
/* A10: the whole outer loop                                                  */
/* ------------------------------------------------------------------------ */

/* outerLoop.cu:65-190 with the RLFC offsets and sigma draws given. The
 * estimation loops' cutoff (whose result the reference never reads,
 * outerLoop.cu:141-146) is skipped. */
int oc_outer_loop(const oc_complex *x, const oc_params *p,
                  const oc_complex *filter_time, const oc_complex *filter_freq,
                  const int *rlfc_offsets, const int *a, const int *ai,
                  unsigned quirks, double floor_rel, oc_node *out, int cap, int *I_F,
                  int *J2_out, int *num_RLFC_out, oc_complex *bins_f_out,
                  int *J_out) {
  const int n = p->n, B = p->B, Bt = p->B_thresh, W = p->W_RLFC;
  const int loops = p->loops;
  int st = OC_OK;
  int *J2 = (int *)malloc(sizeof(int) * (size_t)p->RLFC_loops * Bt);
  oc_complex *bins_f = (oc_complex *)malloc(sizeof(oc_complex) * (size_t)loops * B);
  double *s = (double *)malloc(sizeof(double) * (size_t)B);
  int *J = (int *)malloc(sizeof(int) * (size_t)Bt);
  int *vote = (int *)calloc((size_t)n, sizeof(int));
  int *cand = (int *)malloc(sizeof(int) * (size_t)(cap > 0 ? cap : 1));
  if (!J2 || !bins_f || !s || !J || !vote || !cand) { st = OC_ERR_ALLOC; goto done; }
  for (int r = 0; r < p->RLFC_loops && st == OC_OK; r++)
    st = oc_rlfc(x, n, W, Bt, rlfc_offsets[r], floor_rel, J2 + (size_t)r * Bt, NULL);
  if (st != OC_OK) goto done;
  if (J2_out) memcpy(J2_out, J2, sizeof(int) * (size_t)p->RLFC_loops * Bt);
  int num_RLFC = Bt;
  if (p->RLFC_loops > 1) num_RLFC = oc_merge_j2(J2, p->RLFC_loops * Bt);
  if (num_RLFC_out) *num_RLFC_out = num_RLFC;
  int num_cand = 0;
  for (int i = 0; i < loops; i++) {
    oc_complex *bf = bins_f + (size_t)i * B;
    oc_perm_filter(x, n, filter_time, p->w, B, ai[i], quirks, bf);
    st = oc_fft(bf, B, -1);
    if (st != OC_OK) goto done;
    if (i < p->loops_loc) {
      oc_samples(bf, B, s);
      oc_cutoff_floor_f64(s, B, Bt, floor_rel, J);
      if (J_out) memcpy(J_out + (size_t)i * Bt, J, sizeof(int) * (size_t)Bt);
      int rs = oc_reverse_hash(J, Bt, J2, num_RLFC, n, B, W, a[i], ai[i],
                               p->loops_thresh, vote, cand, &num_cand, cap);
      if (rs != OC_OK) st = rs;
    }
  }
  if (bins_f_out) memcpy(bins_f_out, bins_f, sizeof(oc_complex) * (size_t)loops * B);
  *I_F = num_cand;
  if (st == OC_OK)
    oc_estimate(cand, num_cand, bins_f, loops, n, ai, B, filter_freq, out);
done:
  free(J2); free(bins_f); free(s); free(J); free(vote); free(cand);
  return st;
}
