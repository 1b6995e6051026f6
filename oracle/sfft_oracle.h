/*
 * sfft_oracle.h -- CPU restatement of the pcdslab/gpu-sfft sparse-FFT pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * engine in gpu-sfft_gb300/: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load it.  The product never links,
 * calls or falls back to it.
 *
 * Every function restates the reference algorithm in plain C (FP64), cites the
 * reference file:line it follows, and is deterministic: fixed summation order,
 * no FMA contraction except where an explicit fma() is part of the stated
 * operation sequence, and a canonical output order wherever the reference's
 * order depends on atomics.
 *
 * Parity is pinned by (a) the parameter KATs printed in the reference README
 * (README.md:84-90) and (b) golden vectors produced by the reference's own
 * stage functions (innerLoop.h:32-50) and its outer_loop (outerLoop.cu:65-190),
 * built from the reference's sources and run on a GB300 (oracle/build_ref.py,
 * tests/golden/make_ref_fixtures.py); tests/test_ref_golden.py checks this
 * restatement against them.
 */
#ifndef SFFT_ORACLE_H_
#define SFFT_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as the reference complex_t (utils.h:32-35). */
typedef struct { double x, y; } oc_complex;
/* Same layout as the reference Node (utils.h:42-45): 4-byte key, 4 pad, 16 value. */
typedef struct { unsigned int key; oc_complex value; } oc_node;

/* Derived run parameters, experiment.c:54-84 and cuExperiment.cu:279-284. */
typedef struct {
  int q, n, k;
  int B, B_thresh, W_RLFC, RLFC_loops;
  int loops_loc, loops_thresh, loops_est, loops;
  int b_f, w;
  double Bcst, RLFC_cst, BB, lobefrac, tolerance, t0;
} oc_params;

/* Quirk switches (default 0 = intended algorithm). */
#define OC_QUIRK_RESIDUE   1u  /* perm+filter residue tap index j*tiles+B (innerLoop.cu:745-754) */
#define OC_QUIRK_FILTER_RECURRENCE 2u /* boxcar + phase ramp by sequential recurrence (cuExperiment.cu:389-420) */

/* Status codes (0 = ok). */
#define OC_OK 0
#define OC_ERR_PARAM 1      /* a reference assert would fire */
#define OC_ERR_CAPACITY 2   /* candidate list capacity exceeded */
#define OC_ERR_ALLOC 3

int  oc_floor_to_pow2(double x);
int  oc_gcd(int a, int b);
int  oc_mod_inverse(int a, int n);
int  oc_derive_params(int q, int k, double Bcst, int loops_loc, int loops_thresh,
                      int loops_est, double RLFC_cst, int RLFC_loops,
                      double tolerance, oc_params *out);

/* glibc random streams in the reference's order: RLFC offsets from drand48()
 * (innerLoop.cu:122-123), then per loop a = random()%n until gcd(a,n)==1 and
 * ai = a^-1 mod n (outerLoop.cu:128-134).  seed < 0 keeps the current (e.g.
 * default, never seeded) glibc state; seed >= 0 calls srand48(seed) and
 * srandom(seed) first. */
void oc_draw_glibc(long seed, int n, int W_RLFC, int RLFC_loops, int loops,
                   int *rlfc_offsets, int *a, int *ai);

/* Forward (sign -1) / inverse (sign +1) unnormalised complex DFT of any size
 * (radix-2 for powers of two, Bluestein otherwise).  In place. */
int  oc_fft(oc_complex *data, long N, int sign);

/* A2: flat-window filter (cuExperiment.cu:277-448).  filter_time: w taps,
 * filter_freq: n bins. */
int  oc_design_filter(const oc_params *p, unsigned quirks,
                      oc_complex *filter_time, oc_complex *filter_freq);

/* A6 cutoff: indices of the num largest samples, ascending (innerLoop.cu:551-616). */
void oc_cutoff_f64(const double *samples, int size, int num, int *out);
void oc_cutoff_f32(const float *samples, int size, int num, int *out);
/* Same with the engine's rounding floor: samples below floor_rel * max are
 * taken as exact zeros (floor = max * floor_rel rounded in double, then to the
 * sample type). floor_rel = 0 is the plain cutoff. */
void oc_cutoff_floor_f64(const double *samples, int size, int num, double floor_rel, int *out);
void oc_cutoff_floor_f32(const float *samples, int size, int num, double floor_rel, int *out);

/* |v|^2 without contraction (innerLoop.cu:715). */
void oc_samples(const oc_complex *v, int size, double *samples);

/* A4 one RLFC loop (innerLoop.cu:112-161 + :693-703): J2 block of B_thresh ids. */
int  oc_rlfc(const oc_complex *x, int n, int W_RLFC, int B_thresh, int offset,
             double floor_rel, int *J2_block, oc_complex *y_f /* W_RLFC or NULL */);

/* Sorted, de-duplicated union of RLFC_loops blocks (outerLoop.cu:111-121). */
int  oc_merge_j2(int *J2, int total);

/* A5 perm+filter (innerLoop.cu:194-240, :725-773): bins_t[B]. */
void oc_perm_filter(const oc_complex *x, int n, const oc_complex *filt, int w,
                    int B, int ai, unsigned quirks, oc_complex *bins_t);

/* A7 reverse hash + vote for one location loop (innerLoop.cu:300-384, :783-817,
 * :894-920).  Appends candidates in canonical order (bucket order of J, then
 * position ascending circularly from the window's low end). */
int  oc_reverse_hash(const int *J, int B_thresh, const int *J2, int num_RLFC,
                     int n, int B, int W_RLFC, int a, int ai, int loops_thresh,
                     int *vote, int *cand, int *num_cand, int cap);

/* A8 estimation (innerLoop.cu:396-466, :825-870). */
void oc_estimate(const int *cand, int num, const oc_complex *bins_f, int loops,
                 int n, const int *permute, int B, const oc_complex *filter_freq,
                 oc_node *out);

/* A9 top-k by |value| (cuExperiment.cu:184-193): keeps input order. */
int  oc_topk(const oc_node *nodes, int num, int k, oc_node *out);

/* A10 whole pipeline (outerLoop.cu:65-190) with explicit draws.
 * Optional stage outputs may be NULL: J2_out (RLFC_loops*B_thresh),
 * bins_f_out (loops*B), J_out (loops_loc*B_thresh). */
int  oc_outer_loop(const oc_complex *x, const oc_params *p,
                   const oc_complex *filter_time, const oc_complex *filter_freq,
                   const int *rlfc_offsets, const int *a, const int *ai,
                   unsigned quirks, double floor_rel, oc_node *out, int cap, int *I_F,
                   int *J2_out, int *num_RLFC_out, oc_complex *bins_f_out,
                   int *J_out);

int  oc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
