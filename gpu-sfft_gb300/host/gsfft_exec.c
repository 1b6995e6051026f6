/*
 * gsfft_exec -- command-line driver with the reference binary's interface:
 *
 *   gsfft_exec q k Bcst loops_loc loops_thresh loops_est RLFC_cst RLFC_loops
 *              [--mixed] [--reps R] [--seed S]
 *
 * (the eight arguments of experiment.c:48-63).  It builds the reference's
 * test signal (k locations drawn with drand48, coefficients 1 + 0i, signal =
 * inverse DFT, cuExperiment.cu:84-92), designs the filter on the GPU, runs
 * the sparse FFT R times and prints the reference's report: filter
 * parameters (experiment.c:87-95), the timing table of outerLoop.cu:174-187
 * and the error line of cuExperiment.cu:217-220.  --mixed runs the FP32 /
 * FP64-estimate engine instead of the FP64 one; --seed seeds drand48 and
 * random() (the reference never seeds them).
 *
 * Timing-table columns from this engine's stages: votetable = 0 (the vote
 * table is epoch-tagged and never cleared), restr-loc-index = RLFC FFT +
 * RLFC cutoff + J2 merge, perm+filter, reverse-hash = voting, estimation =
 * estimation + top-k, FFT+Cutoff = bucket FFT + cutoff, other = the rest of
 * the wall time of a run.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gsfft.h"

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

#define CHECK(call)                                                                   \
  do {                                                                                \
    int s_ = (call);                                                                  \
    if (s_ != GSFFT_OK) {                                                             \
      fprintf(stderr, "%s failed: %s (%s)\n", #call, gsfft_status_string(s_),         \
              gsfft_last_error());                                                    \
      exit(1);                                                                        \
    }                                                                                 \
  } while (0)

static int cmp_int(const void *a, const void *b) {
  const int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* RLFC offsets with drand48 (innerLoop.cu:123), then per loop a random odd
 * multiplier and its inverse mod n (outerLoop.cu:128-134). */
static void draw(int n, int W, int R, int loops, int *offs, int *a, int *ai) {
  const int sigma = n / W;
  for (int r = 0; r < R; r++) offs[r] = (int)(unsigned)floor(drand48() * sigma);
  for (int i = 0; i < loops; i++) {
    int av = 0;
    while ((av & 1) == 0) av = (int)(random() % n);
    unsigned inv = (unsigned)av;
    for (int it = 0; it < 5; it++) inv *= 2u - (unsigned)av * inv;
    a[i] = av;
    ai[i] = (int)(inv & (unsigned)(n - 1));
  }
}

int main(int argc, char **argv) {
  if (argc < 9) {
    fprintf(stderr,
            "usage: %s q k Bcst loops_loc loops_thresh loops_est RLFC_cst RLFC_loops "
            "[--mixed] [--reps R] [--seed S]\n",
            argv[0]);
    return 1;
  }
  const int q = atoi(argv[1]), k = atoi(argv[2]);
  const double Bcst = strtod(argv[3], 0);
  const int loops_loc = atoi(argv[4]), loops_thresh = atoi(argv[5]), loops_est = atoi(argv[6]);
  const double RLFC_cst = atoi(argv[7]);
  const int RLFC_loops = atoi(argv[8]);
  int precision = GSFFT_FP64, reps = 1;
  for (int i = 9; i < argc; i++) {
    if (!strcmp(argv[i], "--mixed")) precision = GSFFT_MIXED;
    else if (!strcmp(argv[i], "--reps") && i + 1 < argc) reps = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--seed") && i + 1 < argc) {
      const long sd = atol(argv[++i]);
      srand48(sd);
      srandom((unsigned)sd);
    }
  }
  if (reps < 1) reps = 1;

  gsfft_params p;
  CHECK(gsfft_derive_params(q, k, Bcst, loops_loc, loops_thresh, loops_est, RLFC_cst, RLFC_loops,
                            1e-8, &p));
  const int n = p.n;
  printf("\n\nRUNNING EXPERIMENT: n:%d k:%d loops_loc=%d loops_est:%d\n", n, k, loops_loc, loops_est);
  printf("\nGPU-SFFT filter parameters for: n=%d, k=%d.\n", n, k);
  printf("******************************************************************************\n\n");
  printf(" RLFC Filter: RLFC_loops: %d  B_thresh:%d W_RLFC: %d\n \n", p.RLFC_loops, p.B_thresh,
         p.W_RLFC);
  printf(" Filter: (numlobes=%.1lf, tolerance=%lg, b_f=%d) B: %d \n\n", 0.5 / p.lobefrac,
         p.tolerance, p.b_f, p.B);

  /* test signal: spectrum X on the host, signal = inverse DFT on the device */
  int *large = (int *)malloc(sizeof(int) * k);
  complex_t *hX = (complex_t *)calloc((size_t)n, sizeof(complex_t));
  if (!large || !hX) {
    fprintf(stderr, "host allocation failed\n");
    return 1;
  }
  for (int i = 0; i < k; i++) {
    large[i] = (int)(unsigned)floor(drand48() * n);
    hX[large[i]].x = 1.0;
    hX[large[i]].y = 0.0;
  }
  complex_t *dX = NULL, *dx = NULL;
  void *dx32 = NULL;
  CHECK(gsfft_alloc((void **)&dX, sizeof(complex_t) * (size_t)n));
  CHECK(gsfft_alloc((void **)&dx, sizeof(complex_t) * (size_t)n));
  double t0 = now_s();
  CHECK(gsfft_ingest(hX, n, GSFFT_FP64, dX, NULL));
  CHECK(gsfft_sync(NULL));
  const double t_h2d = now_s() - t0;
  CHECK(gsfft_fft(dX, dx, n, 1, +1, GSFFT_FP64, NULL)); /* x = sum_f X_f e^{+2 pi i f t / n} */
  if (precision == GSFFT_MIXED) {
    CHECK(gsfft_alloc(&dx32, sizeof(float) * 2 * (size_t)n));
    CHECK(gsfft_convert_signal(dx, dx32, n, NULL));
  }

  printf(" computing filter starts\n \n");
  complex_t *dft = NULL, *dff = NULL;
  CHECK(gsfft_alloc((void **)&dft, sizeof(complex_t) * (size_t)p.w));
  CHECK(gsfft_alloc((void **)&dff, sizeof(complex_t) * (size_t)n));
  t0 = now_s();
  CHECK(gsfft_design_filter(&p, dft, dff, NULL));
  CHECK(gsfft_sync(NULL));
  const double t_filter = now_s() - t0;
  printf(" Window size: Filter : %d\n \n", p.w);
  printf(" Time for computing  filter:  %lfs\n \n", t_filter);
  printf("******************************************************************************\n\n");
  printf("Simulation starting:\n\n");
  printf("GPU-SFFT Results (%s engine)\n", precision == GSFFT_MIXED ? "mixed" : "FP64");
  printf("******************************************************************************\n\n");

  gsfft_plan plan;
  CHECK(gsfft_plan_create(&p, precision, 0, 0, &plan));
  CHECK(gsfft_plan_set_filter(plan, dft, dff, NULL));
  int offs[8], a[32], ai[32];
  /* one untimed run builds the device state (twiddles, tensor maps) */
  draw(n, p.W_RLFC, p.RLFC_loops, p.loops, offs, a, ai);
  CHECK(gsfft_run(plan, precision == GSFFT_MIXED ? dx32 : (void *)dx, offs, a, ai, NULL));
  CHECK(gsfft_sync(NULL));
  CHECK(gsfft_plan_enable_timing(plan, 1));
  double wall = 0.0;
  for (int r = 0; r < reps; r++) {
    draw(n, p.W_RLFC, p.RLFC_loops, p.loops, offs, a, ai);
    t0 = now_s();
    CHECK(gsfft_run(plan, precision == GSFFT_MIXED ? dx32 : (void *)dx, offs, a, ai, NULL));
    CHECK(gsfft_sync(NULL));
    wall += now_s() - t0;
  }
  wall /= reps;
  float ms[16];
  int runs = 0;
  CHECK(gsfft_plan_stage_times(plan, ms, 16, &runs));
  double st[16];
  for (int i = 0; i < 16; i++) st[i] = 0;
  for (int i = 0; i < 9; i++) {
    const char *nm = gsfft_stage_name(i);
    const double v = ms[i] * 1e-3;
    if (!strcmp(nm, "rlfc_fft") || !strcmp(nm, "rlfc_select") || !strcmp(nm, "j2_merge")) st[1] += v;
    else if (!strcmp(nm, "perm_filter")) st[2] += v;
    else if (!strcmp(nm, "vote")) st[3] += v;
    else if (!strcmp(nm, "estimate") || !strcmp(nm, "topk")) st[4] += v;
    else if (!strcmp(nm, "bucket_fft") || !strcmp(nm, "cutoff")) st[5] += v;
  }
  const double DDD = wall;
  const double other = DDD - st[1] - st[2] - st[3] - st[4] - st[5];
  printf("Total GPU-SFFT time: %lf\n", DDD);
  printf("Time distribution: votetable  restr-loc-index  perm+filter reverse-hash  estimation FFT+Cutoff    other    total\n");
  printf("                    %2.4lf       %2.4lf          %2.4lf      %2.4lf        %2.4lf     %2.4lf      %2.4lf   %2.4lf\n",
         st[0], st[1], st[2], st[3], st[4], st[5], other, DDD);
  const double tott = DDD / 100;
  printf("                    %4.1f%%         %4.1f%%           %4.1f%%      %4.1f%%         %4.1f%%      %4.1f%%       %4.1f%%   %5.1f%%\n",
         st[0] / tott, st[1] / tott, st[2] / tott, st[3] / tott, st[4] / tott, st[5] / tott,
         other / tott, DDD / tott);
  printf("\n");
  printf("HtoD time = %lfs, HtoD time/total time  = %lf%%, total time + HtoD time = %lfs \n", t_h2d,
         t_h2d / tott, DDD + t_h2d);

  /* results and device-side evaluation against X (= the normalised DFT of x) */
  Node *top = (Node *)malloc(sizeof(Node) * (size_t)k);
  int n_top = 0, I_F = 0;
  t0 = now_s();
  CHECK(gsfft_get_results(plan, NULL, 0, &I_F, top, k, &n_top, NULL));
  const double t_extract = now_s() - t0;
  qsort(large, k, sizeof(int), cmp_int);
  int kd = 0;
  for (int i = 0; i < k; i++)
    if (i == 0 || large[i] != large[i - 1]) large[kd++] = large[i];
  int *dtrue = NULL;
  CHECK(gsfft_alloc((void **)&dtrue, sizeof(int) * (size_t)kd));
  CHECK(gsfft_copy(dtrue, large, sizeof(int) * (size_t)kd, NULL));
  int miss_est = 0, miss_res = 0;
  double err = 0.0;
  CHECK(gsfft_evaluate(plan, dX, dtrue, kd, &miss_est, &miss_res, &err, NULL));
  printf("\nERROR:\n");
  printf("K=%d; MISSED (estimation, result) = (%d, %d), MSE*k = %lg, Mean Square Error (MSE) = %lg\n",
         k, miss_est, miss_res, err, err / k);
  printf("time to extract the values of the largest frequencies: %lfs \n", t_extract);
  printf("******************************************************************************\n\n");
  printf("candidates I_F = %d, distinct true locations = %d, runs timed = %d\n", I_F, kd, runs);

  gsfft_plan_destroy(plan);
  gsfft_free(dtrue);
  gsfft_free(dft);
  gsfft_free(dff);
  gsfft_free(dX);
  gsfft_free(dx);
  gsfft_free(dx32);
  free(top);
  free(hX);
  free(large);
  return 0;
}
