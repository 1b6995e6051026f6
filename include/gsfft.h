/*
 * gsfft.h -- C ABI of the GB300 (sm_103a) sparse-FFT engine.
 *
 * Two layers:
 *   1. Drop-in entry points with the reference's exact names and signatures
 *      (pcdslab/gpu-sfft outerLoop.h:35-38, innerLoop.h:32-50).  A C program
 *      written against the reference links against libgsfft.so unchanged.
 *   2. The native gsfft_* API: explicit plans, status codes instead of exit(),
 *      caller-chosen CUDA stream, random draws passed in by the caller, FP64 or
 *      mixed (FP32 signal/buckets, FP64 estimate) precision.
 *
 * All pointers named d_* are device pointers (managed memory also works).
 * Every gsfft_* call returns a gsfft_status; none of them exits the process.
 */
#ifndef GSFFT_H_
#define GSFFT_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define GSFFT_VERSION_STRING "0.1.0"

/* ---- types shared with the reference (utils.h:32-51) ------------------- */
#ifndef GSFFT_NO_REFERENCE_TYPES
/* complex_t: same layout as cufftDoubleComplex (utils.h:32-35). */
typedef struct double2C { double x; double y; } complex_t;
/* Node: 4-byte key, 4 bytes padding, 16-byte value (utils.h:42-45). */
typedef struct nodes { unsigned int key; complex_t value; } Node;
/* Pair (utils.h:48-51). */
typedef struct pairs { int first; int second; } Pair;
#endif

/* ---- status codes ------------------------------------------------------ */
typedef enum {
  GSFFT_OK = 0,
  GSFFT_ERR_PARAM = 1,       /* a parameter violates a reference assert or a limit */
  GSFFT_ERR_CAPACITY = 2,    /* candidate list larger than the plan's capacity */
  GSFFT_ERR_ALLOC = 3,       /* device or host allocation failed */
  GSFFT_ERR_CUDA = 4,        /* a CUDA runtime call failed (see gsfft_last_error) */
  GSFFT_ERR_UNSUPPORTED = 5, /* size or mode outside what the library supports */
  GSFFT_ERR_STATE = 6,       /* plan used before gsfft_plan_set_filter, or similar */
  GSFFT_ERR_TIMEOUT = 7      /* a bounded device-side wait gave up (a copy or a
                                tensor-core product never completed); the CUDA
                                context stays usable */
} gsfft_status;

typedef enum { GSFFT_FP64 = 0, GSFFT_MIXED = 1 } gsfft_precision;

/* Plan flags. */
#define GSFFT_FLAG_QUIRK_RESIDUE 1u  /* reproduce permFilterTillKernel's residue
                                        tap index (innerLoop.cu:745-754) */
#define GSFFT_FLAG_RAW_SELECTION 2u  /* cutoffs on the raw |X|^2 values.  By
   default samples below 1e-10 x the row maximum count as exact zeros in the
   RLFC and bucket cutoffs, so that bins which are zero in exact arithmetic
   (half the RLFC picks of a noiseless signal) tie and resolve by ascending
   index, the reference's tie rule, instead of by FFT rounding noise. */
#define GSFFT_FLAG_FORCE_GATHER 4u   /* perm+filter by random gathers (one read per
   tap, innerLoop.cu:725-773 order) even when one ordered pass over the signal
   would move fewer DRAM bytes */
#define GSFFT_FLAG_FORCE_STREAM 8u   /* perm+filter (and the RLFC sub-sampling) by
   one ordered pass over the signal whenever the sizes allow it */
#define GSFFT_FLAG_TC_BUCKET_FFT 16u /* MIXED: the B-point bucket FFT with a
   tensor-core pass (tcgen05, three-part bf16 split products accumulated in
   fp32) for any B it supports: a CUDA-core radix-2^(L-6) pass and a radix-64
   last pass on the tensor cores when B = 2^L with 13 <= L <= 20, else a
   4096-point four-step first pass on the tensor cores and a radix-2^(L-12)
   pass when 17 <= L <= 26.  Without this flag or GSFFT_FLAG_CC_BUCKET_FFT,
   MIXED plans take the radix-64 tensor-core form when 2^17 <= B <= 2^20
   (measured faster on the n = 2^27, k = 16000 step; slower for the smaller
   B of batched small signals) and CUDA-core passes otherwise.  Plans that
   run concurrently (several signals in flight) do better with
   GSFFT_FLAG_CC_BUCKET_FFT. */
#define GSFFT_FLAG_TC_RLFC_FFT 32u   /* MIXED: the same tensor-core radix-4096 first
   pass for the W_RLFC-point RLFC FFT, when W_RLFC = 2^L with 17 <= L <= 26 and
   the plan uses the streaming perm+filter (which writes the sub-samples the
   transform reads) */
#define GSFFT_FLAG_CC_BUCKET_FFT 64u /* MIXED: the bucket FFT on CUDA cores only */

/* Run parameters derived exactly as experiment.c:71-84 and
 * cuExperiment.cu:279-284 derive them. */
typedef struct {
  int q, n, k;
  int B, B_thresh, W_RLFC, RLFC_loops;
  int loops_loc, loops_thresh, loops_est, loops;
  int b_f, w;
  double Bcst, RLFC_cst, BB, lobefrac, tolerance, t0;
} gsfft_params;

/* Replaces experiment.c:54-84 (+ the filter-size computation of
 * cuExperiment.cu:279-284).  Returns GSFFT_ERR_PARAM where the reference
 * would fail an assert (experiment.c:77,82-84; cuExperiment.cu:283) and for
 * the degenerate window layouts this engine rejects (W_RLFC >= n,
 * W_RLFC <= n/B). */
int gsfft_derive_params(int q, int k, double Bcst, int loops_loc, int loops_thresh,
                        int loops_est, double RLFC_cst, int RLFC_loops,
                        double tolerance, gsfft_params *out);

/* Replaces the filter part of make_multiple_t (filters.h:44-48,
 * cuExperiment.cu:277-448), entirely on the GPU in FP64.
 * d_filter_time: p->w taps; d_filter_freq: p->n bins (may be NULL).
 * Allocates its own scratch (about 3 * n * 16 bytes) for the call. */
int gsfft_design_filter(const gsfft_params *p, complex_t *d_filter_time,
                        complex_t *d_filter_freq, void *stream);

/* ---- plans ------------------------------------------------------------- */
typedef struct gsfft_plan_s *gsfft_plan;

/* Allocates every buffer the pipeline needs once (no allocation in
 * gsfft_run).  max_candidates <= 0 selects the reference's MAXSIZE_HITS
 * (utils.h:40, 524288). */
int gsfft_plan_create(const gsfft_params *p, int precision, unsigned flags,
                      int max_candidates, gsfft_plan *out);

/* Stage shapes of a plan that gsfft_plan_create otherwise picks by fixed
 * rules; zero in a field keeps the rule.  gsfft_autotune_plan chooses them by
 * timing. */
typedef struct {
  int perm_filter_form;    /* 1: one ordered pass over the signal, 2: gathers */
  int row_groups;          /* ordered pass: row groups of the signal matrix, each
                              with its own partial bins (power of two) */
  int bucket_first_radix;  /* log2 of the bucket FFT's first-pass radix (two-pass sizes) */
  int rlfc_first_radix;    /* log2 of the RLFC FFT's first-pass radix (two-pass sizes) */
  int select_form;         /* 1: single-launch cutoffs (cluster or cooperative),
                              2: multi-launch radix passes */
} gsfft_plan_tuning;

/* gsfft_plan_create with explicit stage shapes (t may be NULL).  Returns
 * GSFFT_ERR_PARAM for a shape the plan's sizes cannot take. */
int gsfft_plan_create_tuned(const gsfft_params *p, int precision, unsigned flags,
                            int max_candidates, const gsfft_plan_tuning *t, gsfft_plan *out);
/* The stage shapes a plan uses (the rules' choices filled in). */
int gsfft_plan_get_tuning(gsfft_plan plan, gsfft_plan_tuning *out);

/* Autotuner.  Times candidate stage shapes for plans of these parameters on
 * the caller's signal, filter and draws (coordinate descent: perm+filter form
 * and row groups, then each FFT's first-pass radix, then the cutoff form;
 * each candidate the mean of `reps` runs after one warm-up run, CUDA events
 * on `stream`) and returns the fastest in *best, with its time in *best_ms.
 * cache_path (may be NULL): a text file of earlier results, keyed by the
 * device, the precision, the flags that change the pipeline (residue quirk,
 * raw selection, tensor-core and CUDA-core FFT choices) and the plan's sizes;
 * a hit returns at once, a new result is appended.  Allocates and frees
 * candidate plans; synchronises the stream.  GSFFT_ERR_TIMEOUT when a
 * candidate's bounded device-side wait gave up. */
int gsfft_autotune_plan(const gsfft_params *p, int precision, unsigned flags, const void *d_x,
                        const complex_t *d_filter_time, const complex_t *d_filter_freq,
                        const int *h_rlfc_offsets, const int *h_a, const int *h_ai, int reps,
                        const char *cache_path, gsfft_plan_tuning *best, float *best_ms,
                        void *stream);
int gsfft_plan_destroy(gsfft_plan plan);

/* Installs the filter: w time taps and the full n-bin response (only the
 * n/B bins around 0 that the estimate reads are kept). */
int gsfft_plan_set_filter(gsfft_plan plan, const complex_t *d_filter_time,
                          const complex_t *d_filter_freq, void *stream);

/* One sparse FFT (the outer_loop of outerLoop.cu:65-190) on stream.
 * d_x: n complex samples, complex_t (FP64) or {float x, y} (MIXED).
 * h_rlfc_offsets[RLFC_loops], h_a[loops], h_ai[loops]: the random draws of
 * innerLoop.cu:123 and outerLoop.cu:128-134 (ai = a^-1 mod n).
 * Asynchronous: results stay on the device until gsfft_get_results. */
int gsfft_run(gsfft_plan plan, const void *d_x, const int *h_rlfc_offsets,
              const int *h_a, const int *h_ai, void *stream);

/* Synchronises stream and copies the results to host memory:
 * all candidates (I_F Nodes, canonical order) and the k largest by |value|
 * (A9 of the evaluation, cuExperiment.cu:184-193).  Either output may be NULL.
 * Returns GSFFT_ERR_CAPACITY when the candidate list overflowed. */
int gsfft_get_results(gsfft_plan plan, Node *h_nodes, int nodes_cap, int *I_F,
                      Node *h_topk, int topk_cap, int *n_topk, void *stream);

/* Device-side views of the last run's results (valid until the next run). */
int gsfft_device_results(gsfft_plan plan, const Node **d_nodes, const int **d_I_F,
                         const Node **d_topk, const int **d_n_topk);

/* Intermediate stage outputs of the last run, copied to host (for checking):
 * J2 (num_RLFC ids), J (loops_loc * B_thresh ids), bins (loops * B complex,
 * complex_t in FP64, {float,float} in MIXED).  Any pointer may be NULL. */
int gsfft_debug_stages(gsfft_plan plan, int *h_J2, int *num_RLFC, int *h_J,
                       void *h_bins, void *stream);

/* Per-stage CUDA-event timing of gsfft_run (off by default).  Stages, in
 * order: rlfc_fft, rlfc_select, j2_merge, perm_filter, bucket_fft, cutoff,
 * vote, estimate, topk.  gsfft_plan_stage_times synchronises the device,
 * returns the average ms per stage over the runs since the last call and
 * restarts the average. */
int gsfft_plan_enable_timing(gsfft_plan plan, int on);
int gsfft_plan_stage_times(gsfft_plan plan, float *ms_avg, int max_stages, int *runs);
const char *gsfft_stage_name(int stage);

/* Number of kernel launches one gsfft_run issues for this plan. */
int gsfft_plan_launches_per_run(gsfft_plan plan);

/* Form of the perm+filter stage the plan chose: *streaming = 1 when it
 * streams the whole signal once (with *row_groups partial bin sets), 0 when
 * it gathers the loops*w tapped samples. */
int gsfft_plan_describe(gsfft_plan plan, int *streaming, int *row_groups);

/* Which FFTs of the plan have a tensor-core pass: *bucket and *rlfc set to 1
 * or 0. */
int gsfft_plan_tensor_core_ffts(gsfft_plan plan, int *bucket, int *rlfc);

/* ---- batches --------------------------------------------------------- */

/* Strides of the per-plan draw arrays of gsfft_run_batched. */
#define GSFFT_MAX_LOOPS 32
#define GSFFT_MAX_RLFC_LOOPS 8

typedef struct gsfft_batch_s *gsfft_batch;

/* A batch of existing plans (any mix of n, k, parameters and precisions;
 * each plan with its filter installed).  streams: internal CUDA streams the
 * runs are spread over (plan i on stream i mod streams).  The plans stay
 * owned by the caller and must outlive the batch. */
int gsfft_batch_create(const gsfft_plan *plans, int count, int streams, gsfft_batch *out);
int gsfft_batch_destroy(gsfft_batch batch);

/* One sparse FFT per plan: plan i transforms d_x[i] with the draws
 * h_rlfc_offsets[i * GSFFT_MAX_RLFC_LOOPS + r], h_a[i * GSFFT_MAX_LOOPS + l],
 * h_ai[i * GSFFT_MAX_LOOPS + l].  Forks from stream and joins back into it
 * (asynchronous); each plan's results are then read with gsfft_get_results
 * and equal those of gsfft_run on the same input and draws. */
int gsfft_run_batched(gsfft_batch batch, const void *const *d_x, const int *h_rlfc_offsets,
                      const int *h_a, const int *h_ai, void *stream);

/* Graph form of gsfft_run_batched: gsfft_batch_capture records one batched
 * run with these signal buffers and draws into a CUDA graph (nothing runs);
 * every gsfft_batch_launch then replays the whole batch with one graph launch
 * on stream, transforming whatever the captured d_x buffers hold at that
 * time, with the captured draws.  Results are read per plan as usual after a
 * launch.  Capturing again replaces the graph.  Returns GSFFT_ERR_STATE when
 * launched before a capture, GSFFT_ERR_UNSUPPORTED when the CUDA graph
 * cannot be built (the error text says why). */
int gsfft_batch_capture(gsfft_batch batch, const void *const *d_x, const int *h_rlfc_offsets,
                        const int *h_a, const int *h_ai);
int gsfft_batch_launch(gsfft_batch batch, void *stream);

/* Persistent voting: on != 0 makes the batch's runs (gsfft_run_batched, and
 * graphs captured afterwards) queue every plan's front -- run state,
 * perm+filter, FFTs, cutoffs, residue bitmaps -- on its stream, then the
 * reverse-hash voting of all plans in ONE cooperative persistent launch (its
 * blocks take runs of the plans' vote blocks from a device work queue in
 * stage order, with bounded waits that end in GSFFT_ERR_TIMEOUT), then every
 * plan's estimation and top-k on its stream.  Results equal the plans' single
 * runs.  Plans with at most 16 location loops (GSFFT_ERR_UNSUPPORTED
 * otherwise).  Drops a captured graph; on = 0 returns to per-plan voting.
 * Off by default; on 256 small signals it measured 5.96 ms per batch against
 * 6.26 ms with per-plan voting (tuned, 64 streams). */
int gsfft_batch_set_persistent_tail(gsfft_batch batch, int on);

/* ---- host I/O and evaluation ---------------------------------------- */

/* Device memory and copies for callers that do not link the CUDA runtime
 * themselves (the command-line driver).  gsfft_copy copies in any direction
 * (unified addressing) and waits for stream. */
int gsfft_alloc(void **d_ptr, size_t bytes);
int gsfft_free(void *d_ptr);
int gsfft_copy(void *dst, const void *src, size_t bytes, void *stream);
int gsfft_sync(void *stream);

/* Signal ingest (replaces the synchronous host-to-device copy of
 * cuExperiment.cu:113-122): n complex_t samples from host memory into d_x,
 * as complex_t (FP64) or converted to {float, float} on the device (MIXED).
 * Pageable memory goes through two pinned 32 MiB staging chunks so the CPU
 * copy overlaps the DMA; pinned FP64 input is copied directly.  Queued on
 * stream (returns once the last chunk is queued); the staging buffers are
 * created on the first call and kept for the process. */
int gsfft_ingest(const complex_t *h_x, long long n, int precision, void *d_x, void *stream);
/* FP64 -> FP32 conversion of a device signal (n complex samples). */
int gsfft_convert_signal(const complex_t *d_in, void *d_out, long long n, void *stream);

/* Device-side evaluation of the plan's last run (run_experiment,
 * cuExperiment.cu:178-216): missed_estimation = true locations that are not
 * candidates, missed_result = true locations not among the k largest,
 * mse_k = sum over all n bins of |xhat_k - x_f|^2, where x_f (n complex_t on
 * the device) is the normalised DFT of the signal and xhat_k holds the k
 * largest estimates.  d_true_loc: the k_true true locations, ascending and
 * distinct.  Synchronises stream. */
int gsfft_evaluate(gsfft_plan plan, const complex_t *d_x_f, const int *d_true_loc, int k_true,
                   int *missed_estimation, int *missed_result, double *mse_k, void *stream);

/* ---- building blocks (also used by the stage drop-ins) ------------------ */

/* Batched unnormalised complex FFT of power-of-two size n_fft >= 256,
 * out-of-place or in place; sign -1 forward, +1 inverse; precision selects
 * complex_t or {float, float} elements. */
int gsfft_fft(const void *d_in, void *d_out, long long n_fft, int batch, int sign,
              int precision, void *stream);

/* The FP32 FFT of the mixed path's tensor-core plans: batch unnormalised
 * complex FFTs of n_fft = 2^L points, 17 <= L <= 26, {float, float} elements,
 * whose first pass (radix 4096 = 64 x 64, both DFT_64 stages as tcgen05
 * products of three-part bf16 splits accumulated in fp32) runs on the tensor
 * cores and whose second pass (radix 2^(L-12)) on the CUDA cores; sign -1
 * forward, +1 inverse.  Replaces cuFFT's C2C plans of the reference's bucket
 * and RLFC transforms (innerLoop.cu:144-152, :252-256) in single precision. */
int gsfft_fft_tc(const void *d_in, void *d_out, long long n_fft, int batch, int sign,
                 void *stream);

/* The other tensor-core FFT plan, used for the bucket FFT where B allows it:
 * n_fft = 2^L points, 13 <= L <= 20, a CUDA-core first pass of radix
 * 2^(L-6), then a radix-64 last pass as one tcgen05 product per 128
 * sub-transforms (three-part bf16 splits, fp32 accumulation), whose loads and
 * stores move whole 1 KiB runs.  Same arguments and conventions as
 * gsfft_fft_tc. */
int gsfft_fft_tc64(const void *d_in, void *d_out, long long n_fft, int batch, int sign,
                   void *stream);

/* Tensor-core building block of the mixed bucket FFT (the DFT stages that
 * replace cuFFT's B-point transform, innerLoop.cu:247-262): nvec independent
 * forward 64-point DFTs of {float, float} vectors (d_in, d_out: nvec * 64
 * elements), computed with tcgen05 matrix products of three-part bf16 splits
 * accumulated in fp32 (FP32-level accuracy). */
int gsfft_tc_dft64(const void *d_in, void *d_out, int nvec, void *stream);

/* Cutoff (innerLoop.cu:551-616): indices of the num largest samples, ascending;
 * ties at the threshold resolved in ascending index order.  batch independent
 * rows of `size` samples each (double or float per precision). */
int gsfft_cutoff(const void *d_samples, int size, int num, int batch, int precision,
                 int *d_out, void *stream);

/* The cutoff of the pipeline's RLFC and bucket stages: gsfft_cutoff with the
 * selection floor, i.e. samples below floor_rel x the row's largest sample
 * count as exact zeros, so that rounding-level samples tie and resolve by
 * ascending index (innerLoop.cu:591-597's tie rule).  d_row_max: the largest
 * sample of each row (double or float per precision), or NULL to have it
 * computed here.  floor_rel = 0 is gsfft_cutoff.  Synchronises stream. */
int gsfft_cutoff_floor(const void *d_samples, int size, int num, int batch, int precision,
                       double floor_rel, const void *d_row_max, int *d_out, void *stream);

/* No counterpart in the reference.  The same cutoff as gsfft_cutoff (same
 * arguments, same output) for callers that must not allocate device memory
 * while they run: a cudaMalloc/cudaFree can wait for the whole device to go
 * idle and can fail when another allocator of the process holds the free
 * memory.  Its scratch is one fixed device array of this library (under
 * 1 MiB), so the call allocates nothing: at most GSFFT_NOALLOC_MAX_BATCH rows
 * of at most GSFFT_NOALLOC_MAX_SIZE samples; larger requests return
 * GSFFT_ERR_CAPACITY.  The work is queued on `stream` and the call returns
 * without waiting; d_out is ready once the stream reaches that point.
 * The first call in each CUDA context (each device, and again after a
 * cudaDeviceReset) looks up the array's device address (and may load this
 * library's device code there), so make it before any stream capture
 * starts.  Every call on a device shares the array: calls that may overlap in
 * time (other streams, unordered host threads) race and give undefined
 * results; calls ordered on one stream are safe. */
#define GSFFT_NOALLOC_MAX_SIZE (1 << 24)
#define GSFFT_NOALLOC_MAX_BATCH 8
int gsfft_cutoff_noalloc(const void *d_samples, int size, int num, int batch, int precision,
                         int *d_out, void *stream);

/* Stage entry points (one stage of the pipeline on caller buffers).
 * A5 (perm_filter_cutoff's first half, innerLoop.cu:194-240): bins[l*B + b]
 * for l < loops, before the bucket FFT.  d_x / d_bins hold complex_t (FP64)
 * or {float, float} (MIXED); the taps are given as complex_t. */
int gsfft_stage_perm_filter(int precision, const void *d_x, int n,
                            const complex_t *d_filter_time, int w, int B, int loops,
                            const int *h_ai, int quirk_residue, void *d_bins, void *stream);
/* A5 as one ordered pass over x (same sums as gsfft_stage_perm_filter, taps
 * of a bucket added in increasing signal position); h_a = sigma per loop. */
int gsfft_stage_perm_filter_stream(int precision, const void *d_x, int n,
                                   const complex_t *d_filter_time, int w, int B, int loops,
                                   const int *h_a, void *d_bins, void *stream);
/* A7 (reverse_hash, innerLoop.cu:300-384) for one location loop.  d_vote: n
 * entries, epoch << 8 | count (epoch 0 = plain counts, the reference's int
 * table).  Appends to d_cand from *h_count on; *h_count is updated (it may
 * exceed cap, in which case GSFFT_ERR_CAPACITY is returned). */
int gsfft_stage_reverse_hash(const int *d_J, int B_thresh, const int *d_J2, int num_RLFC,
                             int n, int B, int W_RLFC, int a, int ai, int loops_thresh,
                             unsigned epoch, unsigned *d_vote, int *d_cand, int cap,
                             int *h_count, void *stream);
/* A8 (estimate_values, innerLoop.cu:396-466): d_out[i] for i < num. */
int gsfft_stage_estimate(int precision, const int *d_cand, int num, const void *d_bins,
                         int loops, int n, int B, const int *h_ai,
                         const complex_t *d_filter_freq, Node *d_out, void *stream);

/* ---- drop-in entry points with the reference's signatures -------------- */

/* outerLoop.h:35-38.  Draws the RLFC offsets with drand48() and the
 * permutations with random() in the reference's order, runs the FP64 engine
 * with the reference's selection rule (raw |X|^2 cutoffs, no floor) and,
 * below n = 2^27, its residue tap index (the kernel switch at
 * innerLoop.cu:230) and returns a malloc'ed host array of *I_F Nodes
 * (caller frees).  d_filter_size is the tap count w.  Returns NULL on error
 * (message in gsfft_last_error). */
Node *outer_loop(complex_t *d_x, int n, complex_t *d_filter_time,
                 complex_t *d_filter_freq, int d_filter_size, int B, int B_thresh,
                 int W_RLFC, int RLFC_loops, int loop_threshold, int loops_loc,
                 int loops, int *I_F, float t_H_to_D);

/* innerLoop.h:32-50.  Same arguments and effects as the reference; the timing
 * accumulators are advanced by the CUDA-event time of the call. */
int restr_loc_freq_coeff(complex_t *d_x, int n, int B_thresh, int W_RLFC, int *d_J2,
                         double *RLFC_Time);
int samples_indices(complex_t *d_samp, int B, int samp_size, int *d_output,
                    double *CTime);
int perm_filter_cutoff(complex_t *d_x, int n, complex_t *d_filter_time,
                       int d_filter_size, int B_thresh, int B, int a, int ai,
                       complex_t *d_bins_f, int *d_J, double *PF_T, double *BC_T);
int reverse_hash(int *d_J, int n, int B_thresh, int B, int a, int ai, int loop_thresh,
                 int *d_vote, int *d_I, int *I_F, double *G_T, int *d_J2,
                 int num_RLFC, int W_RLFC, int RLFC_loops);
Node *estimate_values(int *d_I, int *I_F, complex_t *d_bins_f, int loops, int n,
                      int *permute, int B, complex_t *d_filter_freq, int loops_loc);
int timesmod(const int x, const int a, const int n);

/* Failure-detection self-check.  One CTA waits, with the bounded mbarrier
 * wait every kernel of this library uses, on a barrier that nothing arrives
 * on (no copy or product is issued against it) and gives up after
 * limit_cycles SM clock cycles (1 .. 2^31).  Returns GSFFT_ERR_TIMEOUT, the
 * status a run reports when one of its waits gives up; the CUDA context stays
 * usable.  Synchronises stream. */
int gsfft_check_bounded_wait(long long limit_cycles, void *stream);

/* ---- misc -------------------------------------------------------------- */
const char *gsfft_version(void);
const char *gsfft_last_error(void);
const char *gsfft_status_string(int status);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* GSFFT_H_ */
