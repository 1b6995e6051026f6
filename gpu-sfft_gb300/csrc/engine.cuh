// Plan object and orchestration entry points.
#pragma once
#include "stages.cuh"

#include <vector>

namespace gsfft {

enum Stage {
  ST_RLFC_FFT = 0, ST_RLFC_SELECT, ST_J2, ST_PERM_FILTER, ST_BUCKET_FFT, ST_CUTOFF, ST_VOTE,
  ST_ESTIMATE, ST_TOPK, ST_COUNT
};

struct Plan {
  gsfft_params p;
  int precision = 0;
  unsigned flags = 0;
  int cap = 0;
  size_t es = 16;
  bool filter_set = false;
  bool ran = false;
  unsigned epoch = 0;            // host mirror of *d_epoch after the last queued run
  unsigned *d_epoch = nullptr;   // device copy, advanced by each run's first kernel
  int launches_per_run = 0;
  FftPlan fftB, fftW;
  SelectScratch selB, selW, selK;
  void *filt = nullptr;
  double2 *hinv = nullptr;
  void *rsamp = nullptr;
  int *J2b = nullptr, *J2 = nullptr;
  void *bins = nullptr, *bsamp = nullptr;
  int *J = nullptr;
  unsigned *bm_j2 = nullptr, *bm_sig = nullptr, *tile_tmp = nullptr;
  unsigned *vote = nullptr;  // n epoch-tagged entries, or n/16 words of 2-bit counters
  bool packed_vote = false;  // 2-bit counters (at most 3 location loops)
  int *cand = nullptr, *cnt = nullptr, *blk = nullptr;
  DevNode *nodes = nullptr;
  double *mag2 = nullptr;
  int *topk_idx = nullptr;
  DevNode *topk = nullptr;
  RunCtl *ctl = nullptr;
  void *rmax = nullptr;  // per-row maxima: RLFC_loops rows then loops rows (u64 each)
  void *ybuf = nullptr;  // RLFC sub-samples written by the streaming perm+filter
  void *bpart = nullptr; // row-group partial bins of the streaming perm+filter
  void *filt_bm = nullptr; // bucket-major taps of the streaming perm+filter
  int groups = 1;
  bool use_stream = false;
  bool tc_bucket = false;  // bucket FFT with tensor-core passes
  bool tc_rlfc = false;    // RLFC FFT with a tensor-core first pass
  double floor_rel = 1e-10;
  gsfft_plan_tuning tuning = {};  // the stage shapes in use (rules' choices filled in)
  Draws draws = {};               // the draws of the last front phase queued
  Draws *d_draws = nullptr;       // device copy of them (phased runs)
  // optional per-stage CUDA-event timing (one event set per run, up to 512 runs)
  // side stream of the bucket FFT and cutoff (they need only the perm+filter)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_bins = nullptr;  // the estimation loops' bucket FFT is done
  cudaEvent_t ev_rsel = nullptr;  // the RLFC cutoff has been queued on the main stream
  cudaStream_t aux = nullptr;     // clears the packed vote table beside the FFTs
  cudaEvent_t ev_vclr = nullptr;  // the next run's packed vote table is clear
  bool vclr_eager = false;        // ev_vclr last recorded by an eager run (not in a capture)
  cudaEvent_t ev_voted = nullptr; // this run's voting is done
  bool timing = false;
  std::vector<cudaEvent_t> events;  // 2 * ST_COUNT per recorded run (begin, end)
  int timed_runs = 0;
};

int validate_params(const gsfft_params &p);
int plan_create(const gsfft_params &p, int precision, unsigned flags, int max_candidates,
                Plan **out, const gsfft_plan_tuning *tuning = nullptr);
void plan_destroy(Plan *P);
int plan_set_filter(Plan *P, const void *d_filter_time, const void *d_filter_freq,
                    cudaStream_t st);
// capturing = true while a CUDA graph records the run: the host-side epoch
// bookkeeping and stage timing are then left to whoever launches the graph.
// phases: which part of the run to queue -- PH_FRONT (run state, perm+filter,
// FFTs, cutoffs, residue bitmaps; takes the draws), PH_VOTE (voting), PH_EST
// (estimation), PH_TOPK (the k largest) -- so that a batch can run the voting
// of all its plans in one persistent launch between the fronts and the rest.
enum { PH_FRONT = 1, PH_VOTE = 2, PH_TOPK = 4, PH_EST = 8, PH_ALL = 15 };
int plan_run(Plan *P, const void *d_x, const int *offs, const int *a, const int *ai,
             cudaStream_t st, bool capturing = false, int phases = PH_ALL);
// host side of a run's epoch step (clears the vote table when the 24-bit
// epoch would wrap); called once per queued run, before the run's kernels
int plan_epoch_advance(Plan *P, cudaStream_t st);
int plan_results(Plan *P, Node *h_nodes, int nodes_cap, int *I_F, Node *h_topk, int topk_cap,
                 int *n_topk, cudaStream_t st);
int plan_enable_timing(Plan *P, bool on);
int plan_stage_times(Plan *P, float *ms_avg, int max_stages, int *runs);
const char *stage_name(int i);
int plan_debug(Plan *P, int *h_J2, int *num_RLFC, int *h_J, void *h_bins, cudaStream_t st);

int launch_hinv(const double2 *d_ff, int n, int nb, double2 *hinv, cudaStream_t st);
int launch_vote_clear(unsigned *vote, int n, const unsigned *d_epoch, cudaStream_t st);
int launch_convert_taps(const double2 *d_ft, void *dst, int w, bool to_float, cudaStream_t st);

// persistent tail of a batch (batch_tail.cu): the voting of every plan in
// one cooperative launch
struct BatchTail;
int batch_tail_create(Plan *const *plans, int count, BatchTail **out);
int batch_tail_launch(BatchTail *t, cudaStream_t st);
void batch_tail_free(BatchTail *t);

// batched runs over several plans (batch.cu)
struct Batch;
int batch_create(Plan *const *plans, int count, int nstreams, Batch **out);
int batch_run(Batch *b, const void *const *d_x, const int *offs, const int *a, const int *ai,
              cudaStream_t st, bool capturing = false);
int batch_capture(Batch *b, const void *const *d_x, const int *offs, const int *a, const int *ai);
int batch_launch(Batch *b, cudaStream_t st);
void batch_destroy(Batch *b);
int batch_set_persistent_tail(Batch *b, bool on);

// signal ingest and device-side evaluation (host_io.cu)
int launch_to_float(const complex_t *in, void *out, long long n, cudaStream_t st);
int ingest(const complex_t *h_x, long long n, int precision, void *d_x, cudaStream_t st);
int plan_evaluate(Plan *P, const complex_t *d_xf, const int *d_true_loc, int k_true,
                  int *missed_est, int *missed_res, double *err, cudaStream_t st);

// A2 filter design on the GPU
int design_filter(const gsfft_params &p, double2 *d_ft, double2 *d_ff, cudaStream_t st);

}  // namespace gsfft
