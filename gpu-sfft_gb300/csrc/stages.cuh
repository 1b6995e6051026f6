// Stage kernels of the sparse-FFT pipeline (launch helpers).
#pragma once
#include "gsfft_internal.cuh"

namespace gsfft {

constexpr int MAX_LOOPS = 32;
constexpr int MAX_RLFC_LOOPS = 8;

// Random draws of one run, passed by value to the kernels that need them.
struct Draws {
  int offs[MAX_RLFC_LOOPS];  // RLFC offsets (innerLoop.cu:123)
  int a[MAX_LOOPS];          // sigma (outerLoop.cu:131)
  int ai[MAX_LOOPS];         // sigma^-1 mod n (outerLoop.cu:133)
};

// Device-side state of one run.
struct RunCtl {
  int cand_count;      // candidates appended so far (may exceed capacity)
  int overflow;        // set when cand_count > capacity
  int num_rlfc;        // |J2|
  int n_topk;
  int fmax[MAX_LOOPS]; // largest permuted residue per location loop
  unsigned ticket;
  int err;  // a bounded device-side wait gave up (streaming perm+filter,
            // tensor-core FFT passes, persistent batch voting)
  int pad[2];
};

struct DevNode {  // == Node (utils.h:42-45)
  unsigned key;
  unsigned pad;
  double x, y;
};

// A5: bins[l][b] = sum_{id=b+jB<w} x[(id*ai_l) mod n] * filt[id]  (all loops)
int launch_perm_filter(int precision, const void *x, int n, const void *filt, int w, int B,
                       int loops, const Draws &d, bool quirk_residue, void *bins, cudaStream_t st);

// A5 (and the RLFC sub-sampling) as one ordered pass over x; y receives
// RLFC_loops rows of W samples (x[off_r + m*n/W]).  FP64 or FP32.
bool stream_pf_supported(int n, int B, int loops, int W, int RLFC_loops);
// Row groups of the streaming pass: it writes `groups` partial bin arrays
// (groups x loops x B), to be added in group order.
int stream_pf_groups(int n, int B, int w, int loops, int precision);
int launch_sum_partials(int precision, const void *part, int groups, long long count, void *out,
                        cudaStream_t st);
// Bucket-major tap table of the streaming pass: taps_bm[b * TT + j] =
// filt[j * B + b] (zero past w), TT = w/B + 1 rounded up to even (rows of a
// multiple of 16 bytes); stream_taps_count elements.
int stream_taps_count(int w, int B);
int launch_stream_taps(int precision, const void *filt, int w, int B, void *taps_bm, cudaStream_t st);
// filt here is the bucket-major table
// groups: row groups (partial bin sets) of the pass; 0 = stream_pf_groups
int launch_perm_filter_stream(int precision, const void *x, int n, const void *filt, int w, int B,
                              int loops, const Draws &d, void *bins, int nrlfc, void *y, int W,
                              int *err, cudaStream_t st, int groups = 0);
// whether `groups` row groups suit the streaming pass at this shape (one, or
// a power of two leaving at least four tiles of rows per group)
bool stream_pf_groups_valid(int n, int B, int groups, int precision);

// J2 = sorted distinct union of the RLFC blocks, through a W-bit bitmap.
int launch_j2_merge(const int *J2_blocks, int total, int W, unsigned *bitmap, int *J2,
                    RunCtl *ctl, unsigned *tile_tmp, cudaStream_t st);

// Permuted-residue bitmaps F_l = {J2[m] * ai_l mod W} for the location loops,
// and fmax_l = max F_l.
int launch_sigma_bitmaps(const int *J2, const RunCtl *ctl_num, int max_num, int W, int loops_loc,
                         const Draws &d, unsigned *bitmaps, RunCtl *ctl, cudaStream_t st);

// The same bitmaps and fmax_l straight from the RLFC blocks (total ids, with
// duplicates); the bitmaps and ctl->fmax must be zero on entry.
int launch_sigma_from_blocks(const int *J2b, int total, int W, int loops_loc, const Draws &d,
                             unsigned *bitmaps, RunCtl *ctl, cudaStream_t st);

// A7: one location loop of voting; appends candidates in canonical order.
// epoch: device word with the run's epoch (vote entries are epoch << 8 | count).
// may_complete = false (location loop l < loops_thresh - 1 of a run, where no
// count can reach the threshold) only records the votes.
int launch_vote_loop(int l, const int *J, int B_thresh, int n, int B, int W,
                     const unsigned *bitmap_l, const Draws &d, int loops_thresh, const unsigned *epoch,
                     unsigned *vote, int *cand, int cap, int *cnt, int *blk, RunCtl *ctl,
                     bool may_complete, cudaStream_t st, bool packed = false);
// ints needed by the blk scratch of launch_vote_loop
int vote_block_ints(int B_thresh);

// A8: estimates + |value|^2 keys for the candidates.
// cap: candidate capacity; the grid is sized for `expect` candidates (a
// grid-stride loop covers up to cap)
// bytes of the reciprocal filter-response table: nb + 1 double2, then the
// same values as float2 (hinv_kernel writes both)
inline size_t hinv_bytes(int nb) { return (sizeof(double2) + sizeof(float2)) * (size_t)(nb + 1); }
int launch_estimate(int precision, const int *cand, const RunCtl *ctl, int cap, int expect,
                    const void *bins, int loops, int n, int B, const Draws &d,
                    const double2 *hinv, DevNode *nodes, double *mag2, cudaStream_t st);

// 64-point complex DFTs of nvec float2 vectors on the tensor cores (tcgen05,
// three-part bf16 split, fp32 accumulation); err: set when a wait timed out
int launch_tc_dft64(const void *x, void *y, int nvec, int *err, cudaStream_t st);

// gather selected nodes (A9 output)
int launch_gather_nodes(const DevNode *nodes, const int *idx, const int *count, int cap,
                        DevNode *out, cudaStream_t st);

}  // namespace gsfft
