// A4 tail (J2 merge) and A7 (reverse hash + voting).
//
// Reference: outerLoop.cu:111-121 (host radix sort + de-duplication of the RLFC
// blocks in managed memory); reverse_hash (innerLoop.cu:300-384) builds
// Pair{f = J2*ai mod W, f*a mod n} on the host, qsorts it by f and launches
// reverseHashKernel (:783-817): per heavy bucket J, a binary search
// (findUpperBound, :901-920) and a walk over the sorted f list, voting into a
// dense n-entry table that outer_loop zeroes every call (:89-93).
//
// GB300 formulation (same visited set, no host round trip, no sort):
//  * J2 = the set bits of a W-bit bitmap, compacted in ascending order.
//  * F_l = {J2[m] * ai_l mod W} is another W-bit bitmap per location loop,
//    with fmax_l = max F_l.
//  * Bucket J's window is [low, low + n/B) (mod n), low = ceil((J-0.5) n/B).
//    The positions p in the window whose residue p mod W is in F_l are visited
//    in ascending circular order -- unless key = low mod W exceeds fmax_l, in
//    which case the reference's search clamps to the last f, whose position
//    lies below the window, and the walk stops at once: nothing is visited
//    (findUpperBound's clamp, :906-908).  With n/B < W < n this is exactly the
//    reference's walk.
//  * loc = p * a mod n (the inverse permutation); the vote table is epoch
//    tagged (entry = epoch << 8 | count) so it is never re-zeroed between runs.
//    Each loc is visited at most once per location loop (windows of distinct
//    buckets are disjoint, a window is shorter than W, and p -> p*a is a
//    bijection), so the update is a plain read-modify-write without races.
//  * Candidates (count reaching loops_thresh) are appended in canonical order
//    (location loop, bucket index, window position) by a count pass and a
//    write pass with per-block prefix sums.  The count pass records each
//    bucket's first STASH candidates in window order, so the write pass
//    copies them instead of walking the window and the vote table again
//    (buckets with more candidates are walked again).
#include "vote_dev.cuh"

namespace gsfft {

namespace {

// ------------------------------------------------------------ J2 merge
constexpr int WORDS_PER_THREAD = 8;
constexpr int WORDS_PER_TILE = VT * WORDS_PER_THREAD;

__global__ void j2_set_bits_kernel(const int *__restrict__ J2b, int total, int W, unsigned *bm) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i < total) {
    const int f = J2b[i];
    if (f >= 0 && f < W) atomicOr(&bm[f >> 5], 1u << (f & 31));
  }
}

__global__ void bm_count_kernel(const unsigned *__restrict__ bm, int nwords, unsigned *tile_cnt) {
  __shared__ unsigned ws[VT / 32];
  unsigned c = 0;
  const int w0 = blockIdx.x * WORDS_PER_TILE + threadIdx.x * WORDS_PER_THREAD;
#pragma unroll
  for (int q = 0; q < WORDS_PER_THREAD; q++)
    if (w0 + q < nwords) c += __popc(bm[w0 + q]);
  const unsigned t = blk_sum(c, ws);
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = t;
}

__global__ void bm_write_kernel(const unsigned *__restrict__ bm, int nwords,
                                const unsigned *__restrict__ tile_cnt, int *out, int *count) {
  __shared__ unsigned ws[VT / 32];
  unsigned before = 0;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += VT) before += tile_cnt[t];
  before = blk_sum(before, ws);
  unsigned words[WORDS_PER_THREAD];
  unsigned c = 0;
  const int w0 = blockIdx.x * WORDS_PER_TILE + threadIdx.x * WORDS_PER_THREAD;
#pragma unroll
  for (int q = 0; q < WORDS_PER_THREAD; q++) {
    words[q] = (w0 + q < nwords) ? bm[w0 + q] : 0u;
    c += __popc(words[q]);
  }
  unsigned tot;
  unsigned pos = before + blk_excl_scan(c, ws, &tot);
#pragma unroll
  for (int q = 0; q < WORDS_PER_THREAD; q++) {
    unsigned w = words[q];
    while (w) {
      const int b = __ffs(w) - 1;
      w &= w - 1;
      out[pos++] = (w0 + q) * 32 + b;
    }
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *count = (int)(before + tot);
}

// ------------------------------------------------------------ sigma bitmaps
__global__ void sigma_bits_kernel(const int *__restrict__ J2, const int *num_dev, int W,
                                  Draws d, unsigned *bms, int words_per_map, int *fmax) {
  const int m = blockIdx.x * VT + threadIdx.x;
  const int l = blockIdx.y;
  if (m >= *num_dev) return;
  const unsigned f = ((unsigned)J2[m] * (unsigned)d.ai[l]) & (unsigned)(W - 1);
  atomicOr(&bms[(size_t)l * words_per_map + (f >> 5)], 1u << (f & 31));
  atomicMax(&fmax[l], (int)f);
}

// Same bitmaps straight from the RLFC blocks (duplicates set the same bit
// twice), with the per-loop maximum reduced over the block before one atomic
// (one per warp queued thousands of atomics on the same word).
__global__ void sigma_from_blocks_kernel(const int *__restrict__ J2b, int total, int W, Draws d,
                                         int loops_loc, unsigned *bms, int words_per_map,
                                         int *fmax) {
  pdl_enter();
  __shared__ int wmax[MAX_LOOPS][VT / 32];
  const int m = blockIdx.x * VT + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool ok = m < total;
  const unsigned v = ok ? (unsigned)J2b[m] : 0u;
  for (int l = 0; l < loops_loc; l++) {
    const unsigned f = (v * (unsigned)d.ai[l]) & (unsigned)(W - 1);
    if (ok) atomicOr(&bms[(size_t)l * words_per_map + (f >> 5)], 1u << (f & 31));
    int mx = ok ? (int)f : -1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) wmax[l][warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x < loops_loc) {
    int mx = -1;
    for (int wv = 0; wv < VT / 32; wv++) mx = max(mx, wmax[threadIdx.x][wv]);
    if (mx >= 0) atomicMax(&fmax[threadIdx.x], mx);
  }
}

__global__ void __launch_bounds__(VT)
vote_count_kernel(WalkArgs w, const unsigned *epoch_p, unsigned thresh, unsigned *vote, int *cnt,
                  int *blk, int *blk_pre, int *stash, RunCtl *ctl) {
  pdl_enter();
  vote_count_block(w, *epoch_p, thresh, vote, cnt, blk, blk_pre, stash, ctl, (int)blockIdx.x,
                   (int)gridDim.x);
}

__global__ void __launch_bounds__(VT)
vote_mark_kernel(WalkArgs w, const unsigned *epoch_p, unsigned *vote) {
  pdl_enter();
  vote_mark_block(w, *epoch_p, vote, (int)blockIdx.x);
}

__global__ void __launch_bounds__(VT)
vote_write_kernel(WalkArgs w, const unsigned *epoch_p, unsigned thresh, const unsigned *__restrict__ vote,
                  const int *__restrict__ cnt, const int *__restrict__ blk_pre, int nblk,
                  const int *__restrict__ stash, int *cand, int cap, RunCtl *ctl) {
  pdl_enter();
  vote_write_block(w, *epoch_p, thresh, vote, cnt, blk_pre, stash, cand, cap, ctl, (int)blockIdx.x,
                   nblk);
}

}  // namespace

int launch_j2_merge(const int *J2_blocks, int total, int W, unsigned *bitmap, int *J2, RunCtl *ctl,
                    unsigned *tile_tmp, cudaStream_t st) {
  const int nwords = W / 32;
  GS_CUDA(cudaMemsetAsync(bitmap, 0, sizeof(unsigned) * nwords, st));
  j2_set_bits_kernel<<<(total + VT - 1) / VT, VT, 0, st>>>(J2_blocks, total, W, bitmap);
  GS_LAUNCHED();
  const int tiles = (nwords + WORDS_PER_TILE - 1) / WORDS_PER_TILE;
  bm_count_kernel<<<tiles, VT, 0, st>>>(bitmap, nwords, tile_tmp);
  GS_LAUNCHED();
  bm_write_kernel<<<tiles, VT, 0, st>>>(bitmap, nwords, tile_tmp, J2, &ctl->num_rlfc);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_sigma_bitmaps(const int *J2, const RunCtl *ctl_num, int max_num, int W, int loops_loc,
                         const Draws &d, unsigned *bitmaps, RunCtl *ctl, cudaStream_t st) {
  const int words = W / 32;
  GS_CUDA(cudaMemsetAsync(bitmaps, 0, sizeof(unsigned) * (size_t)words * loops_loc, st));
  GS_CUDA(cudaMemsetAsync(ctl->fmax, 0xff, sizeof(int) * MAX_LOOPS, st));
  dim3 grid((max_num + VT - 1) / VT, loops_loc);
  sigma_bits_kernel<<<grid, VT, 0, st>>>(J2, &ctl_num->num_rlfc, W, d, bitmaps, words, ctl->fmax);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_sigma_from_blocks(const int *J2b, int total, int W, int loops_loc, const Draws &d,
                             unsigned *bitmaps, RunCtl *ctl, cudaStream_t st) {
  const int words = W / 32;
  // the bitmaps are zero on entry and ctl->fmax starts at 0 (the run's first
  // kernel clears both); every F_l is non-empty
  GS_CUDA(launch_pdl(sigma_from_blocks_kernel, dim3((total + VT - 1) / VT), dim3(VT), 0, st, J2b,
                     total, W, d, loops_loc, bitmaps, words, (int *)ctl->fmax));
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_vote_loop(int l, const int *J, int B_thresh, int n, int B, int W,
                     const unsigned *bitmap_l, const Draws &d, int loops_thresh, const unsigned *epoch,
                     unsigned *vote, int *cand, int cap, int *cnt, int *blk, RunCtl *ctl,
                     bool may_complete, cudaStream_t st, bool packed) {
  WalkArgs w;
  w.J = J;
  w.Bt = B_thresh;
  w.n = n;
  w.nb = n / B;
  w.W = W;
  w.bm = bitmap_l;
  w.fmax = &ctl->fmax[l];
  w.a = (unsigned)d.a[l];
  w.packed = packed ? 1 : 0;
  const int grid = (B_thresh + WPB - 1) / WPB;
  if (!may_complete) {
    GS_CUDA(launch_pdl(vote_mark_kernel, dim3(grid), dim3(VT), 0, st, w, epoch, vote));
    GS_LAUNCHED();
    return GSFFT_OK;
  }
  // blk: 2 * (grid + 1) ints of block counts and prefixes, then STASH
  // candidate slots per heavy bucket
  int *blk_pre = blk + grid + 1;
  int *stash = blk + 2 * (grid + 1);
  GS_CUDA(launch_pdl(vote_count_kernel, dim3(grid), dim3(VT), 0, st, w, epoch, (unsigned)loops_thresh,
                     vote, cnt, blk, blk_pre, stash, ctl));
  GS_LAUNCHED();
  GS_CUDA(launch_pdl(vote_write_kernel, dim3(grid), dim3(VT), 0, st, w, epoch, (unsigned)loops_thresh,
                     (const unsigned *)vote, (const int *)cnt, (const int *)blk_pre, grid,
                     (const int *)stash, cand, cap, ctl));
  GS_LAUNCHED();
  return GSFFT_OK;
}

int vote_block_ints(int B_thresh) {
  return 2 * ((B_thresh + WPB - 1) / WPB + 1) + B_thresh * STASH;
}

}  // namespace gsfft
