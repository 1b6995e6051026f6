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
//    write pass with per-block prefix sums.
#include "stages.cuh"

namespace gsfft {

namespace {

constexpr int VT = 256;  // threads per block in this file

__device__ __forceinline__ unsigned blk_excl_scan(unsigned v, unsigned *ws, unsigned *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned w = lane < VT / 32 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < VT / 32) ws[lane] = w;
  }
  __syncthreads();
  unsigned base = wid ? ws[wid - 1] : 0;
  unsigned tot = ws[VT / 32 - 1];
  __syncthreads();
  if (total) *total = tot;
  return base + x - v;
}

__device__ __forceinline__ unsigned blk_sum(unsigned v, unsigned *ws) {
  unsigned t;
  blk_excl_scan(v, ws, &t);
  return t;
}

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

// ------------------------------------------------------------ voting
struct WalkArgs {
  const int *J;
  int Bt, n, nb, W;
  const unsigned *bm;
  const int *fmax;
  unsigned a;
};

// low = ceil((J - 0.5) * n/B) reduced mod n (innerLoop.cu:792), in integers.
__device__ __forceinline__ int window_low(int J, int n, int nb) {
  const long long v = (2LL * J - 1) * nb;  // 2 * (J - 0.5) * nb
  const long long c = v >= 0 ? (v + 1) / 2 : -((-v) / 2);
  return (int)((c + n) & (long long)(n - 1));
}

template <class F>
__device__ __forceinline__ void walk_window(const WalkArgs &w, int J, F &&visit) {
  const int low = window_low(J, w.n, w.nb);
  const int key = low & (w.W - 1);
  if (key > *w.fmax) return;  // reference clamp: nothing visited
  const int base = low - key;
  int pos = 0;
  while (pos < w.nb) {
    const int r = key + pos;
    int rr = r, blk = base;
    if (r >= w.W) { rr = r - w.W; blk = (base + w.W) & (w.n - 1); }
    const int bit = rr & 31;
    const int take = min(32 - bit, w.nb - pos);
    unsigned word = __ldg(&w.bm[rr >> 5]) >> bit;
    if (take < 32) word &= (1u << take) - 1u;
    while (word) {
      const int t = __ffs(word) - 1;
      word &= word - 1;
      visit(blk + rr + t);
    }
    pos += take;
  }
}

__global__ void __launch_bounds__(VT)
vote_count_kernel(WalkArgs w, unsigned epoch, unsigned thresh, unsigned *vote, int *cnt, int *blk) {
  __shared__ unsigned ws[VT / 32];
  const int t = blockIdx.x * VT + threadIdx.x;
  unsigned c = 0;
  if (t < w.Bt) {
    const unsigned nmask = (unsigned)w.n - 1u;
    walk_window(w, w.J[t], [&](int p) {
      const unsigned loc = ((unsigned)p * w.a) & nmask;
      const unsigned e = vote[loc];
      const unsigned cv = ((e >> 8) == epoch) ? (e & 255u) + 1u : 1u;
      vote[loc] = (epoch << 8) | cv;
      c += (cv == thresh);
    });
    cnt[t] = (int)c;
  }
  const unsigned s = blk_sum(c, ws);
  if (threadIdx.x == 0) blk[blockIdx.x] = (int)s;
}

__global__ void __launch_bounds__(VT)
vote_write_kernel(WalkArgs w, unsigned epoch, unsigned thresh, const unsigned *__restrict__ vote,
                  const int *__restrict__ cnt, const int *__restrict__ blk, int *cand, int cap,
                  RunCtl *ctl) {
  __shared__ unsigned ws[VT / 32];
  __shared__ int is_last;
  const int base_prev = ctl->cand_count;
  unsigned before = 0;
  for (int b = threadIdx.x; b < (int)blockIdx.x; b += VT) before += (unsigned)blk[b];
  before = blk_sum(before, ws);
  const int t = blockIdx.x * VT + threadIdx.x;
  const unsigned c = t < w.Bt ? (unsigned)cnt[t] : 0u;
  unsigned tot;
  long long pos = (long long)base_prev + before + blk_excl_scan(c, ws, &tot);
  if (c) {
    const unsigned nmask = (unsigned)w.n - 1u;
    const unsigned want = (epoch << 8) | thresh;
    walk_window(w, w.J[t], [&](int p) {
      const unsigned loc = ((unsigned)p * w.a) & nmask;
      if (vote[loc] == want) {
        if (pos < cap) cand[pos] = (int)loc;
        pos++;
      }
    });
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned tk = atomicAdd(&ctl->ticket, 1u);
    is_last = tk == gridDim.x - 1;
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    long long total = 0;
    for (int b = 0; b < (int)gridDim.x; b++) total += blk[b];
    const long long nc = (long long)base_prev + total;
    ctl->cand_count = (int)(nc > 0x7fffffffLL ? 0x7fffffffLL : nc);
    if (nc > cap) ctl->overflow = 1;
    ctl->ticket = 0;
  }
}

}  // namespace

int j2_merge_launches() { return 3; }

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

int vote_launches_per_loop() { return 2; }

int launch_vote_loop(int l, const int *J, int B_thresh, int n, int B, int W,
                     const unsigned *bitmap_l, const Draws &d, int loops_thresh, unsigned epoch,
                     unsigned *vote, int *cand, int cap, int *cnt, int *blk, RunCtl *ctl,
                     cudaStream_t st) {
  WalkArgs w;
  w.J = J;
  w.Bt = B_thresh;
  w.n = n;
  w.nb = n / B;
  w.W = W;
  w.bm = bitmap_l;
  w.fmax = &ctl->fmax[l];
  w.a = (unsigned)d.a[l];
  const int grid = (B_thresh + VT - 1) / VT;
  vote_count_kernel<<<grid, VT, 0, st>>>(w, epoch, (unsigned)loops_thresh, vote, cnt, blk);
  GS_LAUNCHED();
  vote_write_kernel<<<grid, VT, 0, st>>>(w, epoch, (unsigned)loops_thresh, vote, cnt, blk, cand, cap,
                                         ctl);
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
