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

// One warp per heavy bucket.  The window [low, low + n/B) is cut into chunks;
// in chunk c lane L holds a 32-bit mask of visited positions (window offsets
// 1024c + 32L .. +31 when the window is 32-aligned, else the single offset
// 32c + L).  Chunks, lanes and bits in ascending order give the window in
// ascending order.  chunk_fn(mask, pos_of_bit) is called once per chunk by
// every lane (warp-uniform trip count).
struct ChunkPos {
  int r0, base, key, W, n, aligned;
  // position of bit t of this lane's mask
  __device__ __forceinline__ int operator()(int t) const {
    const int rr = aligned ? r0 + t : r0;
    const int blk = (rr >= key) ? base : ((base + W) & (n - 1));
    return blk + rr;
  }
};

template <class F>
__device__ __forceinline__ void for_each_chunk(const WalkArgs &w, int J, F &&chunk_fn) {
  const int lane = threadIdx.x & 31;
  const int low = window_low(J, w.n, w.nb);
  const int key = low & (w.W - 1);
  if (key > *w.fmax) return;  // reference clamp: nothing visited
  const int base = low - key;
  const int aligned = ((key & 31) == 0 && (w.nb & 31) == 0) ? 1 : 0;
  const int span = aligned ? 1024 : 32;
  for (int c0 = 0; c0 < w.nb; c0 += span) {
    unsigned mask = 0;
    int r0 = 0;
    if (aligned) {
      const int off = c0 + lane * 32;
      if (off < w.nb) {
        r0 = key + off;
        if (r0 >= w.W) r0 -= w.W;  // aligned words never straddle W
        mask = __ldg(&w.bm[r0 >> 5]);
      }
    } else {
      const int off = c0 + lane;
      if (off < w.nb) {
        int r = key + off;
        if (r >= w.W) r -= w.W;
        r0 = r;
        mask = (__ldg(&w.bm[r >> 5]) >> (r & 31)) & 1u;
      }
    }
    ChunkPos pos{r0, base, key, w.W, w.n, aligned};
    chunk_fn(mask, pos);
  }
}

__device__ __forceinline__ unsigned warp_excl_scan(unsigned v, unsigned *total) {
  const int lane = threadIdx.x & 31;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

constexpr int WPB = VT / 32;  // buckets (warps) per block
constexpr int STASH = 32;     // candidates recorded per heavy bucket by the count pass

__global__ void __launch_bounds__(VT)
vote_count_kernel(WalkArgs w, const unsigned *epoch_p, unsigned thresh, unsigned *vote, int *cnt,
                  int *blk, int *blk_pre, int *stash, RunCtl *ctl) {
  pdl_enter();
  const unsigned epoch = *epoch_p;
  __shared__ unsigned ws[VT / 32];
  __shared__ int is_last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * WPB + warp;
  unsigned c = 0;
  if (t < w.Bt) {
    const unsigned nmask = (unsigned)w.n - 1u;
    int *const slot = stash + (size_t)t * STASH;
    unsigned recorded = 0;  // this bucket's candidates so far (warp-uniform)
    for_each_chunk(w, w.J[t], [&](unsigned mask, const ChunkPos &pos) {
      // up to four visited positions at a time: their table reads are
      // independent, so they overlap instead of paying one DRAM latency each
      unsigned app = 0;  // bits of this lane's mask whose count reached the threshold
      while (mask) {
        unsigned loc[4], e[4];
        int nq = 0;
        const unsigned before = mask;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (mask) {
            const int bq = __ffs(mask) - 1;
            mask &= mask - 1;
            loc[q] = ((unsigned)pos(bq) * w.a) & nmask;
            nq = q + 1;
          }
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (q < nq) e[q] = vote[loc[q]];
        unsigned hitq = 0;  // bit q: position q of this round reached the threshold
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (q < nq) {
            const unsigned cv = ((e[q] >> 8) == epoch) ? (e[q] & 255u) + 1u : 1u;
            vote[loc[q]] = (epoch << 8) | cv;
            hitq |= (unsigned)(cv == thresh) << q;
          }
        }
        // the round's positions are the lowest set bits of `before`, in order
        unsigned taken = before & ~mask;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const unsigned low = taken & (0u - taken);
          taken ^= low;
          if ((hitq >> q) & 1u) app |= low;
        }
      }
      c += (unsigned)__popc(app);
      // window order: chunks, then lanes, then bits (as the write pass walks)
      if (__any_sync(0xffffffffu, app != 0u)) {
        unsigned ctot;
        unsigned o = recorded + warp_excl_scan((unsigned)__popc(app), &ctot);
        while (app) {
          const int b = __ffs(app) - 1;
          app &= app - 1;
          if (o < (unsigned)STASH) slot[o] = (int)(((unsigned)pos(b) * w.a) & nmask);
          o++;
        }
        recorded += ctot;
      }
    });
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0 && t < w.Bt) cnt[t] = (int)c;
  const unsigned s = blk_sum(lane == 0 ? c : 0u, ws);
  // last block: exclusive scan of the block counts.  Only the block count has
  // to be visible to it, so only thread 0 fences (a fence in every thread
  // would wait for that thread's vote-table writes to reach memory).
  if (threadIdx.x == 0) {
    blk[blockIdx.x] = (int)s;
    __threadfence();
    const unsigned tk = atomicAdd(&ctl->ticket, 1u);
    is_last = tk == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // Each thread scans a contiguous run of block counts: all its L2 loads are
  // independent, then one block scan (the serial tail used to pay an L2 round
  // trip and three barriers per 256 counts).
  const int nblk = (int)gridDim.x;
  const int per = (nblk + VT - 1) / VT;
  const int i0 = min(nblk, (int)threadIdx.x * per), i1 = min(nblk, i0 + per);
  unsigned sum = 0;
  for (int i = i0; i < i1; i++) sum += (unsigned)__ldcg(&blk[i]);
  unsigned tot;
  unsigned run = blk_excl_scan(sum, ws, &tot);
  for (int i = i0; i < i1; i++) {
    blk_pre[i] = (int)run;
    run += (unsigned)__ldcg(&blk[i]);
  }
  if (threadIdx.x == 0) {
    blk_pre[nblk] = (int)tot;
    ctl->ticket = 0;
  }
}

// Location loops before the (loops_thresh-1)-th cannot bring any count to
// the threshold: they only record their votes.
__global__ void __launch_bounds__(VT)
vote_mark_kernel(WalkArgs w, const unsigned *epoch_p, unsigned *vote) {
  pdl_enter();
  const unsigned epoch = *epoch_p;
  const int warp = threadIdx.x >> 5;
  const int t = blockIdx.x * WPB + warp;
  if (t >= w.Bt) return;
  const unsigned nmask = (unsigned)w.n - 1u;
  for_each_chunk(w, w.J[t], [&](unsigned mask, const ChunkPos &pos) {
    while (mask) {
      unsigned loc[4], e[4];
      int nq = 0;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (mask) {
          const int b = __ffs(mask) - 1;
          mask &= mask - 1;
          loc[q] = ((unsigned)pos(b) * w.a) & nmask;
          nq = q + 1;
        }
      }
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (q < nq) e[q] = vote[loc[q]];
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (q < nq) {
          const unsigned cv = ((e[q] >> 8) == epoch) ? (e[q] & 255u) + 1u : 1u;
          vote[loc[q]] = (epoch << 8) | cv;
        }
    }
  });
}

__global__ void __launch_bounds__(VT)
vote_write_kernel(WalkArgs w, const unsigned *epoch_p, unsigned thresh, const unsigned *__restrict__ vote,
                  const int *__restrict__ cnt, const int *__restrict__ blk_pre, int nblk,
                  const int *__restrict__ stash, int *cand, int cap, RunCtl *ctl) {
  pdl_enter();
  __shared__ unsigned ws[VT / 32];
  __shared__ int is_last;
  const int base_prev = ctl->cand_count;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * WPB + warp;
  const unsigned c = (t < w.Bt && lane == 0) ? (unsigned)cnt[t] : 0u;
  unsigned tot;
  const unsigned wpre = blk_excl_scan(c, ws, &tot);  // lane 0 of each warp carries its count
  long long next = (long long)base_prev + blk_pre[blockIdx.x] + __shfl_sync(0xffffffffu, wpre, 0);
  const unsigned cw = __shfl_sync(0xffffffffu, c, 0);
  if (cw && cw <= (unsigned)STASH) {
    // recorded by the count pass in window order
    const int *slot = stash + (size_t)t * STASH;
    for (unsigned j = lane; j < cw; j += 32) {
      const long long o = next + j;
      if (o < cap) cand[o] = slot[j];
    }
  } else if (cw) {
    const unsigned nmask = (unsigned)w.n - 1u;
    const unsigned want = (*epoch_p << 8) | thresh;
    for_each_chunk(w, w.J[t], [&](unsigned mask, const ChunkPos &pos) {
      // appended positions of this lane, in bit order
      unsigned app = 0;
      unsigned m = mask;
      while (m) {
        unsigned loc[4], bit[4];
        int nq = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (m) {
            bit[q] = __ffs(m) - 1;
            m &= m - 1;
            loc[q] = ((unsigned)pos((int)bit[q]) * w.a) & nmask;
            nq = q + 1;
          }
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (q < nq && vote[loc[q]] == want) app |= 1u << bit[q];
      }
      unsigned ctot;
      long long o = next + warp_excl_scan((unsigned)__popc(app), &ctot);
      while (app) {
        const int b = __ffs(app) - 1;
        app &= app - 1;
        if (o < cap) cand[o] = (int)(((unsigned)pos(b) * w.a) & nmask);
        o++;
      }
      next += ctot;
    });
  }
  // the last block to finish publishes the new candidate count; every block
  // read the old one before its thread 0 takes a ticket (barrier + fence)
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned tk = atomicAdd(&ctl->ticket, 1u);
    is_last = tk == gridDim.x - 1;
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    const long long nc = (long long)base_prev + blk_pre[nblk];
    ctl->cand_count = (int)(nc > 0x7fffffffLL ? 0x7fffffffLL : nc);
    if (nc > cap) ctl->overflow = 1;
    ctl->ticket = 0;
  }
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
                     bool may_complete, cudaStream_t st) {
  WalkArgs w;
  w.J = J;
  w.Bt = B_thresh;
  w.n = n;
  w.nb = n / B;
  w.W = W;
  w.bm = bitmap_l;
  w.fmax = &ctl->fmax[l];
  w.a = (unsigned)d.a[l];
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
