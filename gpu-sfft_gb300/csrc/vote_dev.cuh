// Device code of the voting stage (A7): the block bodies of the mark, count
// and write passes, with the block index and block count as arguments, so
// that the per-plan kernels (vote.cu) and the persistent kernel that runs the
// tails of a whole batch (batch_tail.cu) run the same code.  Loads of data
// that another block of the same launch may have written (the vote table, the
// block counts and scans, the stashed candidates, the candidate count) bypass
// L1 (ld.global.cg), so the persistent kernel sees what its earlier work items
// wrote.
#pragma once
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

// ------------------------------------------------------------ voting
struct WalkArgs {
  const int *J;
  int Bt, n, nb, W;
  const unsigned *bm;
  const int *fmax;
  unsigned a;
  int packed;  // vote tables of 2-bit counters (16 per word; two tables used on alternate
               // runs) instead of epoch-tagged 32-bit entries
};

// The vote table.  Epoch-tagged: entry = epoch << 8 | count, never cleared
// between runs, read and written plainly (a location is visited at most once
// per pass).  Packed (at most 3 location loops, so counts fit 2 bits): 16
// counters per word, n / 4 bytes -- small enough to stay in L2 -- updated
// with word atomics, since neighbouring locations share a word.  There are
// two packed tables, the run with epoch e using table e & 1; after a run's
// voting the other one is cleared for the next run (vote_clear_kernel), so
// the clear overlaps the run's latency-bound tail.
__device__ __forceinline__ unsigned *packed_table(const WalkArgs &w, unsigned *vote, unsigned epoch) {
  return vote + ((epoch & 1u) ? ((unsigned)w.n >> 4) : 0u);
}
// vote_update: the votes of up to four visited locations, independent so
// that their table accesses overlap; cnt[q] = the count after the vote.
__device__ __forceinline__ void vote_update(const WalkArgs &w, unsigned epoch, unsigned *vote,
                                            const unsigned (&loc)[4], int nq, unsigned (&cnt)[4]) {
  if (w.packed) {
    unsigned *tab = packed_table(w, vote, epoch);
    unsigned old[4];
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (q < nq) old[q] = atomicAdd(&tab[loc[q] >> 4], 1u << (2 * (loc[q] & 15u)));
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (q < nq) cnt[q] = ((old[q] >> (2 * (loc[q] & 15u))) & 3u) + 1u;
    return;
  }
  unsigned e[4];
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (q < nq) e[q] = __ldcg(&vote[loc[q]]);
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (q < nq) {
      const unsigned cv = ((e[q] >> 8) == epoch) ? (e[q] & 255u) + 1u : 1u;
      vote[loc[q]] = (epoch << 8) | cv;
      cnt[q] = cv;
    }
}
// whether location loc's count is exactly the threshold (after a pass's votes)
__device__ __forceinline__ bool vote_at_threshold(const WalkArgs &w, unsigned epoch, const unsigned *vote,
                                                  unsigned loc, unsigned thresh) {
  if (w.packed) {
    const unsigned *tab = vote + ((epoch & 1u) ? ((unsigned)w.n >> 4) : 0u);
    return ((__ldcg(&tab[loc >> 4]) >> (2 * (loc & 15u))) & 3u) == thresh;
  }
  return __ldcg(&vote[loc]) == ((epoch << 8) | thresh);
}

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

// Votes of heavy bucket t (one warp): returns this lane's number of visited
// positions whose count reached the threshold, and records the bucket's
// first STASH of them, in window order, at slot[] (global or shared memory).
__device__ __forceinline__ unsigned count_walk(const WalkArgs &w, int t, unsigned epoch, unsigned thresh,
                                               unsigned *vote, int *slot) {
  const unsigned nmask = (unsigned)w.n - 1u;
  unsigned c = 0;
  unsigned recorded = 0;  // this bucket's candidates so far (warp-uniform)
  for_each_chunk(w, w.J[t], [&](unsigned mask, const ChunkPos &pos) {
    // up to four visited positions at a time: their table reads are
    // independent, so they overlap instead of paying one DRAM latency each
    unsigned app = 0;  // bits of this lane's mask whose count reached the threshold
    while (mask) {
      unsigned loc[4];
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
      unsigned cv[4];
      vote_update(w, epoch, vote, loc, nq, cv);
      unsigned hitq = 0;  // bit q: position q of this round reached the threshold
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (q < nq) hitq |= (unsigned)(cv[q] == thresh) << q;
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
  return c;
}

// Appends heavy bucket t's cw candidates (warp-uniform) at cand[next ..]:
// copied from slot[] when the count walk recorded them all (GLOBAL_SLOT: the
// slots were written by another launch or block, so the loads bypass L1),
// else found again by walking the window and the vote table.
template <bool GLOBAL_SLOT>
__device__ __forceinline__ void write_bucket(const WalkArgs &w, int t, unsigned epoch, unsigned thresh,
                                             const unsigned *vote, unsigned cw, const int *slot,
                                             int *cand, int cap, long long next) {
  const int lane = threadIdx.x & 31;
  if (cw <= (unsigned)STASH) {
    for (unsigned j = lane; j < cw; j += 32) {
      const long long o = next + j;
      if (o < cap) cand[o] = GLOBAL_SLOT ? __ldcg(&slot[j]) : slot[j];
    }
    return;
  }
  const unsigned nmask = (unsigned)w.n - 1u;
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
        if (q < nq && vote_at_threshold(w, epoch, vote, loc[q], thresh)) app |= 1u << bit[q];
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

// One block of the count pass (block bid of nblk): votes of the location
// loop, each bucket's candidate count and first STASH candidates; the last
// block to finish writes the exclusive scan of the block counts.
__device__ __forceinline__ void vote_count_block(const WalkArgs &w, unsigned epoch, unsigned thresh,
                                                 unsigned *vote, int *cnt, int *blk, int *blk_pre,
                                                 int *stash, RunCtl *ctl, int bid, int nblk) {
  __shared__ unsigned ws[VT / 32];
  __shared__ int is_last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = bid * WPB + warp;
  unsigned c = 0;
  if (t < w.Bt) c = count_walk(w, t, epoch, thresh, vote, stash + (size_t)t * STASH);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0 && t < w.Bt) cnt[t] = (int)c;
  const unsigned s = blk_sum(lane == 0 ? c : 0u, ws);
  // last block: exclusive scan of the block counts.  Only the block count has
  // to be visible to it, so only thread 0 fences (a fence in every thread
  // would wait for that thread's vote-table writes to reach memory).
  if (threadIdx.x == 0) {
    blk[bid] = (int)s;
    __threadfence();
    const unsigned tk = atomicAdd(&ctl->ticket, 1u);
    is_last = tk == (unsigned)nblk - 1u;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // Each thread scans a contiguous run of block counts: all its L2 loads are
  // independent, then one block scan (the serial tail used to pay an L2 round
  // trip and three barriers per 256 counts).
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
// One block of a location loop that cannot complete a count: votes only.
__device__ __forceinline__ void vote_mark_block(const WalkArgs &w, unsigned epoch, unsigned *vote,
                                                int bid) {
  const int warp = threadIdx.x >> 5;
  const int t = bid * WPB + warp;
  if (t >= w.Bt) return;
  const unsigned nmask = (unsigned)w.n - 1u;
  for_each_chunk(w, w.J[t], [&](unsigned mask, const ChunkPos &pos) {
    while (mask) {
      unsigned loc[4], cv[4];
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
      vote_update(w, epoch, vote, loc, nq, cv);
    }
  });
}

// One block of the write pass: appends the block's candidates at their
// canonical offsets; the last block to finish publishes the new count.
__device__ __forceinline__ void vote_write_block(const WalkArgs &w, unsigned epoch, unsigned thresh,
                                                 const unsigned *vote, const int *cnt,
                                                 const int *blk_pre, const int *stash, int *cand,
                                                 int cap, RunCtl *ctl, int bid, int nblk) {
  __shared__ unsigned ws[VT / 32];
  __shared__ int is_last;
  const int base_prev = __ldcg(&ctl->cand_count);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = bid * WPB + warp;
  const unsigned c = (t < w.Bt && lane == 0) ? (unsigned)__ldcg(&cnt[t]) : 0u;
  unsigned tot;
  const unsigned wpre = blk_excl_scan(c, ws, &tot);  // lane 0 of each warp carries its count
  long long next = (long long)base_prev + __ldcg(&blk_pre[bid]) + __shfl_sync(0xffffffffu, wpre, 0);
  const unsigned cw = __shfl_sync(0xffffffffu, c, 0);
  if (cw) write_bucket<true>(w, t, epoch, thresh, vote, cw, stash + (size_t)t * STASH, cand, cap, next);
  // the last block to finish publishes the new candidate count; every block
  // read the old one before its thread 0 takes a ticket (barrier + fence)
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned tk = atomicAdd(&ctl->ticket, 1u);
    is_last = tk == (unsigned)nblk - 1u;
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    const long long nc = (long long)base_prev + __ldcg(&blk_pre[nblk]);
    ctl->cand_count = (int)(nc > 0x7fffffffLL ? 0x7fffffffLL : nc);
    if (nc > cap) ctl->overflow = 1;
    ctl->ticket = 0;
  }
}


}  // namespace

}  // namespace gsfft
