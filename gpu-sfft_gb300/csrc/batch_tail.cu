// Persistent multi-signal voting of a batch: the reverse hash and voting (A7)
// of every plan of a batch in one cooperative launch.
//
// In a batch of small signals each plan's voting is a chain of short kernels
// (a mark pass per location loop that cannot complete a count, a count and a
// write pass per loop that can), each waiting for the launch and completion
// of the one before.  Here the batch runs every plan's front (run state,
// perm+filter, FFTs, cutoffs, residue bitmaps) on its streams, joins them,
// runs one persistent kernel that takes the voting blocks of all plans as work
// items from a device queue, and then every plan's estimation and top-k:
//   * a plan's stages are, in order, mark(l) for the location loops that
//     cannot complete a count, then count(l) and write(l) for the others; a
//     work item is a run of consecutive blocks of one stage (the per-plan
//     kernel's blocks, run one after another by the item's block);
//   * items are numbered stage-major over all plans (every plan's first
//     stage, then every plan's second stage, ...) and taken in that order
//     with one atomic ticket, so an item only ever waits for items with
//     smaller tickets -- items that running blocks have already taken and
//     that wait for nothing later: no cycle, whatever the residency;
//   * before an item of stage s, one thread waits until every block of stage
//     s - 1 of the same plan has finished (a per-plan, per-stage done
//     counter, read with ld.acquire.gpu); the wait is bounded -- after the
//     limit it flags the plan's run as failed (GSFFT_ERR_TIMEOUT) and the item
//     goes on, so the launch always ends;
//   * each block runs the same block body as the per-plan kernels
//     (vote_dev.cuh), then fences and counts itself done.
// The launch is cooperative: its blocks wait on one another's work.
#include "engine.cuh"
#include "vote_dev.cuh"

#include <vector>

namespace gsfft {

namespace {

constexpr int MAX_STAGES = 2 * MAX_LOOPS;
constexpr long long kTailWaitLimit = 1LL << 31;  // SM cycles, about one second

enum { ST_MARK = 0, ST_COUNT = 1, ST_WRITE = 2 };
constexpr int kBlocksPerItem = 4;  // consecutive blocks of a stage per work item

// One plan's voting as the kernel sees it (device memory, fixed for a batch).
struct TailPlan {
  const int *J;            // loops_loc x B_thresh bucket ids
  const unsigned *bm_sig;  // loops_loc residue bitmaps of W/32 words
  int Bt, n, nb, W, loops_loc, loops_thresh;
  const unsigned *epoch;
  unsigned *vote;
  int *cnt, *blk, *cand;
  int cap;
  RunCtl *ctl;
  const Draws *draws;
  int vote_blocks;         // blocks of each stage (B_thresh / 8 buckets, one a warp)
  int packed;              // vote table of 2-bit counters
  int per_item;            // consecutive blocks of a stage per work item
};

struct TailRange {  // items [first, first + count) cover the blocks of stage `stage` of `plan`
  int first, count, plan, stage;
};

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// stage s of a plan -> (kind, location loop)
__device__ __forceinline__ void stage_of(const TailPlan &tp, int s, int *kind, int *loop) {
  const int marks = min(max(tp.loops_thresh - 1, 0), tp.loops_loc);
  if (s < marks) {
    *kind = ST_MARK;
    *loop = s;
    return;
  }
  const int r = s - marks;
  *kind = (r & 1) ? ST_WRITE : ST_COUNT;
  *loop = marks + r / 2;
}

// Eight CTAs per SM (32 registers): the walks are chains of dependent L2 and
// DRAM reads, so warps in flight set the pace (measured on 256 mixed signals:
// 6.27 ms per batch at 4 CTAs per SM, 6.00 at 6, 5.76 at 8).
__global__ void __launch_bounds__(VT, 8)
batch_tail_kernel(const TailPlan *__restrict__ plans, const TailRange *__restrict__ ranges,
                  const int *__restrict__ item_range, int total, int *queue, int *done, int *err) {
  __shared__ int s_item, s_range;
  while (true) {
    __syncthreads();  // the previous item is finished with the shared memory
    if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    if (threadIdx.x == 0) {
      const int lo = item_range[item];
      s_range = lo;
      const TailRange r = ranges[lo];
      if (r.stage > 0) {
        // every block of the plan's previous stage
        const int *dp = done + r.plan * MAX_STAGES + r.stage - 1;
        const int want = plans[r.plan].vote_blocks;
        const long long t0 = clock64();
        while (ld_acquire(dp) < want) {
          if (clock64() - t0 > kTailWaitLimit) {
            atomicExch(&plans[r.plan].ctl->err, 1);
            atomicExch(err, 1);
            break;
          }
          __nanosleep(64);
        }
      }
    }
    __syncthreads();
    const TailRange r = ranges[s_range];
    const TailPlan &tp = plans[r.plan];
    int kind, l;
    stage_of(tp, r.stage, &kind, &l);
    WalkArgs w;
    w.J = tp.J + (size_t)l * tp.Bt;
    w.Bt = tp.Bt;
    w.n = tp.n;
    w.nb = tp.nb;
    w.W = tp.W;
    w.bm = tp.bm_sig + (size_t)(tp.W / 32) * l;
    w.fmax = &tp.ctl->fmax[l];
    w.a = (unsigned)tp.draws->a[l];
    w.packed = tp.packed;
    const unsigned epoch = *tp.epoch;
    const int nblk = tp.vote_blocks;
    int *blk_pre = tp.blk + nblk + 1;
    int *stash = tp.blk + 2 * (nblk + 1);
    const int b0 = (item - r.first) * tp.per_item;
    const int b1 = min(b0 + tp.per_item, nblk);
    for (int b = b0; b < b1; b++) {
      if (kind == ST_MARK)
        vote_mark_block(w, epoch, tp.vote, b);
      else if (kind == ST_COUNT)
        vote_count_block(w, epoch, (unsigned)tp.loops_thresh, tp.vote, tp.cnt, tp.blk, blk_pre,
                         stash, tp.ctl, b, nblk);
      else
        vote_write_block(w, epoch, (unsigned)tp.loops_thresh, tp.vote, tp.cnt, blk_pre, stash,
                         tp.cand, tp.cap, tp.ctl, b, nblk);
      __syncthreads();  // the block bodies reuse their shared memory
    }
    // every thread's writes of this item reach gpu scope before it is counted
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(done + r.plan * MAX_STAGES + r.stage, b1 - b0);
  }
}

int stages_of(const gsfft_params &p) {
  const int marks = std::min(std::max(p.loops_thresh - 1, 0), p.loops_loc);
  return marks + 2 * (p.loops_loc - marks);
}

}  // namespace

struct BatchTail {
  int nplans = 0, nranges = 0, total = 0, grid = 0;
  TailPlan *d_plans = nullptr;
  TailRange *d_ranges = nullptr;
  int *d_item_range = nullptr;  // work item -> its range
  int *d_done = nullptr;  // nplans x MAX_STAGES, then the queue ticket, then the error flag
  size_t done_ints = 0;
};

void batch_tail_free(BatchTail *t) {
  if (!t) return;
  if (t->d_plans) cudaFree(t->d_plans);
  if (t->d_ranges) cudaFree(t->d_ranges);
  if (t->d_item_range) cudaFree(t->d_item_range);
  if (t->d_done) cudaFree(t->d_done);
  delete t;
}

int batch_tail_create(Plan *const *plans, int count, BatchTail **out) {
  *out = nullptr;
  if (count < 1) return GSFFT_ERR_PARAM;
  std::vector<TailPlan> tps(count);
  int max_stages = 0;
  for (int i = 0; i < count; i++) {
    const Plan *P = plans[i];
    const gsfft_params &p = P->p;
    if (p.loops_loc > MAX_LOOPS) return GSFFT_ERR_UNSUPPORTED;
    TailPlan &t = tps[i];
    t.J = P->J;
    t.bm_sig = P->bm_sig;
    t.Bt = p.B_thresh;
    t.n = p.n;
    t.nb = p.n / p.B;
    t.W = p.W_RLFC;
    t.loops_loc = p.loops_loc;
    t.loops_thresh = p.loops_thresh;
    t.epoch = P->d_epoch;
    t.vote = P->vote;
    t.cnt = P->cnt;
    t.blk = P->blk;
    t.cand = P->cand;
    t.cap = P->cap;
    t.ctl = P->ctl;
    t.draws = P->d_draws;
    t.vote_blocks = (p.B_thresh + WPB - 1) / WPB;
    t.packed = P->packed_vote ? 1 : 0;
    t.per_item = kBlocksPerItem;
    max_stages = std::max(max_stages, stages_of(p));
  }
  // items, stage-major over the plans
  std::vector<TailRange> ranges;
  long long total = 0;
  for (int s = 0; s < max_stages; s++) {
    for (int i = 0; i < count; i++) {
      if (s >= stages_of(plans[i]->p)) continue;
      TailRange r;
      r.first = (int)total;
      r.count = (tps[i].vote_blocks + tps[i].per_item - 1) / tps[i].per_item;
      r.plan = i;
      r.stage = s;
      ranges.push_back(r);
      total += r.count;
      if (total > (1LL << 28)) return GSFFT_ERR_UNSUPPORTED;
    }
  }
  std::vector<int> item_range((size_t)total);
  for (size_t r = 0; r < ranges.size(); r++)
    for (int i = 0; i < ranges[r].count; i++) item_range[(size_t)ranges[r].first + i] = (int)r;
  BatchTail *t = new BatchTail();
  t->nplans = count;
  t->nranges = (int)ranges.size();
  t->total = (int)total;
  t->done_ints = (size_t)count * MAX_STAGES + 2;
  int s = GSFFT_OK;
  if (cudaMalloc(&t->d_plans, sizeof(TailPlan) * count) != cudaSuccess ||
      cudaMalloc(&t->d_ranges, sizeof(TailRange) * ranges.size()) != cudaSuccess ||
      cudaMalloc(&t->d_item_range, sizeof(int) * item_range.size()) != cudaSuccess ||
      cudaMalloc(&t->d_done, sizeof(int) * t->done_ints) != cudaSuccess)
    s = GSFFT_ERR_ALLOC;
  if (s == GSFFT_OK &&
      (cudaMemcpy(t->d_plans, tps.data(), sizeof(TailPlan) * count, cudaMemcpyHostToDevice) !=
           cudaSuccess ||
       cudaMemcpy(t->d_ranges, ranges.data(), sizeof(TailRange) * ranges.size(),
                  cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(t->d_item_range, item_range.data(), sizeof(int) * item_range.size(),
                  cudaMemcpyHostToDevice) != cudaSuccess))
    s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) {
    int dev = 0, sms = 0, per = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_tail_kernel, VT, 0) != cudaSuccess)
      s = GSFFT_ERR_CUDA;
    else if (!coop || per < 1)
      s = GSFFT_ERR_UNSUPPORTED;
    else
      t->grid = (int)std::min<long long>((long long)per * sms, total);
  }
  if (s != GSFFT_OK) {
    if (s == GSFFT_ERR_CUDA || s == GSFFT_ERR_ALLOC)
      set_last_error("persistent batch tail set-up: %s", cudaGetErrorString(cudaGetLastError()));
    batch_tail_free(t);
    return s;
  }
  *out = t;
  return GSFFT_OK;
}

int batch_tail_launch(BatchTail *t, cudaStream_t st) {
  GS_CUDA(cudaMemsetAsync(t->d_done, 0, sizeof(int) * t->done_ints, st));
  int *queue = t->d_done + (size_t)t->nplans * MAX_STAGES;
  int *err = queue + 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(t->grid);
  cfg.blockDim = dim3(VT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GS_CUDA(cudaLaunchKernelEx(&cfg, batch_tail_kernel, (const TailPlan *)t->d_plans,
                             (const TailRange *)t->d_ranges, (const int *)t->d_item_range,
                             t->total, queue,
                             t->d_done, err));
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
