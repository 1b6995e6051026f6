// Deterministic top-`num` selection (the cutoff of innerLoop.cu:551-642).
//
// The reference sorts every sample with thrust::stable_sort to read element
// size-num-1 of the ascending order (nth_element_immutable_cuda, :624-642),
// takes every sample above that threshold through an atomic counter
// (cutoffKernel, :875-890), fills the remaining slots with samples equal to
// the threshold in ascending index order on the host (:591-599) and sorts the
// ids (:605).  Here the same set is computed without a sort and without host
// round trips:
//   1. MSD radix select of the threshold key on the unsigned bit pattern of
//      the (non-negative) samples: 11/11/11/11/10/10-bit digits for doubles,
//      11/11/10 for floats, one histogram pass each; the last CTA of every
//      pass (ticket counter) picks the digit on the device.
//   2. One counting pass (per 4096-sample tile: #greater, #equal) whose last
//      CTA scans the tile counts.
//   3. One writing pass: sample i is taken iff key > thr, or key == thr and
//      fewer than num - #greater equal keys precede it; its output slot is the
//      number of taken samples before it, so ids come out ascending.
// Optional rounding floor: with the row maximum known, samples below
// floor_rel * max are read as exact zeros.  In a noiseless signal most RLFC
// bins are zero in exact arithmetic and an FFT leaves them at rounding level;
// the floor makes their ties resolve by index, the reference's own tie rule,
// instead of by rounding noise, so FP64, FP32 and the CPU oracle pick the
// same ids.
#include "gsfft_internal.cuh"

namespace gsfft {

namespace {

constexpr int SEL_THREADS = 256;
constexpr int SEL_ITEMS = 16;
constexpr int SEL_TILE = SEL_THREADS * SEL_ITEMS;
constexpr int HIST_BINS = 2048;

struct SelState {
  unsigned long long floor;   // keys below this count as 0 (0 = no floor)
  unsigned long long prefix;  // key bits decided so far
  long long rank;             // ascending rank still to find inside the prefix
  int size;                   // live size of the row
  int take_all;               // size <= num: every live sample is taken
  unsigned ticket;
  int total_gt;
  int total_eq;
  int pad;
};

template <typename K> __device__ __forceinline__ K raw_key(const void *p, long long i);
template <> __device__ __forceinline__ unsigned long long raw_key<unsigned long long>(const void *p, long long i) {
  return (unsigned long long)__double_as_longlong(__ldg(reinterpret_cast<const double *>(p) + i));
}
template <> __device__ __forceinline__ unsigned int raw_key<unsigned int>(const void *p, long long i) {
  return __float_as_uint(__ldg(reinterpret_cast<const float *>(p) + i));
}
template <typename K> __device__ __forceinline__ K load_key(const void *p, long long i, K floor) {
  const K k = raw_key<K>(p, i);
  return k < floor ? (K)0 : k;
}

template <typename K>
__global__ void sel_init_kernel(SelState *st, unsigned *hist, long long size, const int *size_dev,
                                int num, const void *row_max, double floor_rel) {
  const int b = blockIdx.x;
  for (int i = threadIdx.x; i < HIST_BINS; i += blockDim.x) hist[(long long)b * HIST_BINS + i] = 0;
  if (threadIdx.x == 0) {
    long long sz = size;
    if (size_dev) {
      long long d = *size_dev;
      sz = d < size ? d : size;
      if (sz < 0) sz = 0;
    }
    SelState s;
    s.floor = 0;
    if (row_max && floor_rel > 0.0) {
      // floor = (T)(max * floor_rel), the product rounded in double
      if (sizeof(K) == 8) {
        const double m = __longlong_as_double((long long)reinterpret_cast<const unsigned long long *>(row_max)[b]);
        s.floor = (unsigned long long)__double_as_longlong(m * floor_rel);
      } else {
        const float m = __uint_as_float(reinterpret_cast<const unsigned *>(row_max)[b]);
        s.floor = __float_as_uint((float)((double)m * floor_rel));
      }
    }
    s.prefix = 0;
    s.size = (int)sz;
    s.take_all = sz <= num ? 1 : 0;
    s.rank = sz - num - 1;
    s.ticket = 0;
    s.total_gt = 0;
    s.total_eq = 0;
    s.pad = 0;
    st[b] = s;
  }
}

// Block-wide exclusive scan of one value per thread (SEL_THREADS threads).
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned *warp_sums, unsigned *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned w = lane < SEL_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SEL_THREADS / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  unsigned base = wid ? warp_sums[wid - 1] : 0;
  unsigned tot = warp_sums[SEL_THREADS / 32 - 1];
  __syncthreads();
  if (total) *total = tot;
  return base + x - v;
}

template <typename K>
__global__ void __launch_bounds__(SEL_THREADS)
sel_hist_kernel(const void *keys, long long row_stride, SelState *st, unsigned *hist, int shift,
                int width) {
  __shared__ unsigned sh[HIST_BINS];
  __shared__ unsigned warp_sums[SEL_THREADS / 32];
  __shared__ int is_last;
  const int b = blockIdx.y;
  SelState *s = st + b;
  if (s->take_all) return;
  const int size = s->size;
  const unsigned long long prefix = s->prefix;
  const K floor = (K)s->floor;
  const int kb = (int)sizeof(K) * 8;
  const unsigned long long hi_mask =
      (shift + width >= kb) ? 0ull : (~0ull << (shift + width)) & (kb == 64 ? ~0ull : 0xffffffffull);
  const unsigned dmask = (1u << width) - 1u;
  for (int i = threadIdx.x; i < HIST_BINS; i += SEL_THREADS) sh[i] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * SEL_TILE;
  const void *row = reinterpret_cast<const char *>(keys) + (size_t)b * row_stride * sizeof(K);
  const int lane = threadIdx.x & 31;
#pragma unroll 4
  for (int it = 0; it < SEL_ITEMS; it++) {
    const long long i = base + it * SEL_THREADS + threadIdx.x;
    bool hit = false;
    unsigned digit = 0;
    if (i < size) {
      const unsigned long long k = (unsigned long long)load_key<K>(row, i, floor);
      hit = (k & hi_mask) == prefix;
      digit = (unsigned)(k >> shift) & dmask;
    }
    // warp-aggregated increment: lanes with the same digit add once
    // (invalid lanes get distinct keys above the digit range)
    const unsigned key = hit ? digit : (0x80000000u | (unsigned)lane);
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (hit && lane == __ffs(peers) - 1) atomicAdd(&sh[digit], (unsigned)__popc(peers));
  }
  __syncthreads();
  unsigned *gh = hist + (size_t)b * HIST_BINS;
  for (int i = threadIdx.x; i < HIST_BINS; i += SEL_THREADS)
    if (sh[i]) atomicAdd(&gh[i], sh[i]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(&s->ticket, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // last CTA: find the digit holding ascending rank s->rank
  const long long rank = s->rank;
  const int per = HIST_BINS / SEL_THREADS;  // 8 bins per thread
  unsigned local[HIST_BINS / SEL_THREADS];
  unsigned sum = 0;
#pragma unroll
  for (int q = 0; q < per; q++) {
    local[q] = atomicAdd(&gh[threadIdx.x * per + q], 0u);
    sum += local[q];
  }
  unsigned tot;
  unsigned before = block_excl_scan(sum, warp_sums, &tot);
  // exactly one thread owns the bin with before_bin <= rank < before_bin + count
  unsigned run = before;
#pragma unroll
  for (int q = 0; q < per; q++) {
    if ((long long)run <= rank && rank < (long long)run + local[q]) {
      s->prefix = prefix | ((unsigned long long)(threadIdx.x * per + q) << shift);
      s->rank = rank - run;
    }
    run += local[q];
  }
  for (int i = threadIdx.x; i < HIST_BINS; i += SEL_THREADS) gh[i] = 0;
  __syncthreads();
  if (threadIdx.x == 0) s->ticket = 0;
}

template <typename K>
__global__ void __launch_bounds__(SEL_THREADS)
sel_count_kernel(const void *keys, long long row_stride, SelState *st, unsigned *tiles,
                 int max_tiles) {
  __shared__ unsigned warp_sums[SEL_THREADS / 32];
  __shared__ int is_last;
  const int b = blockIdx.y;
  SelState *s = st + b;
  if (s->take_all) return;
  const int size = s->size;
  const K thr = (K)s->prefix;
  const K floor = (K)s->floor;
  const long long base = (long long)blockIdx.x * SEL_TILE;
  const void *row = reinterpret_cast<const char *>(keys) + (size_t)b * row_stride * sizeof(K);
  unsigned gt = 0, eq = 0;
#pragma unroll 4
  for (int it = 0; it < SEL_ITEMS; it++) {
    const long long i = base + it * SEL_THREADS + threadIdx.x;
    if (i < size) {
      const K k = load_key<K>(row, i, floor);
      gt += k > thr;
      eq += k == thr;
    }
  }
  unsigned tgt, teq;
  block_excl_scan(gt, warp_sums, &tgt);
  block_excl_scan(eq, warp_sums, &teq);
  unsigned *tb = tiles + (size_t)b * max_tiles * 4;  // [gt, eq, gt_before, eq_before]
  if (threadIdx.x == 0) {
    tb[blockIdx.x * 4 + 0] = tgt;
    tb[blockIdx.x * 4 + 1] = teq;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(&s->ticket, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // last CTA: exclusive scan of the tile counts, in chunks of SEL_THREADS
  const int ntiles = gridDim.x;
  unsigned run_gt = 0, run_eq = 0;
  for (int c = 0; c < ntiles; c += SEL_THREADS) {
    const int t = c + threadIdx.x;
    unsigned vg = t < ntiles ? atomicAdd(&tb[t * 4 + 0], 0u) : 0;
    unsigned ve = t < ntiles ? atomicAdd(&tb[t * 4 + 1], 0u) : 0;
    unsigned cg, ce;
    unsigned eg = block_excl_scan(vg, warp_sums, &cg);
    unsigned ee = block_excl_scan(ve, warp_sums, &ce);
    if (t < ntiles) {
      tb[t * 4 + 2] = run_gt + eg;
      tb[t * 4 + 3] = run_eq + ee;
    }
    run_gt += cg;
    run_eq += ce;
  }
  if (threadIdx.x == 0) {
    s->total_gt = (int)run_gt;
    s->total_eq = (int)run_eq;
    s->ticket = 0;
  }
}

template <typename K>
__global__ void __launch_bounds__(SEL_THREADS)
sel_write_kernel(const void *keys, long long row_stride, const SelState *st, const unsigned *tiles,
                 int max_tiles, int num, int *out, long long out_stride, int *count_out) {
  __shared__ unsigned warp_sums[SEL_THREADS / 32];
  const int b = blockIdx.y;
  const SelState *s = st + b;
  const int size = s->size;
  int *o = out + (size_t)b * out_stride;
  const long long base = (long long)blockIdx.x * SEL_TILE;
  if (s->take_all) {
    for (int it = 0; it < SEL_ITEMS; it++) {
      const long long i = base + it * SEL_THREADS + threadIdx.x;
      if (i < size) o[i] = (int)i;
    }
    if (count_out && blockIdx.x == 0 && threadIdx.x == 0) count_out[b] = size;
    return;
  }
  const K thr = (K)s->prefix;
  const K floor = (K)s->floor;
  const unsigned *tb = tiles + (size_t)b * max_tiles * 4;
  unsigned gt_run = tb[blockIdx.x * 4 + 2];
  unsigned eq_run = tb[blockIdx.x * 4 + 3];
  const unsigned need_eq = (unsigned)(num - s->total_gt);
  const void *row = reinterpret_cast<const char *>(keys) + (size_t)b * row_stride * sizeof(K);
  for (int it = 0; it < SEL_ITEMS; it++) {
    const long long i = base + it * SEL_THREADS + threadIdx.x;
    unsigned g = 0, e = 0;
    if (i < size) {
      const K k = load_key<K>(row, i, floor);
      g = k > thr;
      e = k == thr;
    }
    unsigned cg, ce;
    const unsigned pg = block_excl_scan(g, warp_sums, &cg);
    const unsigned pe = block_excl_scan(e, warp_sums, &ce);
    const unsigned eq_before = eq_run + pe;
    if (g || (e && eq_before < need_eq)) {
      const unsigned pos = gt_run + pg + (eq_before < need_eq ? eq_before : need_eq);
      if (pos < (unsigned)num) o[pos] = (int)i;
    }
    gt_run += cg;
    eq_run += ce;
  }
  if (count_out && blockIdx.x == 0 && threadIdx.x == 0) count_out[b] = num;
}

template <typename K>
int select_impl(const void *keys, long long size, const int *size_dev, int num, int batch,
                long long row_stride, int *out, long long out_stride, int *count_out,
                SelectScratch &s, cudaStream_t st, const void *row_max, double floor_rel) {
  if (batch > s.max_batch || size <= 0) return GSFFT_ERR_PARAM;
  const long long tiles = (size + SEL_TILE - 1) / SEL_TILE;
  if (tiles > s.max_tiles) return GSFFT_ERR_PARAM;
  SelState *state = reinterpret_cast<SelState *>(s.state);
  unsigned *hist = reinterpret_cast<unsigned *>(s.hist);
  unsigned *tl = reinterpret_cast<unsigned *>(s.tiles);
  sel_init_kernel<K><<<batch, 256, 0, st>>>(state, hist, size, size_dev, num, row_max, floor_rel);
  GS_LAUNCHED();
  dim3 grid((unsigned)tiles, (unsigned)batch);
  const int kb = (int)sizeof(K) * 8;
  const int w64[6] = {11, 11, 11, 11, 10, 10};
  const int w32[3] = {11, 11, 10};
  const int *widths = kb == 64 ? w64 : w32;
  const int npass = kb == 64 ? 6 : 3;
  int shift = kb;
  for (int p = 0; p < npass; p++) {
    shift -= widths[p];
    sel_hist_kernel<K><<<grid, SEL_THREADS, 0, st>>>(keys, row_stride, state, hist, shift, widths[p]);
    GS_LAUNCHED();
  }
  sel_count_kernel<K><<<grid, SEL_THREADS, 0, st>>>(keys, row_stride, state, tl, s.max_tiles);
  GS_LAUNCHED();
  sel_write_kernel<K><<<grid, SEL_THREADS, 0, st>>>(keys, row_stride, state, tl, s.max_tiles, num,
                                                    out, out_stride, count_out);
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace

int select_scratch_init(SelectScratch &s, int max_batch, long long max_size) {
  select_scratch_free(s);
  s.max_batch = max_batch;
  s.max_tiles = (int)((max_size + SEL_TILE - 1) / SEL_TILE);
  GS_CUDA(cudaMalloc(&s.hist, sizeof(unsigned) * HIST_BINS * max_batch));
  GS_CUDA(cudaMalloc(&s.state, sizeof(SelState) * max_batch));
  GS_CUDA(cudaMalloc(&s.tiles, sizeof(unsigned) * 4 * (size_t)s.max_tiles * max_batch));
  GS_CUDA(cudaMemset(s.state, 0, sizeof(SelState) * max_batch));
  return GSFFT_OK;
}

void select_scratch_free(SelectScratch &s) {
  if (s.hist) cudaFree(s.hist);
  if (s.state) cudaFree(s.state);
  if (s.tiles) cudaFree(s.tiles);
  s.hist = s.state = s.tiles = nullptr;
}

int select_launches(int key_bytes) { return key_bytes == 8 ? 9 : 6; }

int select_top(const void *keys, int key_bytes, long long size, const int *size_dev, int num,
               int batch, long long row_stride, int *out, long long out_stride, int *count_out,
               SelectScratch &s, cudaStream_t st, const void *row_max, double floor_rel) {
  if (size_dev && batch != 1) return GSFFT_ERR_PARAM;
  if (key_bytes == 8)
    return select_impl<unsigned long long>(keys, size, size_dev, num, batch, row_stride, out,
                                           out_stride, count_out, s, st, row_max, floor_rel);
  if (key_bytes == 4)
    return select_impl<unsigned int>(keys, size, size_dev, num, batch, row_stride, out,
                                     out_stride, count_out, s, st, row_max, floor_rel);
  return GSFFT_ERR_PARAM;
}

}  // namespace gsfft
