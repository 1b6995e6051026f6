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

#include <cooperative_groups.h>

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


// ---------------------------------------------------------------------------
// Single-launch form: the same selection in one cooperative kernel.  Row b
// is split into `cpr` contiguous chunks, one per CTA.  Each radix pass builds
// the CTA's chunk histogram in shared memory and adds it to the row's global
// histogram once; after a grid-wide sync every CTA derives its row's digit
// itself.  A pass ends the descent early when the threshold's bin is "pure":
// it holds one sample, or it is the first pass's digit 0 while the rounding
// floor maps every key of that digit to exact zero.  Keys are then compared
// on the bits decided so far; in the second case the first pass has already
// stored every chunk's (nonzero, zero) counts, which are the (#greater,
// #equal) counts of threshold 0, so the counting pass is skipped too (a
// noiseless spectrum: one histogram pass and the write pass).  Counting and
// writing use per-thread runs of contiguous samples and one packed block scan
// per sub-tile, so ids come out ascending.  Rows that start on 16-byte
// boundaries (with a capacity of whole 16-byte words) are read with 16-byte
// loads.  Histograms are left zeroed for the next call.
//
// Two launch forms of the same kernel, differing only in their barrier:
//   - cooperative (CLU = false): one grid over all rows, `grid.sync()`; used
//     for long rows, which need every SM's bandwidth;
//   - one thread-block cluster per row (CLU = true): `cpr` <= 16 CTAs whose
//     co-residency the hardware guarantees, `barrier.cluster` between passes.
//     An ordinary launch, so selections of several plans on several streams
//     run side by side (cooperative launches of different streams do not
//     overlap), and its barrier is far cheaper than a grid-wide one.
// ---------------------------------------------------------------------------
namespace cg = cooperative_groups;

constexpr int MAXB = 8;         // rows per cooperative call
constexpr int CT = 512;         // threads per CTA
constexpr int SPT = 8;          // contiguous samples per thread in the write pass
constexpr int CHUNK_MIN = 2048; // smallest chunk per CTA
constexpr int UN = 8;           // loads in flight per thread in the scan passes
constexpr int UQ = 4;           // 16-byte loads in flight per thread (aligned rows)
constexpr int COOP_SMEM = (CT / 32) * (HIST_BINS / 2) * 4;  // per-warp histograms
constexpr long long MAX_CHUNK = 16LL * 65535;  // keeps a warp's 16-bit counters exact
constexpr int CLUSTER_MAX = 16;  // CTAs per row in the cluster form (non-portable size)
// Rows up to this many samples (and top-k rows with a device-side live size)
// take the cluster form.
constexpr long long CLUSTER_ROW_MAX = 1LL << 18;
// CTAs per SM the register budget is set for: three for 32-bit keys (the
// large scans need the memory parallelism; two measured slower), two for
// 64-bit keys (no spills; the top-k rows are short).
template <typename K> constexpr int coop_ctas_per_sm() { return sizeof(K) == 4 ? 3 : 2; }

struct CoopArgs {
  const void *keys;
  long long size;        // capacity per row
  const int *size_dev;   // live size (batch 1) or null
  int num, batch, cpr;
  long long row_stride;
  int *out;
  long long out_stride;
  int *count_out;
  const void *row_max;
  double floor_rel;
  unsigned *hist;        // [6][MAXB][HIST_BINS], zero on entry and on exit
  unsigned *tiles;       // [MAXB][max_tiles][2]: per-chunk (#greater, #equal)
  int max_tiles;
};

// Block-wide exclusive scan over CT threads (two syncs).
__device__ __forceinline__ unsigned ct_excl_scan(unsigned v, unsigned *ws, unsigned *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned w = lane < CT / 32 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < CT / 32) ws[lane] = w;
  }
  __syncthreads();
  const unsigned base = wid ? ws[wid - 1] : 0;
  const unsigned tot = ws[CT / 32 - 1];
  __syncthreads();
  if (total) *total = tot;
  return base + x - v;
}

// Calls fn(i, key) for every sample i in [lo, hi) of the row, its key read
// as 0 below the floor; UN scalar loads per thread in flight, or (VEC: the
// row and its capacity are 16-byte aligned) UQ 16-byte loads.  lo is a
// multiple of 32 samples unless the chunk is empty (lo = hi = the live size,
// which may fall inside a 16-byte word: hence the i >= lo test).
template <typename K> __host__ __device__ constexpr int keys_per_quad() { return 16 / (int)sizeof(K); }

template <typename K>
__device__ __forceinline__ void unpack_quad(const uint4 &v, K (&ks)[keys_per_quad<K>()]) {
  if constexpr (sizeof(K) == 4) {
    ks[0] = v.x;
    ks[1] = v.y;
    ks[2] = v.z;
    ks[3] = v.w;
  } else {
    ks[0] = (unsigned long long)v.x | ((unsigned long long)v.y << 32);
    ks[1] = (unsigned long long)v.z | ((unsigned long long)v.w << 32);
  }
}

template <typename K, bool VEC, class F>
__device__ __forceinline__ void for_chunk_keys(const void *row, long long lo, long long hi, K floor,
                                               F &&fn) {
  const int tid = threadIdx.x;
  if constexpr (VEC) {
    constexpr int EPQ = keys_per_quad<K>();
    const uint4 *rq = reinterpret_cast<const uint4 *>(row);
    const long long q_lo = lo / EPQ, q_hi = (hi + EPQ - 1) / EPQ;
    for (long long qb = q_lo; qb < q_hi; qb += (long long)CT * UQ) {
      uint4 v[UQ];
#pragma unroll
      for (int u = 0; u < UQ; u++) {
        const long long q = qb + (long long)u * CT + tid;
        v[u] = q < q_hi ? __ldg(rq + q) : make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int u = 0; u < UQ; u++) {
        const long long q = qb + (long long)u * CT + tid;
        K ks[EPQ];
        unpack_quad<K>(v[u], ks);
#pragma unroll
        for (int e = 0; e < EPQ; e++) {
          const long long i = q * EPQ + e;
          if (q < q_hi && i >= lo && i < hi) fn(i, ks[e] < floor ? (K)0 : ks[e]);
        }
      }
    }
  } else {
    for (long long base = lo; base < hi; base += (long long)CT * UN) {
      K kv[UN];
#pragma unroll
      for (int u = 0; u < UN; u++) {
        const long long i = base + (long long)u * CT + tid;
        kv[u] = i < hi ? load_key<K>(row, i, floor) : (K)0;
      }
#pragma unroll
      for (int u = 0; u < UN; u++) {
        const long long i = base + (long long)u * CT + tid;
        if (i < hi) fn(i, kv[u]);
      }
    }
  }
}

template <typename K, bool CLU, bool VEC>
__global__ void __launch_bounds__(CT, coop_ctas_per_sm<K>()) sel_coop_kernel(CoopArgs a) {
  // Launched without programmatic serialization (it follows its predecessor
  // completely); the trigger lets the next kernel's launch overlap this one,
  // whose blocks are all resident already.
  pdl_enter();
  // Every barrier below is reached by all threads of all CTAs that take part
  // in it: the conditions around them are uniform over the grid (cooperative
  // form) or over the row's cluster (cluster form).
  auto sync_all = [&]() {
    if constexpr (CLU) cg::this_cluster().sync();
    else cg::this_grid().sync();
  };
  // one private histogram per warp, two 16-bit counters per word, so warps
  // never contend on a bin (a warp counts at most chunk / 16 < 65536 keys)
  extern __shared__ unsigned wh[];  // [CT / 32][HIST_BINS / 2]
  __shared__ unsigned ws[CT / 32];
  __shared__ unsigned long long s_prefix;
  __shared__ unsigned s_settled[MAXB];  // per row: its rank falls among its floored zeros
  __shared__ long long s_rank;
  __shared__ unsigned s_bincount;
  const int tid = threadIdx.x, lane = tid & 31;
  constexpr int kb = (int)sizeof(K) * 8;
  const int w64[6] = {11, 11, 11, 11, 10, 10};
  const int w32[3] = {11, 11, 10};
  constexpr int npass = kb == 64 ? 6 : 3;
  constexpr int shift0 = kb - 11;  // shift of the first pass's digit
  const int b = blockIdx.x / a.cpr, ci = blockIdx.x % a.cpr;
  // row state (identical in every CTA of the row)
  long long sz = a.size;
  if (a.size_dev) {
    const long long dv = *a.size_dev;
    sz = dv < a.size ? dv : a.size;
    if (sz < 0) sz = 0;
  }
  // rounding floor of row r (0: none)
  auto row_floor = [&](int r) -> K {
    if (!(a.row_max && a.floor_rel > 0.0)) return (K)0;
    if (kb == 64) {
      const double m = __longlong_as_double((long long)reinterpret_cast<const unsigned long long *>(a.row_max)[r]);
      return (K)(unsigned long long)__double_as_longlong(m * a.floor_rel);
    }
    const float m = __uint_as_float(reinterpret_cast<const unsigned *>(a.row_max)[r]);
    return (K)__float_as_uint((float)((double)m * a.floor_rel));
  };
  // With a floor of at least 2^shift0, every key is either 0 or at least the
  // floor, so digit 0 of the first pass holds exactly the row's zeros.
  auto zero_digit = [&](int r) -> bool { return (unsigned long long)row_floor(r) >= (1ull << shift0); };
  const K floor = row_floor(b);
  const bool zdig = zero_digit(b);
  const bool take_all = sz <= a.num;
  const long long chunk = ((sz + a.cpr - 1) / a.cpr + 31) & ~31LL;
  const long long lo = (long long)ci * chunk < sz ? (long long)ci * chunk : sz;
  const long long hi = lo + chunk < sz ? lo + chunk : sz;
  const void *row = reinterpret_cast<const char *>(a.keys) + (size_t)b * a.row_stride * sizeof(K);
  const long long rank0 = sz - a.num - 1;  // the same for every row (rows share one size)
  unsigned long long prefix = 0;
  long long rank = rank0;
  int cmp_shift = 0;  // low bits ignored by the final comparisons
  bool done = take_all;
  bool counted = false;  // the chunk counts for the final threshold are already stored
  // every row settled (the cluster form: this row settled): uniform over the
  // CTAs sharing the barrier, so every one of them skips the same barriers
  bool all_done = take_all;
  int shift = kb;
  for (int p = 0; p < npass && !all_done; p++) {
    const int width = kb == 64 ? w64[p] : w32[p];
    shift -= width;
    if (!done) {
      const unsigned dmask = (1u << width) - 1u;
      const unsigned long long hi_mask =
          (shift + width >= kb) ? 0ull : (~0ull << (shift + width)) & (kb == 64 ? ~0ull : 0xffffffffull);
      unsigned *mine = wh + (tid >> 5) * (HIST_BINS / 2);
      for (int i = lane; i < HIST_BINS / 2; i += 32) mine[i] = 0;
      __syncwarp();
      // Digit 0 (floored zeros dominate the first pass of a noiseless
      // spectrum) is counted in a register; other digits go to the warp's
      // private table, where only collisions inside the warp remain.
      unsigned zeros = 0;
      for_chunk_keys<K, VEC>(row, lo, hi, floor, [&](long long, K key) {
        const unsigned long long k = (unsigned long long)key;
        if ((k & hi_mask) == prefix) {
          const unsigned digit = (unsigned)(k >> shift) & dmask;
          if (digit == 0) zeros++;
          else atomicAdd(&mine[digit >> 1], 1u << ((digit & 1u) * 16));
        }
      });
      zeros = __reduce_add_sync(0xffffffffu, zeros);
      if (lane == 0 && zeros) atomicAdd(&mine[0], zeros);  // bin 0 = low half of word 0
      __syncthreads();
      unsigned *gh = a.hist + ((size_t)p * MAXB + b) * HIST_BINS;
      for (int word = tid; word < HIST_BINS / 2; word += CT) {
        unsigned lo16 = 0, hi16 = 0;
#pragma unroll 4
        for (int wv = 0; wv < CT / 32; wv++) {
          const unsigned v = wh[wv * (HIST_BINS / 2) + word];
          lo16 += v & 0xffffu;
          hi16 += v >> 16;
        }
        if (lo16) atomicAdd(&gh[2 * word], lo16);
        if (hi16) atomicAdd(&gh[2 * word + 1], hi16);
        // Bin 0 of the first pass is this chunk's zero count: with the
        // threshold at 0, (nonzero, zero) are the (#greater, #equal) counts
        // the write pass needs.
        if (p == 0 && word == 0 && zdig) {
          a.tiles[((size_t)b * a.max_tiles + ci) * 2 + 0] = (unsigned)(hi - lo) - lo16;
          a.tiles[((size_t)b * a.max_tiles + ci) * 2 + 1] = lo16;
        }
      }
      __syncthreads();  // the per-warp histograms are rebuilt next pass
    }
    sync_all();
    if (!done) {
      // the digit holding ascending rank `rank` of this row
      const unsigned *gh = a.hist + ((size_t)p * MAXB + b) * HIST_BINS;
      constexpr int per = HIST_BINS / CT;
      static_assert(per == 4, "one 16-byte histogram load per thread");
      // every CTA of the row reads these words: one 16-byte load per thread
      // keeps the requests per L2 line down
      const uint4 h4 = __ldcg(reinterpret_cast<const uint4 *>(gh) + tid);
      const unsigned local[per] = {h4.x, h4.y, h4.z, h4.w};
      const unsigned sum = h4.x + h4.y + h4.z + h4.w;
      unsigned tot;
      const unsigned before = ct_excl_scan(sum, ws, &tot);
      unsigned run = before;
#pragma unroll
      for (int q = 0; q < per; q++) {
        if ((long long)run <= rank && rank < (long long)run + local[q]) {
          s_prefix = prefix | ((unsigned long long)(tid * per + q) << shift);
          s_rank = rank - run;
          s_bincount = local[q];
        }
        run += local[q];
      }
      __syncthreads();
      prefix = s_prefix;
      rank = s_rank;
      const unsigned cnt = s_bincount;
      __syncthreads();
      if (cnt == 1) {
        cmp_shift = shift;
        done = true;
      } else if (p == 0 && (prefix >> shift) == 0 && zdig) {
        done = true;  // the threshold is a floored zero; its counts are stored
        counted = true;
      }
      if (p == npass - 1) done = true;
    }
    if (CLU || a.batch == 1) {
      all_done = done;  // one row behind the barrier
    } else if (p == 0) {
      // Several rows: all of them settle here when each one's threshold is a
      // floored zero.  Every CTA reads the same final bin-0 counts, so every
      // CTA reaches the same decision (one thread per row loads them: every
      // thread loading the same words made an L2 hot spot).
      if (tid < a.batch)
        s_settled[tid] = zero_digit(tid) &&
                         (long long)__ldcg(&a.hist[(size_t)tid * HIST_BINS]) > rank0;
      __syncthreads();
      bool all = true;
      for (int r = 0; r < a.batch; r++) all = all && s_settled[r];
      all_done = all;
    }
  }
  // counting pass: (#greater, #equal) of this chunk
  const K thr = (K)prefix;
  const unsigned long long thr_c = (unsigned long long)thr >> cmp_shift;
  unsigned gt = 0, eq = 0;
  if (!take_all && !counted)
    for_chunk_keys<K, VEC>(row, lo, hi, floor, [&](long long, K key) {
      const unsigned long long kc = (unsigned long long)key >> cmp_shift;
      gt += kc > thr_c;
      eq += kc == thr_c;
    });
  unsigned tgt, teq;
  ct_excl_scan(gt, ws, &tgt);
  ct_excl_scan(eq, ws, &teq);
  if (tid == 0 && !counted) {
    a.tiles[((size_t)b * a.max_tiles + ci) * 2 + 0] = tgt;
    a.tiles[((size_t)b * a.max_tiles + ci) * 2 + 1] = teq;
  }
  sync_all();
  // the histograms were read by every CTA before the barrier above: zero
  // them for the next call (the cluster form: its own row's)
  if constexpr (CLU) {
    for (int i = ci * CT + tid; i < npass * HIST_BINS; i += a.cpr * CT)
      a.hist[((size_t)(i / HIST_BINS) * MAXB + b) * HIST_BINS + (i % HIST_BINS)] = 0;
  } else {
    for (long long i = (long long)blockIdx.x * CT + tid; i < (long long)npass * MAXB * HIST_BINS;
         i += (long long)gridDim.x * CT)
      a.hist[i] = 0;
  }
  // writing pass
  int *o = a.out + (size_t)b * a.out_stride;
  if (take_all) {
    for (long long i = lo + tid; i < hi; i += CT) o[i] = (int)i;
  } else {
    // chunk prefix and row totals
    unsigned bg = 0, be = 0, tg = 0;
    const unsigned *tb = a.tiles + (size_t)b * a.max_tiles * 2;
    for (int c2 = tid; c2 < a.cpr; c2 += CT) {
      const unsigned vg = __ldcg(&tb[c2 * 2]), ve = __ldcg(&tb[c2 * 2 + 1]);
      if (c2 < ci) {
        bg += vg;
        be += ve;
      }
      tg += vg;
    }
    unsigned s_bg, s_be, s_tg;
    ct_excl_scan(bg, ws, &s_bg);
    ct_excl_scan(be, ws, &s_be);
    ct_excl_scan(tg, ws, &s_tg);
    const unsigned need_eq = (unsigned)(a.num - (int)s_tg);
    unsigned gt_run = s_bg, eq_run = s_be;
    for (long long base = lo; base < hi; base += (long long)CT * SPT) {
      const long long i0 = base + (long long)tid * SPT;  // a multiple of SPT
      unsigned gm = 0, em = 0;  // bit q: sample i0 + q is greater / equal
      if constexpr (VEC) {
        constexpr int EPQ = keys_per_quad<K>();
        static_assert(SPT % EPQ == 0, "whole 16-byte loads per run");
        const uint4 *rq = reinterpret_cast<const uint4 *>(row) + i0 / EPQ;
        uint4 v[SPT / EPQ];
#pragma unroll
        for (int c = 0; c < SPT / EPQ; c++)
          v[c] = i0 + c * EPQ < hi ? __ldg(rq + c) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
        for (int c = 0; c < SPT / EPQ; c++) {
          K ks[EPQ];
          unpack_quad<K>(v[c], ks);
#pragma unroll
          for (int e = 0; e < EPQ; e++) {
            const int q = c * EPQ + e;
            if (i0 + q < hi) {
              const unsigned long long kc = (unsigned long long)(ks[e] < floor ? (K)0 : ks[e]) >> cmp_shift;
              gm |= (unsigned)(kc > thr_c) << q;
              em |= (unsigned)(kc == thr_c) << q;
            }
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < SPT; q++) {
          const long long i = i0 + q;
          if (i < hi) {
            const unsigned long long kc = (unsigned long long)load_key<K>(row, i, floor) >> cmp_shift;
            gm |= (unsigned)(kc > thr_c) << q;
            em |= (unsigned)(kc == thr_c) << q;
          }
        }
      }
      unsigned tot;
      const unsigned pre = ct_excl_scan((unsigned)__popc(gm) | ((unsigned)__popc(em) << 16), ws, &tot);
      const unsigned gb = gt_run + (pre & 0xffffu), eb = eq_run + (pre >> 16);
      // equal samples are taken while fewer than need_eq equal ones precede
      unsigned take = gm;
      if (eb < need_eq) {
        unsigned room = need_eq - eb, m = em;
        while (m && room) {
          take |= m & (0u - m);
          m &= m - 1;
          room--;
        }
      }
      while (take) {
        const int q = __ffs(take) - 1;
        take &= take - 1;
        const unsigned below = (1u << q) - 1u;
        const unsigned eq_before = eb + (unsigned)__popc(em & below);
        const unsigned pos = gb + (unsigned)__popc(gm & below) + (eq_before < need_eq ? eq_before : need_eq);
        if (pos < (unsigned)a.num) o[pos] = (int)(i0 + q);
      }
      gt_run += tot & 0xffffu;
      eq_run += tot >> 16;
    }
  }
  if (a.count_out && ci == 0 && tid == 0) a.count_out[b] = take_all ? (int)sz : a.num;
}

// CTAs of the cooperative form on the current device (-1: not available).
template <typename K, bool VEC>
int coop_grid() {
  static PerContext<int> cache;
  return cache.get([] {
    int dev = 0, sms = 0, per = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (!coop) return -1;
    if (cudaFuncSetAttribute(sel_coop_kernel<K, false, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             COOP_SMEM) != cudaSuccess) {
      cudaGetLastError();
      return -1;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sel_coop_kernel<K, false, VEC>, CT, COOP_SMEM);
    cudaGetLastError();
    if (per > coop_ctas_per_sm<K>()) per = coop_ctas_per_sm<K>();
    return per > 0 ? per * sms : -1;
  });
}

// Largest cluster (CTAs per row) the device schedules for the cluster form:
// 16 where non-portable sizes are allowed, else 8; 0 if clusters are not
// available.
template <typename K, bool VEC>
int cluster_max() {
  static PerContext<int> cache;
  return cache.get([] {
    int g = 0;
    if (cudaFuncSetAttribute(sel_coop_kernel<K, true, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             COOP_SMEM) != cudaSuccess) {
      cudaGetLastError();
      return g;
    }
    const bool np = cudaFuncSetAttribute(sel_coop_kernel<K, true, VEC>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    for (int c = np ? CLUSTER_MAX : 8; c >= 2 && !g; c /= 2) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(CT);
      cfg.dynamicSmemBytes = COOP_SMEM;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = c;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nc = 0;
      if (cudaOccupancyMaxActiveClusters(&nc, sel_coop_kernel<K, true, VEC>, &cfg) == cudaSuccess && nc > 0)
        g = c;
    }
    cudaGetLastError();  // a refused size leaves no error behind
    return g;
  });
}

// One launch of the single-launch select: the cluster form (CLU) or the
// cooperative form, with 16-byte key loads when every row and the row
// capacity are 16-byte aligned.
template <typename K, bool CLU, bool VEC>
int select_single_launch(const void *keys, long long size, const int *size_dev, int num, int batch,
                         long long row_stride, int *out, long long out_stride, int *count_out,
                         SelectScratch &s, cudaStream_t st, const void *row_max, double floor_rel) {
  const int cap = CLU ? cluster_max<K, VEC>() : coop_grid<K, VEC>() / batch;
  if (cap <= 0) return GSFFT_ERR_UNSUPPORTED;
  long long cpr = (size + CHUNK_MIN - 1) / CHUNK_MIN;
  if (cpr > cap) cpr = cap;
  if (cpr > s.max_tiles) cpr = s.max_tiles;
  if (cpr < 1 || (size + cpr - 1) / cpr + 32 > MAX_CHUNK) return GSFFT_ERR_UNSUPPORTED;
  CoopArgs a;
  a.keys = keys;
  a.size = size;
  a.size_dev = size_dev;
  a.num = num;
  a.batch = batch;
  a.cpr = (int)cpr;
  a.row_stride = row_stride;
  a.out = out;
  a.out_stride = out_stride;
  a.count_out = count_out;
  a.row_max = row_max;
  a.floor_rel = floor_rel;
  a.hist = reinterpret_cast<unsigned *>(s.coop_hist);
  a.tiles = reinterpret_cast<unsigned *>(s.tiles);
  a.max_tiles = s.max_tiles;
  if constexpr (CLU) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(cpr * batch));
    cfg.blockDim = dim3(CT);
    cfg.dynamicSmemBytes = COOP_SMEM;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cpr;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    GS_CUDA(cudaLaunchKernelEx(&cfg, sel_coop_kernel<K, true, VEC>, a));
  } else {
    void *args[] = {&a};
    GS_CUDA(cudaLaunchCooperativeKernel((const void *)sel_coop_kernel<K, false, VEC>,
                                        dim3((unsigned)(cpr * batch)), dim3(CT), args, COOP_SMEM, st));
  }
  GS_LAUNCHED();
  return GSFFT_OK;
}

template <typename K>
int select_single(bool clu, const void *keys, long long size, const int *size_dev, int num, int batch,
                  long long row_stride, int *out, long long out_stride, int *count_out,
                  SelectScratch &s, cudaStream_t st, const void *row_max, double floor_rel) {
  const bool vec = reinterpret_cast<uintptr_t>(keys) % 16 == 0 &&
                   ((unsigned long long)row_stride * sizeof(K)) % 16 == 0 &&
                   ((unsigned long long)size * sizeof(K)) % 16 == 0;
#define SEL_GO(C, V)                                                                                 \
  return select_single_launch<K, C, V>(keys, size, size_dev, num, batch, row_stride, out, out_stride, \
                                       count_out, s, st, row_max, floor_rel)
  if (clu) {
    if (vec) SEL_GO(true, true);
    SEL_GO(true, false);
  }
  if (vec) SEL_GO(false, true);
  SEL_GO(false, false);
#undef SEL_GO
}

}  // namespace

SelectScratchBytes select_scratch_bytes(int max_batch, long long max_size) {
  SelectScratchBytes b;
  b.max_tiles = (int)((max_size + SEL_TILE - 1) / SEL_TILE);
  b.hist = sizeof(unsigned) * HIST_BINS * (size_t)max_batch;
  b.state = sizeof(SelState) * (size_t)max_batch;
  b.tiles = sizeof(unsigned) * 4 * (size_t)b.max_tiles * max_batch;
  // single-launch form: one histogram per radix pass (at most 6) and row
  b.coop_hist = sizeof(unsigned) * 6 * MAXB * HIST_BINS;
  return b;
}

int select_scratch_init(SelectScratch &s, int max_batch, long long max_size) {
  select_scratch_free(s);
  const SelectScratchBytes b = select_scratch_bytes(max_batch, max_size);
  s.max_batch = max_batch;
  s.max_tiles = b.max_tiles;
  GS_CUDA(cudaMalloc(&s.hist, b.hist));
  GS_CUDA(cudaMalloc(&s.state, b.state));
  GS_CUDA(cudaMalloc(&s.tiles, b.tiles));
  GS_CUDA(cudaMemset(s.state, 0, b.state));
  GS_CUDA(cudaMalloc(&s.coop_hist, b.coop_hist));
  GS_CUDA(cudaMemset(s.coop_hist, 0, b.coop_hist));
  return GSFFT_OK;
}

void select_scratch_free(SelectScratch &s) {
  if (s.hist) cudaFree(s.hist);
  if (s.state) cudaFree(s.state);
  if (s.tiles) cudaFree(s.tiles);
  if (s.coop_hist) cudaFree(s.coop_hist);
  s.hist = s.state = s.tiles = s.coop_hist = nullptr;
}

size_t select_state_bytes() { return sizeof(SelState); }

int select_top(const void *keys, int key_bytes, long long size, const int *size_dev, int num,
               int batch, long long row_stride, int *out, long long out_stride, int *count_out,
               SelectScratch &s, cudaStream_t st, const void *row_max, double floor_rel) {
  if (size_dev && batch != 1) return GSFFT_ERR_PARAM;
  if (s.single_launch && batch <= MAXB && batch <= s.max_batch &&
      (size + SEL_TILE - 1) / SEL_TILE <= s.max_tiles) {
    for (const bool clu : {true, false}) {
      if (clu && !(size <= CLUSTER_ROW_MAX || size_dev)) continue;
      const int r = key_bytes == 8
                        ? select_single<unsigned long long>(clu, keys, size, size_dev, num, batch, row_stride,
                                                            out, out_stride, count_out, s, st, row_max,
                                                            floor_rel)
                        : select_single<unsigned int>(clu, keys, size, size_dev, num, batch, row_stride,
                                                      out, out_stride, count_out, s, st, row_max, floor_rel);
      if (r != GSFFT_ERR_UNSUPPORTED) return r;
    }
  }
  if (key_bytes == 8)
    return select_impl<unsigned long long>(keys, size, size_dev, num, batch, row_stride, out,
                                           out_stride, count_out, s, st, row_max, floor_rel);
  if (key_bytes == 4)
    return select_impl<unsigned int>(keys, size, size_dev, num, batch, row_stride, out,
                                     out_stride, count_out, s, st, row_max, floor_rel);
  return GSFFT_ERR_PARAM;
}

}  // namespace gsfft
