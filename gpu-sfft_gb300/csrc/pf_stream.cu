// A5 + the RLFC sub-sampling of A4 in one ordered pass over the signal.
//
// The gather form (pf.cu) reads each tap's sample at a random address; at the
// n = 2^27 sizes every such read costs a whole DRAM burst (~64-96 bytes for
// an 8-byte sample).  When loops * w random reads cost more than reading x
// once, this kernel streams x through shared memory with TMA instead.
//
// View x as an (n/B) x B matrix, x[r*B + c].  For loop l the tap of position
// t = r*B + c is i = t*a_l mod n (t = i*ai_l mod n, innerLoop.cu:738,769):
//   i = B * ((q_l + r*alpha_l) mod nb) + b_l,    nb = n/B,
//   b_l = (c*a_l) mod B,  q_l = ((c*a_l) mod n) / B,  alpha_l = a_l mod nb.
// Every tap of column c therefore belongs to the one bucket b_l (c -> b_l is
// a bijection since a_l is odd), and tap j of that bucket sits in row
//   r_j = (j*beta_l + s_l) mod nb,  beta_l = alpha_l^-1 mod nb,  s_l = -q_l*beta_l,
// i.e. the column's hit rows are one per-loop set {j*beta_l mod nb} shifted by
// s_l.  The host sorts that set once per run; one thread per (column, loop)
// walks its rotated copy in ascending row order, so it touches only its own
// ~w/B hits while the CTA streams every row of its 64 (or 32) columns exactly
// once.  Sums run in ascending row (= signal position) order: fixed, no
// atomics.
//
// Tiles of rt rows x 64 columns arrive by cp.async.bulk.tensor.2d, issued by a
// producer warp, into a shared-memory ring (three stages at two CTAs per SM;
// four at one CTA per SM in the staged-tap form) guarded by full / empty
// mbarriers whose waits are bounded (a timeout sets an error flag instead of
// hanging).  Taps: in the staged form (FP32, up to 9 loops) each consumer
// thread copies its bucket's taps into its own shared-memory slot with one
// bulk copy per work item; otherwise each hit's tap is loaded from a
// bucket-major table in L2, one hit ahead.
//
// RLFC loop r samples positions off_r + m*(n/W) (restLocFreqCoeffKernel,
// innerLoop.cu:693-703); (n/W) divides B, so those are whole columns and the
// CTA copies them from the tile to y_r[t / (n/W)].
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <vector>

#include "stages.cuh"

namespace gsfft {

namespace {

constexpr int ST = 128;      // B must be a multiple of this
constexpr int NSTAGE = 3;    // shared-memory ring of tiles (taps read from L2)
constexpr int NSTAGE_STG = 4; // ring of the staged-tap form (one CTA per SM)
constexpr int MAXT = 32;     // full tiles of taps per bucket (w / B) supported
constexpr int MAXL = 16;     // loops supported
constexpr int PFD = 1;        // filter taps loaded ahead per thread
constexpr int CTAS_PER_SM = 2;
constexpr unsigned NONE = 0x7fffffffu;

// columns per work item: one consumer thread per (column, loop)
inline int cols_per_item(int loops) { return 64 * loops + 64 <= 1024 ? 64 : 32; }

// taps per bucket in the bucket-major table: the w/B full-tile taps plus the
// partial one, rounded up to even so that every bucket's row is a multiple of
// 16 bytes (bulk copies)
__host__ __device__ inline int taps_per_bucket(int tiles) { return (tiles + 2) & ~1; }

struct HitTab {
  unsigned s[MAXL][MAXT];  // (row offset << 8) | j, sorted by row offset
  unsigned beta[MAXL];
  unsigned xrow[MAXL];     // (tiles * beta) mod nb: row offset of the partial tap
};

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// The signal streams through L2 once; marking its tiles evict-first keeps the
// (re-read) filter taps resident in L2 instead of being pushed out by it.
__device__ __forceinline__ unsigned long long policy_evict_first() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long policy_evict_last() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ void tma_load_tile(void *dst, const CUtensorMap *tm, int x0, int y0,
                                              unsigned long long *bar, unsigned bytes,
                                              unsigned long long pol) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x0), "r"(y0), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}

// one bucket's taps (bytes: a multiple of 16) into this thread's slot
__device__ __forceinline__ void bulk_load_taps(void *dst, const void *src, unsigned bytes,
                                               unsigned long long *bar, unsigned long long pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}

// read-only tap load that asks L2 to keep the line
__device__ __forceinline__ float2 ld_tap(const float2 *p, unsigned long long pol) {
  float2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
               : "=f"(v.x), "=f"(v.y)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ld_tap(const double2 *p, unsigned long long pol) {
  double2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
               : "=d"(v.x), "=d"(v.y)
               : "l"(p), "l"(pol));
  return v;
}

// Bounded wait on an mbarrier phase; false after ~0.5 s without completion.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
  return mbar_wait_bounded(smem_u32(bar), parity);
}

// Persistent, warp-specialised.  A work item is (block of CW columns, row
// group); CTA b takes items b, b + grid, ...  Warp roles:
//  * threads [0, CW*loops): consumers.  Thread (l, col) walks loop l of
//    column col, so each warp covers 32 columns of one loop; its taps come
//    from its shared-memory slot (staged form) or from the bucket-major tap
//    table one hit ahead, so the L2 reads overlap the stream.
//  * the next warp: producer.  One lane streams every tile of the CTA's
//    items, in order, into an NSTAGE ring (full[s]: tile landed, tx-counted;
//    empty[s]: every releasing warp is done with it).
//  * the last warp (RLFC loops only): copies the RLFC sub-samples out of
//    each tile.
// No block-wide barrier inside the stream.
template <typename T, int CW, int MAXTH, int NS, bool STG>
__global__ void __launch_bounds__(MAXTH, (MAXTH <= 640 && !STG) ? CTAS_PER_SM : 1)
pf_tma_kernel(const __grid_constant__ CUtensorMap tmap, const typename Cx<T>::V *__restrict__ filt,
              int logn, int logB, int w, int rt, int tiles, int rows_per_group, int groups, int L,
              Draws d, HitTab ht, typename Cx<T>::V *__restrict__ bins, int nrlfc, int logsig,
              typename Cx<T>::V *__restrict__ y, int W, int *err) {
  pdl_enter();
  typedef typename Cx<T>::V V;
  constexpr int LOGCW = CW == 64 ? 6 : 5;
  const int NCT = CW * L;  // consumer threads
  const int NCW = NCT / 32;
  const int NREL = NCW + (nrlfc > 0 ? 1 : 0);  // warps releasing each stage
  extern __shared__ __align__(128) unsigned char dsm[];
  // each loop's sorted list twice in a row, so a rotated walk needs no wrap
  __shared__ unsigned S2[MAXL][2 * MAXT];
  __shared__ unsigned s_a[MAXL], s_beta[MAXL], s_xrow[MAXL];
  __shared__ __align__(8) unsigned long long full[NS], empty[NS];
  __shared__ __align__(8) unsigned long long tapbar[STG ? MAXTH / 32 : 1];
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x;
  const int B = 1 << logB;
  const int lognb = logn - logB;
  const int nb = 1 << lognb;
  const unsigned nbm = (unsigned)nb - 1u;
  const unsigned nmask = (1u << logn) - 1u;
  const int TT = taps_per_bucket(tiles);  // row length of the bucket-major table
  const unsigned stage_bytes = (unsigned)(rt * CW * sizeof(V));
  const int ntile = rows_per_group / rt;
  const int ncb = B / CW;
  const int items = ncb * groups;
  const int xmul = (int)(sizeof(V) / 8);  // tensor elements are 8-byte words
  V *tile0 = reinterpret_cast<V *>(dsm);

  for (int e = tid; e < L * 2 * MAXT; e += blockDim.x) {
    const int l = e / (2 * MAXT), m = e % (2 * MAXT);
    S2[l][m] = m < tiles ? ht.s[l][m] : (m < 2 * tiles ? ht.s[l][m - tiles] : 0u);
  }
  if (tid < L) {
    s_a[tid] = (unsigned)d.a[tid];
    s_beta[tid] = ht.beta[tid];
    s_xrow[tid] = ht.xrow[tid];
  }
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < NS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NREL);
    }
    if (STG)
      for (int i = 0; i < NCW; i++) mbar_init(&tapbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const unsigned smask = (1u << logsig) - 1u;
  if (tid >= NCT + 32) {
    // ---------------- RLFC warp: loop r samples positions off_r + m*(n/W)
    // (restLocFreqCoeffKernel, innerLoop.cu:693-703); n/W divides B, so those
    // are whole columns, copied from the tile to y_r[t / (n/W)]
    if (nrlfc == 0) return;
    const int lane = tid & 31;
    long long k = 0;
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
      const int cb = it % ncb, g = it / ncb;
      const int c0 = cb * CW;
      for (int t = 0; t < ntile; t++, k++) {
        const int st = (int)(k % NS);
        const V *tl = tile0 + (size_t)st * rt * CW;
        if (!mbar_wait(&full[st], (unsigned)((k / NS) & 1))) {
          abort_flag = 1;
          atomicExch(err, 1);
          return;
        }
        const unsigned r0 = (unsigned)(g * rows_per_group + t * rt);
        for (int rr = 0; rr < nrlfc; rr++) {
          const unsigned off = (unsigned)d.offs[rr];
          const unsigned first = ((off - (unsigned)c0) & smask);  // first matching column
          if (first >= (unsigned)CW) continue;
          const int lognc = logsig >= LOGCW ? 0 : LOGCW - logsig;  // log2 of the column count
          for (int e = lane; e < (rt << lognc); e += 32) {
            const int row = e >> lognc, ci = e & ((1 << lognc) - 1);
            const unsigned cc = first + ((unsigned)ci << logsig);
            const unsigned tpos = ((r0 + row) << logB) + (unsigned)c0 + cc;
            y[(size_t)rr * W + ((tpos - off) >> logsig)] = tl[(row << LOGCW) + cc];
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
      }
    }
    return;
  }
  if (tid >= NCT) {
    // ---------------- producer
    if (tid == NCT) {
      const unsigned long long pol = policy_evict_first();
      long long k = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
        const int cb = it % ncb, g = it / ncb;
        for (int t = 0; t < ntile; t++, k++) {
          const int st = (int)(k % NS);
          if (!mbar_wait(&empty[st], (unsigned)((k / NS) & 1) ^ 1u) || abort_flag) {
            abort_flag = 1;
            ok = false;
            break;
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          tma_load_tile(reinterpret_cast<char *>(tile0) + (size_t)st * stage_bytes, &tmap,
                        cb * CW * xmul, g * rows_per_group + t * rt, &full[st], stage_bytes, pol);
        }
      }
      // stay until the last load of every stage has landed (bounded)
      for (long long j = k - NS < 0 ? 0 : k - NS; j < k; j++)
        if (!mbar_wait(&full[j % NS], (unsigned)((j / NS) & 1))) {
          atomicExch(err, 1);
          break;
        }
    }
    return;
  }

  // ---------------- consumers
  const int col = tid & (CW - 1), l = tid >> LOGCW, lane = tid & 31;
  const int residue = w & (B - 1);
  const unsigned a = s_a[l], beta = s_beta[l], xrow = s_xrow[l];
  const unsigned *S = S2[l];
  const unsigned long long keep = policy_evict_last();
  long long k = 0;
  // staged form: this thread's slot of TT taps after the tile ring, and its
  // warp's copy barrier
  V *const tslot = reinterpret_cast<V *>(dsm + (size_t)NS * stage_bytes) + (size_t)tid * TT;
  unsigned long long *const tbar = &tapbar[STG ? (tid >> 5) : 0];
  unsigned tap_phase = 0;
  for (int it = blockIdx.x; it < items; it += gridDim.x) {
    const int cb = it % ncb, g = it / ncb;
    const int c0 = cb * CW;
    const unsigned c = (unsigned)(c0 + col);
    const int rbeg = g * rows_per_group;
    // Walk state.  Rotated position k of the column's hit list is
    // doubled-list entry m = mw + k; its row is v + s - nb when m < tiles (the
    // entry wrapped past nb) and v + s otherwise.
    const unsigned prod = c * a;
    const int bl = (int)(prod & (unsigned)(B - 1));
    const unsigned q = (prod & nmask) >> logB;
    const unsigned sl = (0u - q * beta) & nbm;
    const V *fcol = filt + (size_t)bl * TT;  // the bucket's taps, contiguous
    if constexpr (STG) {
      // One bulk copy of the bucket's taps into this thread's slot per item,
      // completing on the warp's barrier.  At the first __syncwarp every lane
      // is past its last read of the previous taps and its wait on the
      // previous phase; the proxy fence orders those reads before the copy.
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive_expect(tbar, 32u * (unsigned)(TT * sizeof(V)));
      __syncwarp();
      bulk_load_taps(tslot, fcol, (unsigned)(TT * sizeof(V)), tbar, keep);
    }
    // mw: first sorted entry with v >= nb - s (binary search)
    int lo = 0, hi = tiles;
    const unsigned lim = (unsigned)nb - sl;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if ((S[mid] >> 8) < lim) lo = mid + 1;
      else hi = mid;
    }
    const int mw = lo;
    // first rotated position with row >= rbeg (binary search)
    lo = 0;
    hi = tiles;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      const int m = mw + mid;
      const unsigned row = (S[m] >> 8) + sl - (m < tiles ? (unsigned)nb : 0u);
      if (row < (unsigned)rbeg) lo = mid + 1;
      else hi = mid;
    }
    int mc = mw + lo;
    const int me = mw + tiles;
    unsigned nm = NONE, er = NONE, ent = 0;
    // taps of the next PFD hits, loaded ahead (the last entries of the
    // doubled list are valid indices, so loading past me is harmless)
    V fv[PFD];
    if constexpr (!STG) {
#pragma unroll
      for (int u = 0; u < PFD; u++)
        fv[u] = ld_tap(fcol + (S[min(mc + u, 2 * tiles - 1)] & 255u), keep);
    }
    V fe = mk((T)0, (T)0);
    if (mc < me) {
      ent = S[mc];
      nm = (ent >> 8) + sl - (mc < tiles ? (unsigned)nb : 0u);
    }
    if (bl < residue) {
      er = (xrow + sl) & nbm;
      if (er < (unsigned)rbeg) er = NONE;
      else if constexpr (!STG) fe = ld_tap(fcol + tiles, keep);
    }
    if constexpr (STG) {
      if (!mbar_wait(tbar, tap_phase)) {
        abort_flag = 1;
        atomicExch(err, 1);
        return;
      }
      tap_phase ^= 1u;
      if (er != NONE) fe = tslot[tiles];
    }
    T re = 0, im = 0;

    for (int t = 0; t < ntile; t++, k++) {
      const int st = (int)(k % NS);
      const V *tl = tile0 + (size_t)st * rt * CW;
      if (!mbar_wait(&full[st], (unsigned)((k / NS) & 1))) {
        abort_flag = 1;
        atomicExch(err, 1);
        return;
      }
      const unsigned r0 = (unsigned)(rbeg + t * rt), r1 = r0 + (unsigned)rt;
      // full-tile taps in ascending row order, then the partial tap if it
      // falls in this tile
      while (nm < r1) {
        const V xv = tl[((nm - r0) << LOGCW) + col];
        V f;
        if constexpr (STG) f = tslot[ent & 255u];
        else f = fv[0];
        re = fma(xv.x, f.x, re);
        re = fma(-xv.y, f.y, re);
        im = fma(xv.x, f.y, im);
        im = fma(xv.y, f.x, im);
        const int m = ++mc;
        if constexpr (STG) {
          nm = NONE;
          if (m < me) {
            ent = S[m];
            nm = (ent >> 8) + sl - (m < tiles ? (unsigned)nb : 0u);
          }
        } else {
#pragma unroll
          for (int u = 0; u + 1 < PFD; u++) fv[u] = fv[u + 1];
          fv[PFD - 1] = ld_tap(fcol + (S[min(m + PFD - 1, 2 * tiles - 1)] & 255u), keep);
          nm = m < me ? (S[m] >> 8) + sl - (m < tiles ? (unsigned)nb : 0u) : NONE;
        }
      }
      if (er < r1) {
        const V xv = tl[((er - r0) << LOGCW) + col];
        re = fma(xv.x, fe.x, re);
        re = fma(-xv.y, fe.y, re);
        im = fma(xv.x, fe.y, im);
        im = fma(xv.y, fe.x, im);
        er = NONE;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[st]);
    }
    // partial sums of this row group: bins[group][l][b]
    bins[((size_t)g * L + l) * B + bl] = mk(re, im);
  }
}

// Bucket-major copy of the taps: tb[b * TT + j] = filt[j * B + b] (0 past w).
template <typename V>
__global__ void bucket_major_kernel(const V *__restrict__ filt, int w, int B, int TT, V *tb) {
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i >= (long long)B * TT) return;
  const int b = (int)(i / TT), j = (int)(i % TT);
  const long long src = (long long)j * B + b;
  V v = filt[src < w ? src : 0];
  if (src >= w) v.x = v.y = 0;
  tb[i] = v;
}

template <typename V>
__global__ void sum_partials_kernel(const V *__restrict__ part, int groups, long long count, V *out) {
  pdl_enter();
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i >= count) return;
  V v = part[i];
  for (int g = 1; g < groups; g++) v = cadd(v, part[(long long)g * count + i]);
  out[i] = v;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // the driver's entry point is the same for every context; looked up once,
  // thread-safely (function-local static initialisation)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return nullptr;
  }();
  return fn;
}

int ilog2(long long v) {
  int l = 0;
  while ((1LL << l) < v) l++;
  return l;
}

unsigned inv_odd(unsigned a) {  // a^-1 mod 2^32 for odd a (Newton)
  unsigned x = a;
  for (int i = 0; i < 5; i++) x *= 2u - a * x;
  return x;
}

// dynamic shared memory of one CTA: the tile ring, plus the consumers' tap
// slots in the staged form
inline int pf_smem_bytes(int es, int cw, int rt, int loops, int tiles, int ns, bool stg) {
  return ns * rt * cw * es + (stg ? cw * loops * taps_per_bucket(tiles) * es : 0);
}
constexpr int PF_SMEM_LIMIT = 218 * 1024;  // dynamic bytes, leaving room for the static tables

template <typename T, int CW, int MAXTH, int NS, bool STG>
int launch_CW(const CUtensorMap &tm, const void *filt, int logn, int logB, int w, int rt, int tiles,
              int groups, int loops, const Draws &d, const HitTab &ht, void *bins, int nrlfc,
              int logsig, void *y, int W, int *err, cudaStream_t st) {
  typedef typename Cx<T>::V V;
  const int B = 1 << logB;
  const int smem = pf_smem_bytes((int)sizeof(V), CW, rt, loops, tiles, NS, STG);
  const int threads = CW * loops + (nrlfc > 0 ? 64 : 32);
  static PerContext<int> attr;  // the kernel's dynamic shared memory limit, per context
  GS_CHECK(attr.ensure_at_least(smem, [](int v) {
    if (cudaFuncSetAttribute(pf_tma_kernel<T, CW, MAXTH, NS, STG>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, v) == cudaSuccess)
      return (int)GSFFT_OK;
    set_last_error("pf_tma_kernel: %d bytes of shared memory refused: %s", v,
                   cudaGetErrorString(cudaGetLastError()));
    return (int)GSFFT_ERR_CUDA;
  }));
  int dev = 0, sms = 0, per_sm = 0;
  GS_CUDA(cudaGetDevice(&dev));
  GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pf_tma_kernel<T, CW, MAXTH, NS, STG>,
                                                        threads, smem));
  const int items = (B / CW) * groups;
  const int grid = std::max(1, std::min(items, std::max(per_sm, 1) * sms));
  const int rows_per_group = (1 << (logn - logB)) / groups;
  GS_CUDA(launch_pdl(pf_tma_kernel<T, CW, MAXTH, NS, STG>, dim3(grid), dim3(threads), smem, st, tm,
                     (const V *)filt, logn, logB, w, rt, tiles, rows_per_group, groups, loops, d, ht,
                     (V *)bins, nrlfc, logsig, (V *)y, W, err));
  return GSFFT_OK;
}

// FP32 reads the taps from a per-thread shared-memory copy (one bulk copy per
// work item) when the slots fit beside a ring of NSTAGE_STG tiles: a warp's
// scattered 8-byte tap loads from L2 touched 32 cache lines each and were the
// limit of the pass.
inline bool pf_stream_staged(int cw, int rt, int loops, int tiles) {
  return pf_smem_bytes(8, cw, rt, loops, tiles, NSTAGE_STG, true) <= PF_SMEM_LIMIT;
}
// The same form for 10 to 15 loops (up to 1024 threads): the slots take more
// room, so the ring keeps NSTAGE tiles.
inline bool pf_stream_staged_wide(int cw, int rt, int loops, int tiles) {
  return cw == 64 && 64 * loops + 64 <= 1024 &&
         pf_smem_bytes(8, cw, rt, loops, tiles, NSTAGE, true) <= PF_SMEM_LIMIT;
}

template <typename T>
int dispatch(int loops, const CUtensorMap &tm, const void *filt, int logn, int logB, int w, int rt,
             int tiles, int groups, const Draws &d, const HitTab &ht, void *bins, int nrlfc,
             int logsig, void *y, int W, int *err, cudaStream_t st) {
  const int cw = cols_per_item(loops);
  const bool small = cw * loops + (nrlfc > 0 ? 64 : 32) <= 640;
#define GO(CWV, MT, NSV, STGV)                                                                     \
  return launch_CW<T, CWV, MT, NSV, STGV>(tm, filt, logn, logB, w, rt, tiles, groups, loops, d, ht, \
                                          bins, nrlfc, logsig, y, W, err, st)
  if (cw == 64) {
    if (small) {
      if constexpr (sizeof(T) == 4)
        if (pf_stream_staged(cw, rt, loops, tiles)) GO(64, 640, NSTAGE_STG, true);
      GO(64, 640, NSTAGE, false);
    }
    if constexpr (sizeof(T) == 4)
      if (pf_stream_staged_wide(cw, rt, loops, tiles)) GO(64, 1024, NSTAGE, true);
    GO(64, 1024, NSTAGE, false);
  }
  if (small) GO(32, 640, NSTAGE, false);
  GO(32, 1024, NSTAGE, false);
#undef GO
}

}  // namespace

int stream_taps_count(int w, int B) { return B * taps_per_bucket(w / B); }

int launch_stream_taps(int precision, const void *filt, int w, int B, void *taps_bm,
                       cudaStream_t st) {
  const int TT = taps_per_bucket(w / B);
  const long long cnt = (long long)B * TT;
  const unsigned grid = (unsigned)((cnt + 255) / 256);
  if (precision == GSFFT_FP64)
    bucket_major_kernel<double2><<<grid, 256, 0, st>>>((const double2 *)filt, w, B, TT, (double2 *)taps_bm);
  else
    bucket_major_kernel<float2><<<grid, 256, 0, st>>>((const float2 *)filt, w, B, TT, (float2 *)taps_bm);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_sum_partials(int precision, const void *part, int groups, long long count, void *out,
                        cudaStream_t st) {
  const unsigned grid = (unsigned)((count + 255) / 256);
  if (precision == GSFFT_FP64)
    GS_CUDA(launch_pdl(sum_partials_kernel<double2>, dim3(grid), dim3(256), 0, st,
                       (const double2 *)part, groups, count, (double2 *)out));
  else
    GS_CUDA(launch_pdl(sum_partials_kernel<float2>, dim3(grid), dim3(256), 0, st,
                       (const float2 *)part, groups, count, (float2 *)out));
  GS_LAUNCHED();
  return GSFFT_OK;
}

bool stream_pf_supported(int n, int B, int loops, int W, int RLFC_loops) {
  if (loops < 2 || loops > MAXL || B < ST || (B % ST) != 0 || n / B < 2) return false;
  if (RLFC_loops > MAX_RLFC_LOOPS || (W > 0 && n / W > B)) return false;
  if (n / B > (1 << 23)) return false;  // row offsets must fit 24 bits
  return encode_fn() != nullptr;
}

static int stream_rows_per_tile(int n, int B, int precision) {
  return std::min(n / B, precision == GSFFT_FP64 ? 32 : 64);  // 32 KiB tiles of 64 columns
}

int stream_pf_groups(int n, int B, int w, int loops, int precision) {
  const int nb = n / B;
  const int rt = stream_rows_per_tile(n, B, precision);
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int cw = cols_per_item(loops);
  // the staged FP32 forms run one CTA per SM (the dispatch's choice)
  const bool stg = precision != GSFFT_FP64 && cw == 64 &&
                   (64 * loops + 64 <= 640 ? pf_stream_staged(cw, rt, loops, w / B)
                                           : pf_stream_staged_wide(cw, rt, loops, w / B));
  // enough work items (column block x row group) for ~6 per persistent CTA,
  // each item at least four tiles long
  const long long want = 6LL * (stg ? 1 : CTAS_PER_SM) * sms;
  int groups = 1;
  while ((long long)(B / cw) * groups < want && nb / (groups * 2) >= 4 * rt) groups *= 2;
  return groups;
}

bool stream_pf_groups_valid(int n, int B, int groups, int precision) {
  if (groups < 1 || (groups & (groups - 1))) return false;
  if (groups == 1) return true;
  const int nb = n / B;
  return nb / groups >= 4 * stream_rows_per_tile(n, B, precision) && nb % groups == 0;
}

int launch_perm_filter_stream(int precision, const void *x, int n, const void *filt, int w, int B,
                              int loops, const Draws &d, void *bins, int nrlfc, void *y, int W,
                              int *err, cudaStream_t st, int groups_req) {
  if (!stream_pf_supported(n, B, loops, W, nrlfc)) return GSFFT_ERR_UNSUPPORTED;
  const int tiles = w / B;
  if (tiles >= MAXT || tiles > 255) return GSFFT_ERR_UNSUPPORTED;
  const int logn = ilog2(n), logB = ilog2(B), logsig = ilog2(n / W);
  const int nb = n / B;
  const unsigned nbm = (unsigned)nb - 1u;
  // sorted hit rows of each loop: j * beta mod nb for j < tiles
  HitTab ht;
  memset(&ht, 0, sizeof(ht));
  std::vector<std::pair<unsigned, unsigned>> v(tiles);
  for (int l = 0; l < loops; l++) {
    const unsigned alpha = (unsigned)d.a[l] & nbm;
    const unsigned beta = inv_odd(alpha) & nbm;
    ht.beta[l] = beta;
    ht.xrow[l] = ((unsigned)tiles * beta) & nbm;
    for (int j = 0; j < tiles; j++) v[j] = {((unsigned)j * beta) & nbm, (unsigned)j};
    std::sort(v.begin(), v.end());
    for (int j = 0; j < tiles; j++) ht.s[l][j] = (v[j].first << 8) | v[j].second;
  }
  // x as a 2-D tensor of 8-byte words: nb rows of B (FP32) or 2B (FP64) words
  const bool dbl = precision == GSFFT_FP64;
  const int es = dbl ? 16 : 8;
  const int rt = stream_rows_per_tile(n, B, precision);
  int groups = stream_pf_groups(n, B, w, loops, precision);
  if (groups_req > 0) {
    if (!stream_pf_groups_valid(n, B, groups_req, precision)) return GSFFT_ERR_PARAM;
    groups = groups_req;
  }
  const int cw = cols_per_item(loops);
  CUtensorMap tm;
  const cuuint64_t gdim[2] = {(cuuint64_t)B * (es / 8), (cuuint64_t)nb};
  const cuuint64_t gstride[1] = {(cuuint64_t)B * es};
  const cuuint32_t box[2] = {(cuuint32_t)(cw * (es / 8)), (cuuint32_t)rt};
  const cuuint32_t estr[2] = {1, 1};
  CUresult cr = encode_fn()(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void *>(x), gdim,
                            gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_last_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return GSFFT_ERR_CUDA;
  }
  int s = dbl ? dispatch<double>(loops, tm, filt, logn, logB, w, rt, tiles, groups, d, ht, bins,
                                 nrlfc, logsig, y, W, err, st)
              : dispatch<float>(loops, tm, filt, logn, logB, w, rt, tiles, groups, d, ht, bins, nrlfc,
                                logsig, y, W, err, st);
  if (s != GSFFT_OK) return s;
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
