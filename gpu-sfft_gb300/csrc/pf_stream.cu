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
// s_l.  The host sorts that set once per run; each thread walks its rotated
// copy in ascending row order, so a thread touches only its own ~loops*w/B
// hits while the CTA streams every row of its 128 columns exactly once.
// Sums run in ascending row (= signal position) order: fixed, no atomics.
//
// Tiles of rt rows x 128 columns arrive by cp.async.bulk.tensor.2d into a
// three-stage shared-memory ring, each stage guarded by an mbarrier whose
// waits are bounded (a timeout sets an error flag instead of hanging).
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

constexpr int ST = 128;      // columns per CTA
constexpr int NSTAGE = 2;    // tiles in flight
constexpr int MAXT = 32;     // full tiles of taps per bucket (w / B) supported
constexpr int MAXL = 16;     // loops supported
constexpr unsigned NONE = 0x7fffffffu;

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

__device__ __forceinline__ void tma_load_tile(void *dst, const CUtensorMap *tm, int x0, int y0,
                                              unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x0), "r"(y0), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait on an mbarrier phase; false after ~0.5 s without completion.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
  const long long t0 = clock64();
  while (true) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > (1LL << 30)) return false;
  }
}

template <typename T, int L>
__global__ void __launch_bounds__(ST, 5)
pf_tma_kernel(const __grid_constant__ CUtensorMap tmap, const typename Cx<T>::V *__restrict__ filt,
              int logn, int logB, int w, int rt, int tiles, int rows_per_group, Draws d, HitTab ht,
              typename Cx<T>::V *__restrict__ bins, int nrlfc, int logsig,
              typename Cx<T>::V *__restrict__ y, int W, int *err) {
  typedef typename Cx<T>::V V;
  extern __shared__ __align__(128) unsigned char dsm[];
  // each loop's sorted list twice in a row, so a rotated walk needs no wrap
  __shared__ unsigned S2[L][2 * MAXT];
  __shared__ __align__(8) unsigned long long bar[NSTAGE];
  __shared__ int abort_flag;
  const int tid = threadIdx.x;
  const int B = 1 << logB;
  const int lognb = logn - logB;
  const int nb = 1 << lognb;
  const unsigned nbm = (unsigned)nb - 1u;
  const unsigned nmask = (1u << logn) - 1u;
  const int c0 = blockIdx.x * ST;
  const unsigned c = (unsigned)(c0 + tid);
  const unsigned stage_bytes = (unsigned)(rt * ST * sizeof(V));
  const int rbeg = blockIdx.y * rows_per_group;  // this CTA's rows: [rbeg, rbeg + rows_per_group)
  const int ntile = rows_per_group / rt;
  const int xmul = (int)(sizeof(V) / 8);  // tensor elements are 8-byte words
  V *tile0 = reinterpret_cast<V *>(dsm);

  for (int e = tid; e < L * 2 * MAXT; e += ST) {
    const int l = e / (2 * MAXT), m = e % (2 * MAXT);
    S2[l][m] = m < tiles ? ht.s[l][m] : (m < 2 * tiles ? ht.s[l][m - tiles] : 0u);
  }
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < NSTAGE; s++) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0)
    for (int t = 0; t < NSTAGE && t < ntile; t++)
      tma_load_tile(reinterpret_cast<char *>(tile0) + (size_t)t * stage_bytes, &tmap, c0 * xmul,
                    rbeg + t * rt, &bar[t], stage_bytes);

  // Walk state per loop.  Rotated position k of the column's hit list is
  // doubled-list entry m = mw + k; its row is v + s - nb when m < tiles (the
  // entry wrapped past nb) and v + s otherwise.
  const int residue = w & (B - 1);
  int bl[L], mc[L], me[L];
  unsigned sl[L], nm[L], er[L];
  T re[L], im[L];
#pragma unroll
  for (int l = 0; l < L; l++) {
    const unsigned a = (unsigned)d.a[l];
    const unsigned prod = c * a;
    bl[l] = (int)(prod & (unsigned)(B - 1));
    const unsigned q = (prod & nmask) >> logB;
    sl[l] = (0u - q * ht.beta[l]) & nbm;
    // mw: first sorted entry with v >= nb - s (binary search)
    int lo = 0, hi = tiles;
    const unsigned lim = (unsigned)nb - sl[l];
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if ((S2[l][mid] >> 8) < lim) lo = mid + 1;
      else hi = mid;
    }
    const int mw = lo;
    // first rotated position with row >= rbeg (binary search)
    lo = 0;
    hi = tiles;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      const int m = mw + mid;
      const unsigned row = (S2[l][m] >> 8) + sl[l] - (m < tiles ? (unsigned)nb : 0u);
      if (row < (unsigned)rbeg) lo = mid + 1;
      else hi = mid;
    }
    mc[l] = mw + lo;
    me[l] = mw + tiles;
    nm[l] = mc[l] < me[l] ? (S2[l][mc[l]] >> 8) + sl[l] - (mc[l] < tiles ? (unsigned)nb : 0u) : NONE;
    er[l] = bl[l] < residue ? ((ht.xrow[l] + sl[l]) & nbm) : NONE;
    if (er[l] < (unsigned)rbeg) er[l] = NONE;
    re[l] = 0;
    im[l] = 0;
  }

  const unsigned smask = (1u << logsig) - 1u;
  for (int t = 0; t < ntile; t++) {
    const int st = t % NSTAGE;
    const V *tl = tile0 + (size_t)st * rt * ST;
    if (tid == 0 && !mbar_wait(&bar[st], (unsigned)(t / NSTAGE) & 1u)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) break;
    const unsigned r0 = (unsigned)(rbeg + t * rt), r1 = r0 + (unsigned)rt;
    // Loop-major: each lane adds loop l's hits of its column inside the tile
    // (full-tile taps in ascending row order, then the partial tap if it falls
    // in this tile).
#pragma unroll
    for (int l = 0; l < L; l++) {
      while (nm[l] < r1) {
        const unsigned ent = S2[l][mc[l]];
        const V xv = tl[(nm[l] - r0) * ST + tid];
        const V f = __ldg(&filt[((size_t)(ent & 255u) << logB) + bl[l]]);
        re[l] = fma(xv.x, f.x, re[l]);
        re[l] = fma(-xv.y, f.y, re[l]);
        im[l] = fma(xv.x, f.y, im[l]);
        im[l] = fma(xv.y, f.x, im[l]);
        const int m = ++mc[l];
        nm[l] = m < me[l] ? (S2[l][m] >> 8) + sl[l] - (m < tiles ? (unsigned)nb : 0u) : NONE;
      }
      if (er[l] < r1) {
        const V xv = tl[(er[l] - r0) * ST + tid];
        const V f = __ldg(&filt[((size_t)tiles << logB) + bl[l]]);
        re[l] = fma(xv.x, f.x, re[l]);
        re[l] = fma(-xv.y, f.y, re[l]);
        im[l] = fma(xv.x, f.y, im[l]);
        im[l] = fma(xv.y, f.x, im[l]);
        er[l] = NONE;
      }
    }
    // RLFC sub-samples held by this tile: columns c == off (mod n/W); with
    // n/W <= 128 there are 128 >> logsig of them, else at most one
    for (int rr = 0; rr < nrlfc; rr++) {
      const unsigned off = (unsigned)d.offs[rr];
      const unsigned first = ((off - (unsigned)c0) & smask);  // first matching column index
      if (first >= (unsigned)ST) continue;
      const int lognc = logsig >= 7 ? 0 : 7 - logsig;         // log2 of the column count
      for (int e = tid; e < (rt << lognc); e += ST) {
        const int row = e >> lognc, ci = e & ((1 << lognc) - 1);
        const unsigned cc = first + ((unsigned)ci << logsig);
        const unsigned tpos = ((r0 + row) << logB) + (unsigned)c0 + cc;
        y[(size_t)rr * W + ((tpos - off) >> logsig)] = tl[row * ST + cc];
      }
    }
    __syncthreads();  // every thread is done with stage st
    if (tid == 0 && t + NSTAGE < ntile) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tma_load_tile(reinterpret_cast<char *>(tile0) + (size_t)st * stage_bytes, &tmap, c0 * xmul,
                    rbeg + (t + NSTAGE) * rt, &bar[st], stage_bytes);
    }
  }
  if (abort_flag) {
    // drain: wait (bounded) for any copy still in flight into this CTA
    if (tid == 0) {
      for (int s = 0; s < NSTAGE; s++) (void)mbar_wait(&bar[s], 0);
      atomicExch(err, 1);
    }
    return;
  }
  // partial sums of this row group: bins[group][l][b]
  V *part = bins + (size_t)blockIdx.y * L * B;
#pragma unroll
  for (int l = 0; l < L; l++) part[(size_t)l * B + bl[l]] = mk(re[l], im[l]);
}

template <typename V>
__global__ void sum_partials_kernel(const V *__restrict__ part, int groups, long long count, V *out) {
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i >= count) return;
  V v = part[i];
  for (int g = 1; g < groups; g++) v = cadd(v, part[(long long)g * count + i]);
  out[i] = v;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
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

template <typename T, int L>
int launch_L(const CUtensorMap &tm, const void *filt, int logn, int logB, int w, int rt, int tiles,
             int groups, const Draws &d, const HitTab &ht, void *bins, int nrlfc, int logsig, void *y,
             int W, int *err, cudaStream_t st) {
  typedef typename Cx<T>::V V;
  const int B = 1 << logB;
  const int smem = NSTAGE * rt * ST * (int)sizeof(V);
  static bool attr = false;
  if (!attr) {
    GS_CUDA(cudaFuncSetAttribute(pf_tma_kernel<T, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem));
    attr = true;
  }
  const int rows_per_group = (1 << (logn - logB)) / groups;
  pf_tma_kernel<T, L><<<dim3(B / ST, groups), ST, smem, st>>>(tm, (const V *)filt, logn, logB, w, rt,
                                                              tiles, rows_per_group, d, ht, (V *)bins,
                                                              nrlfc, logsig, (V *)y, W, err);
  return GSFFT_OK;
}

template <typename T>
int dispatch(int loops, const CUtensorMap &tm, const void *filt, int logn, int logB, int w, int rt,
             int tiles, int groups, const Draws &d, const HitTab &ht, void *bins, int nrlfc,
             int logsig, void *y, int W, int *err, cudaStream_t st) {
  switch (loops) {
#define C(LL) \
  case LL: return launch_L<T, LL>(tm, filt, logn, logB, w, rt, tiles, groups, d, ht, bins, nrlfc, logsig, y, W, err, st);
    C(2) C(3) C(4) C(5) C(6) C(7) C(8) C(9) C(10) C(11) C(12) C(13) C(14) C(15) C(16)
#undef C
    default: return GSFFT_ERR_UNSUPPORTED;
  }
}

}  // namespace

int launch_sum_partials(int precision, const void *part, int groups, long long count, void *out,
                        cudaStream_t st) {
  const unsigned grid = (unsigned)((count + 255) / 256);
  if (precision == GSFFT_FP64)
    sum_partials_kernel<double2><<<grid, 256, 0, st>>>((const double2 *)part, groups, count,
                                                       (double2 *)out);
  else
    sum_partials_kernel<float2><<<grid, 256, 0, st>>>((const float2 *)part, groups, count,
                                                      (float2 *)out);
  GS_LAUNCHED();
  return GSFFT_OK;
}

bool stream_pf_supported(int n, int B, int loops, int W, int RLFC_loops) {
  if (loops < 2 || loops > MAXL || B < ST || (B % ST) != 0 || n / B < 2) return false;
  if (RLFC_loops > MAX_RLFC_LOOPS || (W > 0 && n / W > B)) return false;
  if (n / B > (1 << 23)) return false;  // row offsets must fit 24 bits
  return encode_fn() != nullptr;
}

int stream_pf_groups(int n, int B, int precision) {
  const int nb = n / B;
  const int rt = std::min(nb, precision == GSFFT_FP64 ? 8 : 16);
  // at least ~2400 CTAs (several waves of ~5 resident CTAs on 152 SMs), each
  // group at least one tile
  int groups = 1;
  while ((long long)(B / ST) * groups < 1500 && nb / (groups * 2) >= rt) groups *= 2;
  return groups;
}

int launch_perm_filter_stream(int precision, const void *x, int n, const void *filt, int w, int B,
                              int loops, const Draws &d, void *bins, int nrlfc, void *y, int W,
                              int *err, cudaStream_t st) {
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
  const int rt = std::min(nb, dbl ? 8 : 16);
  const int groups = stream_pf_groups(n, B, precision);
  CUtensorMap tm;
  const cuuint64_t gdim[2] = {(cuuint64_t)B * (es / 8), (cuuint64_t)nb};
  const cuuint64_t gstride[1] = {(cuuint64_t)B * es};
  const cuuint32_t box[2] = {(cuuint32_t)(ST * (es / 8)), (cuuint32_t)rt};
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
