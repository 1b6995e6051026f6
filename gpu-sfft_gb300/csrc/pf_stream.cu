// A5 + the RLFC sub-sampling of A4 in one streaming pass over the signal.
//
// The gather form (pf.cu) reads each tap's sample at a random address; at the
// n = 2^27 sizes every such read costs a full DRAM burst (~64-96 bytes for an
// 8-byte sample).  When loops * w random reads cost more than reading the
// whole signal once, this kernel reads x exactly once, in order:
//
// View x as an (n/B) x B matrix, x[r*B + c].  For loop l the tap of position
// t = r*B + c is i = t*a_l mod n (t = i*ai_l mod n, innerLoop.cu:738,769), and
//   i = B * ((q_l + r*alpha_l) mod (n/B)) + b_l,
//   b_l = (c*a_l) mod B,  q_l = ((c*a_l) mod n) / B,  alpha_l = a_l mod (n/B).
// So every tap of column c belongs to the single bucket b_l, and c -> b_l is
// a bijection (a_l odd).  One thread per column walks its rows in order,
// keeps j = (q_l + r*alpha_l) mod (n/B) for each loop, and accumulates
// x[t] * filt[j*B + b_l] whenever j*B + b_l < w -- no atomics, fixed order.
// j lives in the top bits of a 32-bit word so the mod (n/B) is the wrap.
//
// RLFC loop r samples positions off_r + m*(n/W) (restLocFreqCoeffKernel,
// innerLoop.cu:693-703); (n/W) divides B, so they are exactly the columns
// c = off_r mod (n/W) -- those threads also copy x[t] to y_r[t / (n/W)].
#include "stages.cuh"

namespace gsfft {

namespace {

constexpr int ST = 128;  // columns per block
constexpr int U = 8;     // rows loaded ahead per thread

template <typename T, int L>
__global__ void __launch_bounds__(ST)
pf_stream_kernel(const typename Cx<T>::V *__restrict__ x, int logn, int logB,
                 const typename Cx<T>::V *__restrict__ filt, int w, Draws d,
                 typename Cx<T>::V *__restrict__ bins, int nrlfc, int logsig,
                 typename Cx<T>::V *__restrict__ y, int W) {
  typedef typename Cx<T>::V V;
  const unsigned c = blockIdx.x * ST + threadIdx.x;
  const int B = 1 << logB;
  const int lognb = logn - logB;
  const int nb = 1 << lognb;
  const int sh = 32 - lognb;  // j is kept as j << sh
  const unsigned nmask = (1u << logn) - 1u;
  const int tiles = w >> logB, residue = w & (B - 1);
  unsigned js[L], as[L], tl[L];
  int bl[L];
  T re[L], im[L];
#pragma unroll
  for (int l = 0; l < L; l++) {
    const unsigned a = (unsigned)d.a[l];
    const unsigned prod = c * a;
    bl[l] = (int)(prod & (unsigned)(B - 1));
    const unsigned q = (prod & nmask) >> logB;
    js[l] = lognb ? (q << sh) : 0u;
    as[l] = lognb ? ((a & (unsigned)(nb - 1)) << sh) : 0u;
    const unsigned long long nt = (unsigned long long)(tiles + (bl[l] < residue ? 1 : 0)) << sh;
    tl[l] = nt > 0xffffffffull ? 0xffffffffu : (unsigned)nt;
    re[l] = 0;
    im[l] = 0;
  }
  // RLFC loops that sample this column
  const unsigned smask = (1u << logsig) - 1u;
  unsigned rl = 0;
  for (int rr = 0; rr < nrlfc; rr++)
    if ((c & smask) == (unsigned)d.offs[rr]) rl |= 1u << rr;
  const V *__restrict__ xc = x + c;
  for (int r0 = 0; r0 < nb; r0 += U) {
    V xv[U];
#pragma unroll
    for (int u = 0; u < U; u++) xv[u] = (r0 + u < nb) ? xc[(size_t)(r0 + u) << logB] : mk((T)0, (T)0);
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (r0 + u >= nb) break;
#pragma unroll
      for (int l = 0; l < L; l++) {
        if (js[l] < tl[l]) {
          const unsigned i = ((js[l] >> sh) << logB) + (unsigned)bl[l];
          const V f = __ldg(&filt[i]);
          re[l] = fma(xv[u].x, f.x, re[l]);
          re[l] = fma(-xv[u].y, f.y, re[l]);
          im[l] = fma(xv[u].x, f.y, im[l]);
          im[l] = fma(xv[u].y, f.x, im[l]);
        }
        js[l] += as[l];
      }
      if (rl) {
        const unsigned t = ((unsigned)(r0 + u) << logB) + c;
        for (int rr = 0; rr < nrlfc; rr++)
          if (rl & (1u << rr)) y[(size_t)rr * W + ((t - (unsigned)d.offs[rr]) >> logsig)] = xv[u];
      }
    }
  }
#pragma unroll
  for (int l = 0; l < L; l++) bins[(size_t)l * B + bl[l]] = mk(re[l], im[l]);
}

template <typename T, int L>
void launch_L(const void *x, int logn, int logB, const void *filt, int w, const Draws &d, void *bins,
              int nrlfc, int logsig, void *y, int W, cudaStream_t st) {
  typedef typename Cx<T>::V V;
  const int B = 1 << logB;
  pf_stream_kernel<T, L><<<B / ST, ST, 0, st>>>((const V *)x, logn, logB, (const V *)filt, w, d,
                                                 (V *)bins, nrlfc, logsig, (V *)y, W);
}

template <typename T>
int dispatch(int loops, const void *x, int logn, int logB, const void *filt, int w, const Draws &d,
             void *bins, int nrlfc, int logsig, void *y, int W, cudaStream_t st) {
  switch (loops) {
#define C(LL) \
  case LL: launch_L<T, LL>(x, logn, logB, filt, w, d, bins, nrlfc, logsig, y, W, st); break;
    C(2) C(3) C(4) C(5) C(6) C(7) C(8) C(9) C(10) C(11) C(12) C(13) C(14) C(15) C(16)
#undef C
    default: return GSFFT_ERR_UNSUPPORTED;
  }
  return GSFFT_OK;
}

int ilog2(long long v) {
  int l = 0;
  while ((1LL << l) < v) l++;
  return l;
}

}  // namespace

bool stream_pf_supported(int n, int B, int loops, int W, int RLFC_loops) {
  return loops >= 2 && loops <= 16 && B >= ST && (B % ST) == 0 && n / B >= 2 &&
         RLFC_loops <= MAX_RLFC_LOOPS && (n / W) <= B && RLFC_loops <= 32;
}

int launch_perm_filter_stream(int precision, const void *x, int n, const void *filt, int w, int B,
                              int loops, const Draws &d, void *bins, int nrlfc, void *y, int W,
                              cudaStream_t st) {
  if (!stream_pf_supported(n, B, loops, W, nrlfc)) return GSFFT_ERR_UNSUPPORTED;
  const int logn = ilog2(n), logB = ilog2(B), logsig = ilog2(n / W);
  int s = precision == GSFFT_FP64
              ? dispatch<double>(loops, x, logn, logB, filt, w, d, bins, nrlfc, logsig, y, W, st)
              : dispatch<float>(loops, x, logn, logB, filt, w, d, bins, nrlfc, logsig, y, W, st);
  if (s != GSFFT_OK) return s;
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
