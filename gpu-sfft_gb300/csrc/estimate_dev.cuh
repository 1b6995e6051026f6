// Device code of the estimation stage (A8), shared by the per-plan kernels
// (estimate.cu) and the persistent batch-tail kernel (batch_tail.cu).  The
// candidate list and count may have been written by another block of the
// same launch, so they are read past L1 (ld.global.cg).
#pragma once
#include "stages.cuh"

namespace gsfft {

namespace {

// Order-preserving integer key of a double (finite values): comparing keys
// as unsigned integers orders the values, so the ranking below runs on the
// integer pipe instead of GB300's narrow FP64 pipe.  (-0.0 ranks just below
// +0.0; both are the same value.)
__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Element (L-1)/2 of the ascending order (ties by index), by rank counting.
__device__ __forceinline__ double median_of(const double *v, int L) {
  const int want = (L - 1) / 2;
  double res = v[0];
  for (int i = 0; i < L; i++) {
    const unsigned long long ki = dkey(v[i]);
    int rank = 0;
    for (int j = 0; j < L; j++) {
      const unsigned long long kj = dkey(v[j]);
      rank += (kj < ki) || (kj == ki && j < i);
    }
    if (rank == want) res = v[i];
  }
  return res;
}

// Compile-time loop count: the per-loop values and keys live in registers.
template <int L>
__device__ __forceinline__ double median_reg(const double (&v)[L]) {
  constexpr int want = (L - 1) / 2;
  unsigned long long k[L];
#pragma unroll
  for (int i = 0; i < L; i++) k[i] = dkey(v[i]);
  double res = v[0];
#pragma unroll
  for (int i = 0; i < L; i++) {
    int rank = 0;
#pragma unroll
    for (int j = 0; j < L; j++) rank += (k[j] < k[i]) || (k[j] == k[i] && j < i);
    if (rank == want) res = v[i];
  }
  return res;
}

// Order-preserving integer key of a float, and the index of element (L-1)/2
// of the ascending order (ties by index) of L floats.
__device__ __forceinline__ unsigned fkey(float x) {
  const unsigned b = __float_as_uint(x);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
template <int L>
__device__ __forceinline__ int median_idx_f(const float (&v)[L]) {
  constexpr int want = (L - 1) / 2;
  unsigned k[L];
#pragma unroll
  for (int i = 0; i < L; i++) k[i] = fkey(v[i]);
  int res = 0;
#pragma unroll
  for (int i = 0; i < L; i++) {
    int rank = 0;
#pragma unroll
    for (int j = 0; j < L; j++) rank += (k[j] < k[i]) || (k[j] == k[i] && j < i);
    if (rank == want) res = i;
  }
  return res;
}

// Estimates of candidates bid * blockDim.x + threadIdx.x, then every
// nblk * blockDim.x further (a grid-stride loop over nblk blocks).
//
// FP64 bins: every loop's estimate in FP64, the medians ranked in FP64.
// FP32 bins (mixed path): the loops' estimates are ranked in FP32 (from the
// float copy of the reciprocal response that follows hinv) to find the loops
// whose real and imaginary parts are the medians, and only those two
// estimates are computed in FP64 -- GB300's FP64 rate is low, and the ranking
// needs no more than the FP32 bins carry.  Estimates closer than FP32
// rounding may rank the other way round, which moves the result by at most
// that rounding.
template <typename T, int L>
__device__ __forceinline__ void estimate_block(const int *__restrict__ cand, const RunCtl *ctl,
                                               int cap, const typename Cx<T>::V *__restrict__ bins,
                                               unsigned nmask, int lognb, int B, const Draws &d,
                                               const double2 *__restrict__ hinv, DevNode *nodes,
                                               double *mag2, int bid, int nblk) {
  const int count = min(__ldcg(&ctl->cand_count), cap);
  const int nb = 1 << lognb;
  const int nt = (int)blockDim.x;
  if constexpr (sizeof(T) == 4) {
    const float2 *__restrict__ hinv_f = reinterpret_cast<const float2 *>(hinv + nb + 1);
    for (int i = bid * nt + threadIdx.x; i < count; i += nblk * nt) {
      const unsigned loc = (unsigned)__ldcg(&cand[i]);
      float fr[L], fi[L], bxs[L], bys[L];
      int ds[L];
#pragma unroll
      for (int j = 0; j < L; j++) {
        const unsigned p = ((unsigned)d.ai[j] * loc) & nmask;
        int h = (int)(p >> lognb);
        int dd = (int)(p & (unsigned)(nb - 1));
        if (dd > nb / 2) {
          h = (h + 1) & (B - 1);
          dd -= nb;
        }
        const float2 Hf = __ldg(&hinv_f[dd + nb / 2]);
        const typename Cx<T>::V bv = bins[(size_t)j * B + h];
        bxs[j] = bv.x;
        bys[j] = bv.y;
        ds[j] = dd;
        fr[j] = fmaf(bv.x, Hf.x, -(bv.y * Hf.y));
        fi[j] = fmaf(bv.x, Hf.y, bv.y * Hf.x);
      }
      const int jr = median_idx_f<L>(fr), ji = median_idx_f<L>(fi);
      float bxr = 0.f, byr = 0.f, bxi = 0.f, byi = 0.f;
      int dr = 0, di = 0;
#pragma unroll
      for (int j = 0; j < L; j++) {
        if (j == jr) {
          bxr = bxs[j];
          byr = bys[j];
          dr = ds[j];
        }
        if (j == ji) {
          bxi = bxs[j];
          byi = bys[j];
          di = ds[j];
        }
      }
      const double2 Hr = __ldg(&hinv[dr + nb / 2]), Hi = __ldg(&hinv[di + nb / 2]);
      const double re = fma((double)bxr, Hr.x, -((double)byr * Hr.y));
      const double im = fma((double)bxi, Hi.y, (double)byi * Hi.x);
      DevNode nd;
      nd.key = loc;
      nd.pad = 0;
      nd.x = re;
      nd.y = im;
      nodes[i] = nd;
      // the top-k key: |estimate|^2 in FP32 (the mixed path selects on 4-byte keys)
      const float fre = (float)re, fim = (float)im;
      reinterpret_cast<float *>(mag2)[i] = __fadd_rn(__fmul_rn(fre, fre), __fmul_rn(fim, fim));
    }
  } else {
    for (int i = bid * nt + threadIdx.x; i < count; i += nblk * nt) {
      const unsigned loc = (unsigned)__ldcg(&cand[i]);
      double vr[L], vi[L];
#pragma unroll
      for (int j = 0; j < L; j++) {
        const unsigned p = ((unsigned)d.ai[j] * loc) & nmask;
        int h = (int)(p >> lognb);
        int dd = (int)(p & (unsigned)(nb - 1));
        if (dd > nb / 2) {
          h = (h + 1) & (B - 1);
          dd -= nb;
        }
        const double2 H = __ldg(&hinv[dd + nb / 2]);
        const typename Cx<T>::V bv = bins[(size_t)j * B + h];
        const double bx = (double)bv.x, by = (double)bv.y;
        vr[j] = fma(bx, H.x, -(by * H.y));
        vi[j] = fma(bx, H.y, by * H.x);
      }
      const double re = median_reg<L>(vr), im = median_reg<L>(vi);
      DevNode nd;
      nd.key = loc;
      nd.pad = 0;
      nd.x = re;
      nd.y = im;
      nodes[i] = nd;
      mag2[i] = __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
    }
  }
}

}  // namespace

}  // namespace gsfft
