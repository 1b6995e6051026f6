// A8: per-candidate value estimate (estimate_values, innerLoop.cu:396-466;
// estimateValuesKernel, :825-870) and the A9 gather of the top-k nodes.
//
// The reference allocates two arrays with device malloc in every thread and
// insertion-sorts them; here each thread keeps its loops' values in local
// arrays and picks the median by rank.  For loop j:
//   p = ai_j * loc mod n, h = p / (n/B), d = p mod (n/B);
//   if d > (n/B)/2 then h = (h + 1) mod B, d -= n/B;          (innerLoop.cu:838-845)
//   v_j = bins_j[h] * conj(H[(n - d) mod n]) / |H[(n - d) mod n]|^2
// The reciprocal response conj(H)/|H|^2 is precomputed in FP64 for the n/B + 1
// offsets d the formula can produce, so the estimate is one complex multiply
// in FP64 per loop.  The median of the real parts and of the imaginary parts
// is taken separately, element (loops-1)/2 of the ascending order
// (:855-861).  In the mixed path (FP32 bins) the ranking runs in FP32 and only
// the two median estimates are computed in FP64 (estimate_dev.cuh).
// mag2 receives the top-k keys |estimate|^2: doubles in the FP64 path, floats
// (in the same buffer) in the mixed path, whose top-k selects on 4-byte keys.
#include "estimate_dev.cuh"

namespace gsfft {

namespace {

constexpr int ET = 128;

template <typename T, int L>
__global__ void __launch_bounds__(ET)
estimate_kernel_fixed(const int *__restrict__ cand, const RunCtl *ctl, int cap,
                      const typename Cx<T>::V *__restrict__ bins, unsigned nmask, int lognb, int B,
                      Draws d, const double2 *__restrict__ hinv, DevNode *nodes, double *mag2) {
  pdl_enter();
  estimate_block<T, L>(cand, ctl, cap, bins, nmask, lognb, B, d, hinv, nodes, mag2, (int)blockIdx.x,
                       (int)gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(ET)
estimate_kernel(const int *__restrict__ cand, const RunCtl *ctl, int cap,
                const typename Cx<T>::V *__restrict__ bins, int loops, unsigned nmask, int lognb,
                int B, Draws d, const double2 *__restrict__ hinv, DevNode *nodes, double *mag2) {
  pdl_enter();
  const int i = blockIdx.x * ET + threadIdx.x;
  const int count = min(ctl->cand_count, cap);
  if (i >= count) return;
  const unsigned loc = (unsigned)cand[i];
  const int nb = 1 << lognb;
  double vr[MAX_LOOPS], vi[MAX_LOOPS];
  for (int j = 0; j < loops; j++) {
    const unsigned p = ((unsigned)d.ai[j] * loc) & nmask;
    int h = (int)(p >> lognb);
    int dd = (int)(p & (unsigned)(nb - 1));
    if (dd > nb / 2) {
      h = (h + 1) & (B - 1);
      dd -= nb;
    }
    const double2 H = hinv[dd + nb / 2];
    const typename Cx<T>::V bv = bins[(size_t)j * B + h];
    const double bx = (double)bv.x, by = (double)bv.y;
    vr[j] = fma(bx, H.x, -(by * H.y));
    vi[j] = fma(bx, H.y, by * H.x);
  }
  const double re = median_of(vr, loops), im = median_of(vi, loops);
  DevNode nd;
  nd.key = loc;
  nd.pad = 0;
  nd.x = re;
  nd.y = im;
  nodes[i] = nd;
  if constexpr (sizeof(T) == 4) {
    const float fre = (float)re, fim = (float)im;  // the mixed path's 4-byte top-k key
    reinterpret_cast<float *>(mag2)[i] = __fadd_rn(__fmul_rn(fre, fre), __fmul_rn(fim, fim));
  } else {
    mag2[i] = __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
  }
}

__global__ void gather_nodes_kernel(const DevNode *__restrict__ nodes, const int *__restrict__ idx,
                                    const int *count, int cap, DevNode *out) {
  pdl_enter();
  const int k = blockIdx.x * 256 + threadIdx.x;
  if (k < min(*count, cap)) out[k] = nodes[idx[k]];
}

}  // namespace

int launch_estimate(int precision, const int *cand, const RunCtl *ctl, int cap, int expect,
                    const void *bins, int loops, int n, int B, const Draws &d, const double2 *hinv,
                    DevNode *nodes, double *mag2, cudaStream_t st) {
  int lognb = 0;
  while ((1 << lognb) < n / B) lognb++;
  const unsigned nmask = (unsigned)n - 1u;
  if (loops >= 2 && loops <= 16) {
    // sized for `expect` candidates; the grid-stride loop takes up to `cap`
    const int grid = max(1, min((min(expect, cap) + ET - 1) / ET, 152 * 8));
#define EST_CASE(LL)                                                                              \
  case LL:                                                                                        \
    if (precision == GSFFT_FP64)                                                                  \
      GS_CUDA(launch_pdl(estimate_kernel_fixed<double, LL>, dim3(grid), dim3(ET), 0, st, cand, ctl, \
                         cap, (const double2 *)bins, nmask, lognb, B, d, hinv, nodes, mag2));       \
    else                                                                                          \
      GS_CUDA(launch_pdl(estimate_kernel_fixed<float, LL>, dim3(grid), dim3(ET), 0, st, cand, ctl,  \
                         cap, (const float2 *)bins, nmask, lognb, B, d, hinv, nodes, mag2));        \
    break;
    switch (loops) {
      EST_CASE(2) EST_CASE(3) EST_CASE(4) EST_CASE(5) EST_CASE(6) EST_CASE(7) EST_CASE(8)
      EST_CASE(9) EST_CASE(10) EST_CASE(11) EST_CASE(12) EST_CASE(13) EST_CASE(14) EST_CASE(15)
      EST_CASE(16)
      default: break;
    }
#undef EST_CASE
    GS_LAUNCHED();
    return GSFFT_OK;
  }
  const int grid = (cap + ET - 1) / ET;
  if (precision == GSFFT_FP64)
    estimate_kernel<double><<<grid, ET, 0, st>>>(cand, ctl, cap, (const double2 *)bins, loops,
                                                 nmask, lognb, B, d, hinv, nodes, mag2);
  else
    estimate_kernel<float><<<grid, ET, 0, st>>>(cand, ctl, cap, (const float2 *)bins, loops, nmask,
                                                lognb, B, d, hinv, nodes, mag2);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_gather_nodes(const DevNode *nodes, const int *idx, const int *count, int cap,
                        DevNode *out, cudaStream_t st) {
  GS_CUDA(launch_pdl(gather_nodes_kernel, dim3((cap + 255) / 256), dim3(256), 0, st, nodes, idx, count,
                     cap, out));
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
