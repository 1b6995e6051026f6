// A5: fused permutation + flat-window filter + folding into B buckets, every
// loop of the outer loop in one launch.
//
// Reference: perm_filter_cutoff (innerLoop.cu:194-240) launching
// permFilterTillKernel (n < 2^27, :725-757) or permFilterKernel (:761-773) once
// per loop, both with unsynchronised read-modify-writes of shared buckets.
//
// Here one thread owns bucket b and sums its taps id = b + j*B (j ascending)
// for up to LCH loops at a time, so no two threads touch the same bucket and
// the summation order is fixed (bit-identical run to run):
//   re = fma(xr, fr, re); re = fma(-xi, fi, re); im = fma(xr, fi, im); im = fma(xi, fr, im)
// The permuted index (id * ai) mod n is exact: the 32-bit product wraps mod
// 2^32 and n divides 2^32.  Each tap is read once per LCH loops (coalesced:
// consecutive threads read consecutive taps); the signal gathers are random,
// one 32-byte sector each, with LCH * 2 independent loads in flight per thread.
#include "stages.cuh"

namespace gsfft {

namespace {

constexpr int PF_THREADS = 128;
constexpr int LCH = 8;

template <typename T>
__global__ void __launch_bounds__(PF_THREADS)
pf_kernel(const typename Cx<T>::V *__restrict__ x, unsigned nmask,
          const typename Cx<T>::V *__restrict__ filt, int w, int B, int loops, int per, Draws d,
          int quirk, typename Cx<T>::V *__restrict__ bins) {
  pdl_enter();
  typedef typename Cx<T>::V V;
  const int b = blockIdx.x * PF_THREADS + threadIdx.x;
  if (b >= B) return;
  const int l0 = blockIdx.y * per;
  const int nl = min(per, loops - l0);
  const int tiles = w / B, residue = w % B;
  const int ntaps = tiles + (b < residue ? 1 : 0);
  unsigned ai[LCH];
#pragma unroll
  for (int c = 0; c < LCH; c++) ai[c] = (unsigned)d.ai[l0 + (c < nl ? c : 0)];
  T re[LCH], im[LCH];
#pragma unroll
  for (int c = 0; c < LCH; c++) { re[c] = 0; im[c] = 0; }
#pragma unroll 2
  for (int j = 0; j < ntaps; j++) {
    unsigned id = (unsigned)j * (unsigned)B + (unsigned)b;
    if (quirk && j == tiles && tiles > 0) id = (unsigned)b * (unsigned)tiles + (unsigned)B;
    const V f = filt[id];
    V xv[LCH];
#pragma unroll
    for (int c = 0; c < LCH; c++)
      if (c < nl) xv[c] = x[(id * ai[c]) & nmask];
#pragma unroll
    for (int c = 0; c < LCH; c++) {
      if (c >= nl) continue;
      re[c] = fma(xv[c].x, f.x, re[c]);
      re[c] = fma(-xv[c].y, f.y, re[c]);
      im[c] = fma(xv[c].x, f.y, im[c]);
      im[c] = fma(xv[c].y, f.x, im[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < LCH; c++)
    if (c < nl) bins[(size_t)(l0 + c) * B + b] = mk(re[c], im[c]);
}

}  // namespace

int launch_perm_filter(int precision, const void *x, int n, const void *filt, int w, int B,
                       int loops, const Draws &d, bool quirk_residue, void *bins,
                       cudaStream_t st) {
  if (loops > MAX_LOOPS || B <= 0 || w <= 0) return GSFFT_ERR_PARAM;
  const int chunks = (loops + LCH - 1) / LCH;
  const int per = (loops + chunks - 1) / chunks;  // balanced loops per chunk
  dim3 grid((B + PF_THREADS - 1) / PF_THREADS, chunks);
  const unsigned nmask = (unsigned)n - 1u;
  if (precision == GSFFT_FP64)
    GS_CUDA(launch_pdl(pf_kernel<double>, grid, dim3(PF_THREADS), 0, st, (const double2 *)x, nmask,
                       (const double2 *)filt, w, B, loops, per, d, quirk_residue ? 1 : 0,
                       (double2 *)bins));
  else
    GS_CUDA(launch_pdl(pf_kernel<float>, grid, dim3(PF_THREADS), 0, st, (const float2 *)x, nmask,
                       (const float2 *)filt, w, B, loops, per, d, quirk_residue ? 1 : 0,
                       (float2 *)bins));
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
