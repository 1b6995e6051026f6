// 64-point complex DFTs on the 5th-generation tensor cores (tcgen05).
//
// A batch of length-64 complex vectors is transformed as one real matrix
// product D = F * X: F is the 128 x 128 real form of the DFT matrix
// ([Re; Im] of the output from [Re; Im] of the input), X holds 64 vectors as
// the N = 64 columns, D (fp32) lives in tensor memory.  The operands are
// split into three bf16 parts (x = x0 + x1 + x2, 8 significant bits each, so
// together they carry FP32's 24) and the six products with part-index sum
// <= 2 are accumulated in fp32 -- the terms dropped are below 2^-24 of the
// result, so the product matches an FP32 DFT to rounding level.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, core (row group r, k group c) at byte
// (r * K/8 + c) * 128, so a descriptor's leading-dimension offset (next core
// along K) is 128 bytes and its stride offset (next 8-row group) K/8 * 128.
#include "gsfft_internal.cuh"

#include <cuda_bf16.h>

namespace gsfft {

namespace {

constexpr int TC_THREADS = 128;  // one warpgroup: TMEM lanes 0..127
constexpr int TC_M = 128;        // rows of F (real form of 64 outputs)
constexpr int TC_K = 128;        // columns of F (real form of 64 inputs)
constexpr int TC_N = 64;         // vectors per MMA tile
constexpr int A_BYTES = TC_M * TC_K * 2;   // one bf16 part of F: 32 KiB
constexpr int B_BYTES = TC_N * TC_K * 2;   // one bf16 part of X: 16 KiB
constexpr int TC_SMEM = 3 * A_BYTES + 3 * B_BYTES + 64;

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// byte offset of element (row, k) in a K-major, no-swizzle operand with K columns
__device__ __forceinline__ int kmajor_off(int row, int k, int K) {
  return ((row >> 3) * (K >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor (tcgen05): start, leading / stride byte
// offsets (>> 4), descriptor version 1, no swizzle
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  unsigned long long d = 0;
  d |= (unsigned long long)((addr >> 4) & 0x3FFFu);
  d |= (unsigned long long)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (unsigned long long)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;  // version
  return d;         // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor, kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N >> 3 and M >> 4
constexpr unsigned idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void split3(float v, __nv_bfloat16 &p0, __nv_bfloat16 &p1, __nv_bfloat16 &p2) {
  p0 = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(p0);
  p1 = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(p1);
  p2 = __float2bfloat16_rn(r2);
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
  const long long t0 = clock64();
  while (true) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > (1LL << 30)) return false;
  }
}

// y[v] = DFT_64(x[v]) (forward, unnormalised) for v < nvec; float2 vectors.
__global__ void __launch_bounds__(TC_THREADS, 1)
tc_dft64_kernel(const float2 *__restrict__ x, float2 *__restrict__ y, int nvec, int *err) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char *A = tsm;                      // 3 parts of F
  unsigned char *Bm = tsm + 3 * A_BYTES;       // 3 parts of X
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(tsm + 3 * A_BYTES + 3 * B_BYTES);
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // F in real form, split in three bf16 parts
  for (int e = tid; e < TC_M * TC_K; e += TC_THREADS) {
    const int m = e / TC_K, k = e % TC_K;
    const int o = m & 63, i = k & 63;
    double s, c;
    sincospi(-2.0 * (double)((o * i) & 63) / 64.0, &s, &c);  // e^{-2 pi i o i / 64} = c + i s
    float f;
    if (m < 64) f = (k < 64) ? (float)c : (float)(-s);  // Re out = c*xr - s*xi
    else f = (k < 64) ? (float)s : (float)c;            // Im out = s*xr + c*xi
    __nv_bfloat16 p0, p1, p2;
    split3(f, p0, p1, p2);
    const int off = kmajor_off(m, k, TC_K);
    *reinterpret_cast<__nv_bfloat16 *>(A + off) = p0;
    *reinterpret_cast<__nv_bfloat16 *>(A + A_BYTES + off) = p1;
    *reinterpret_cast<__nv_bfloat16 *>(A + 2 * A_BYTES + off) = p2;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(TC_N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;
  constexpr unsigned IDESC = idesc_bf16(TC_M, TC_N);
  unsigned phase = 0;
  bool ok = true;

  for (int v0 = blockIdx.x * TC_N; v0 < nvec && ok; v0 += gridDim.x * TC_N) {
    // X tile: row v (vector), k < 64 real parts, k >= 64 imaginary parts
    for (int e = tid; e < TC_N * 64; e += TC_THREADS) {
      const int v = e >> 6, i = e & 63;
      const float2 xv = (v0 + v < nvec) ? x[(size_t)(v0 + v) * 64 + i] : make_float2(0.f, 0.f);
      __nv_bfloat16 p0, p1, p2;
      const int offr = kmajor_off(v, i, TC_K), offi = kmajor_off(v, 64 + i, TC_K);
      split3(xv.x, p0, p1, p2);
      *reinterpret_cast<__nv_bfloat16 *>(Bm + offr) = p0;
      *reinterpret_cast<__nv_bfloat16 *>(Bm + B_BYTES + offr) = p1;
      *reinterpret_cast<__nv_bfloat16 *>(Bm + 2 * B_BYTES + offr) = p2;
      split3(xv.y, p0, p1, p2);
      *reinterpret_cast<__nv_bfloat16 *>(Bm + offi) = p0;
      *reinterpret_cast<__nv_bfloat16 *>(Bm + B_BYTES + offi) = p1;
      *reinterpret_cast<__nv_bfloat16 *>(Bm + 2 * B_BYTES + offi) = p2;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // the six products with part-index sum <= 2, smallest first
      const int pa[6] = {1, 0, 2, 0, 1, 0};
      const int pb[6] = {1, 2, 0, 1, 0, 0};
      for (int t = 0; t < 6; t++) {
        const unsigned abase = smem_addr(A + pa[t] * A_BYTES);
        const unsigned bbase = smem_addr(Bm + pb[t] * B_BYTES);
#pragma unroll
        for (int kk = 0; kk < TC_K / 16; kk++) {
          const unsigned long long ad = smem_desc(abase + kk * 256, 128, (TC_K / 8) * 128);
          const unsigned long long bd = smem_desc(bbase + kk * 256, 128, (TC_K / 8) * 128);
          const unsigned acc = (t > 0 || kk > 0) ? 1u : 0u;
          asm volatile(
              "{ .reg .pred p; setp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
              : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_addr(bar))
                   : "memory");
    }
    if (!mbar_wait_bounded(smem_addr(bar), phase)) {
      ok = false;
      if (tid == 0) atomicExch(err, 1);
    }
    ok = __syncthreads_and(ok) != 0;  // warp-collective TMEM loads below: all or none
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
      // warp w reads TMEM lanes 32w..32w+31 = rows of D: Re (w < 2) or Im of output 32(w&1)+lane
      const int o = 32 * (warp & 1) + lane;
      const bool im = warp >= 2;
#pragma unroll
      for (int c0 = 0; c0 < TC_N; c0 += 8) {
        unsigned r[8];
        const unsigned taddr = tmem + ((unsigned)(32 * warp) << 16) + (unsigned)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int v = v0 + c0 + j;
          if (v < nvec) reinterpret_cast<float *>(y)[((size_t)v * 64 + o) * 2 + (im ? 1 : 0)] = __uint_as_float(r[j]);
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // TMEM and the X tile are reused by the next tile
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N) : "memory");
}

}  // namespace

int launch_tc_dft64(const void *x, void *y, int nvec, int *err, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    GS_CUDA(cudaFuncSetAttribute(tc_dft64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    attr = true;
  }
  int dev = 0, sms = 0;
  GS_CUDA(cudaGetDevice(&dev));
  GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int tiles = (nvec + TC_N - 1) / TC_N;
  const int grid = tiles < sms ? tiles : sms;
  if (grid < 1) return GSFFT_OK;
  tc_dft64_kernel<<<grid, TC_THREADS, TC_SMEM, st>>>((const float2 *)x, (float2 *)y, nvec, err);
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
