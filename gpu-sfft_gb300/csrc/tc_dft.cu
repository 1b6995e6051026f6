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

// The three bf16 parts of F' (the real form of DFT_64 with the real and
// imaginary rows of each output interleaved: row 2o = Re, row 2o + 1 = Im of
// output o) in the K-major layout, 3 x 32 KiB, built once per FFT plan.
// With theta = 2 pi o i / 64 and W = e^{-i theta}:
//   Re(W x) = cos(theta) xr + sin(theta) xi,  Im(W x) = cos(theta) xi - sin(theta) xr.
__global__ void tc_build_F_kernel(unsigned char *F) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= TC_M * TC_K) return;
  const int m = e / TC_K, k = e % TC_K;
  const int o = m >> 1, i = k & 63;
  double s, c;
  sincospi(2.0 * (double)((o * i) & 63) / 64.0, &s, &c);
  float f;
  if ((m & 1) == 0) f = (k < 64) ? (float)c : (float)s;
  else f = (k < 64) ? (float)(-s) : (float)c;
  __nv_bfloat16 p0, p1, p2;
  split3(f, p0, p1, p2);
  const int off = kmajor_off(m, k, TC_K);
  *reinterpret_cast<__nv_bfloat16 *>(F + off) = p0;
  *reinterpret_cast<__nv_bfloat16 *>(F + A_BYTES + off) = p1;
  *reinterpret_cast<__nv_bfloat16 *>(F + 2 * A_BYTES + off) = p2;
}

// ---- radix-4096 pass ------------------------------------------------------
constexpr int TP_THREADS = 256;  // 8 warps: warp w reads TMEM lanes 32 (w % 4) .. + 31
constexpr int TP_N = 128;        // vectors per product: two sub-transforms x 64
constexpr int X_BYTES = TP_N * TC_K * 2;  // one bf16 part of the X operand: 32 KiB
constexpr int TW_BYTES = 4096 * 8;        // exp(-2 pi i m / 4096), m < 4096
constexpr int TC4K_SMEM = 3 * A_BYTES + 3 * X_BYTES + TW_BYTES + 64;
static_assert(TC4K_SMEM <= 227 * 1024, "radix-4096 pass exceeds the shared memory of a CTA");

// issue the six bf16 products D = F' * X (N = TP_N vectors) and commit them to bar
__device__ __forceinline__ void tc_issue(unsigned char *A, unsigned char *xb, unsigned tmem, unsigned bar) {
  constexpr unsigned IDESC = idesc_bf16(TC_M, TP_N);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int pa[6] = {1, 0, 2, 0, 1, 0};
  const int pb[6] = {1, 2, 0, 1, 0, 0};
  for (int t = 0; t < 6; t++) {
    const unsigned abase = smem_addr(A + pa[t] * A_BYTES);
    const unsigned bbase = smem_addr(xb + pb[t] * X_BYTES);
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
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// 32 consecutive TMEM columns of this warp's lane quadrant
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// three bf16 parts of eight consecutive K values of operand row `row` at
// columns k0..k0+7, one 16-byte store per part
__device__ __forceinline__ void store_parts8_row(unsigned char *xb, int row, int k0, const float *v) {
  unsigned w[3][4];
#pragma unroll
  for (int q = 0; q < 8; q += 2) {
    __nv_bfloat16 a[3], b[3];
    split3(v[q], a[0], a[1], a[2]);
    split3(v[q + 1], b[0], b[1], b[2]);
#pragma unroll
    for (int pp = 0; pp < 3; pp++)
      w[pp][q >> 1] = (unsigned)__bfloat16_as_ushort(a[pp]) | ((unsigned)__bfloat16_as_ushort(b[pp]) << 16);
  }
  const int off = kmajor_off(row, k0, TC_K);
#pragma unroll
  for (int pp = 0; pp < 3; pp++)
    *reinterpret_cast<uint4 *>(xb + pp * X_BYTES + off) = make_uint4(w[pp][0], w[pp][1], w[pp][2], w[pp][3]);
}

// A first radix-4096 Stockham pass (Ns = 1) of an FP32 FFT as a four-step
// transform on the tensor cores, two sub-transforms j, j + 1 (adjacent in
// memory) per tile.  With r = r1 + 64 r2 and k = k2 + 64 k1:
//   Y[r1][k2] = sum_r2 v[r1 + 64 r2] W64^(r2 k2)                   (product 1)
//   V[k2 + 64 k1] = sum_r1 W64^(r1 k1) W4096^(r1 k2) Y[r1][k2]       (product 2)
// where v[r] = in[j + r S] (S = N / 4096 sub-transforms per row, the sum of
// nsum partial inputs sstride apart) and out[j 4096 + k] = V[k].
// Product 1's X operand: row n = (jj, r1) = 64 jj + r1, column K = r2 (Re) and
// 64 + r2 (Im).  Its result D (TMEM lane 2 k2 + c, column n) is read back
// lane by lane: lanes 2 k2 and 2 k2 + 1 (adjacent threads of one warp) hold
// Re and Im of Y[r1][k2], exchange them with a shuffle, apply W4096^(r1 k2)
// and write product 2's X operand: row (jj, k2), column r1 (Re) / 64 + r1 (Im).
// Product 2's result, lane 2 k1 + c and column (jj, k2), is V[k2 + 64 k1]:
// each thread pair again exchanges halves so that each thread stores 32
// consecutive outputs.
__global__ void __launch_bounds__(TP_THREADS, 1) tc4096_pass_kernel(TcPassArgs a) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char *A = tsm;                       // 3 parts of F'
  unsigned char *X = tsm + 3 * A_BYTES;         // 3 parts of the operand of the current product
  float2 *t4k = reinterpret_cast<float2 *>(tsm + 3 * A_BYTES + 3 * X_BYTES);
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(tsm + 3 * A_BYTES + 3 * X_BYTES + TW_BYTES);
  unsigned long long *fbar = bar + 1;
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;
  const float2 *__restrict__ in = reinterpret_cast<const float2 *>(a.in);
  float2 *__restrict__ out = reinterpret_cast<float2 *>(a.out);
  const float2 *__restrict__ twg = reinterpret_cast<const float2 *>(a.tw_R);
  const int logS = a.logN - 12;
  const long long S = 1LL << logS;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(TP_N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(fbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(fbar)),
                 "r"(3 * A_BYTES)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(A)),
        "l"(a.F), "r"(3 * A_BYTES), "r"(smem_addr(fbar))
        : "memory");
  }
  for (int i = tid; i < 4096; i += TP_THREADS) t4k[i] = twg[i];
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;
  const unsigned tq = tmem + ((unsigned)(32 * quad) << 16);  // this warp's lane quadrant
  const int L = 32 * quad + lane;                             // TMEM lane of this thread
  const int kc = L >> 1, c = L & 1;                           // output index, Re (0) / Im (1)
  const int jj = half;                                        // sub-transform of this thread's columns
  unsigned phase = 0;
  bool ok = true, f_ready = false;
  const long long ntiles = (a.total + 1) >> 1;

  for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const long long u0 = 2 * t;
    const bool two = u0 + 1 < a.total;
    const long long b = u0 >> logS, j = u0 & (S - 1);  // j even: j and j + 1 share a row
    const float2 *src = in + b * a.bstride + j;
    // ---- product 1 operand: items (r1, g), r2 = 8 g + q
#pragma unroll 1
    for (int it = 0; it < 2; it++) {
      const int item = tid + it * TP_THREADS;
      const int r1 = item & 63, g = item >> 6;
      float4 xv[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const long long off = (long long)(r1 + 64 * (8 * g + q)) << logS;
        if (two) {
          xv[q] = *reinterpret_cast<const float4 *>(src + off);
        } else {
          const float2 v = src[off];
          xv[q] = make_float4(v.x, v.y, 0.f, 0.f);
        }
      }
      for (int s2 = 1; s2 < a.nsum; s2++) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const long long off = s2 * a.sstride + ((long long)(r1 + 64 * (8 * g + q)) << logS);
          float4 v;
          if (two) {
            v = *reinterpret_cast<const float4 *>(src + off);
          } else {
            const float2 w = src[off];
            v = make_float4(w.x, w.y, 0.f, 0.f);
          }
          xv[q].x += v.x;
          xv[q].y += v.y;
          xv[q].z += v.z;
          xv[q].w += v.w;
        }
      }
      float re0[8], im0[8], re1[8], im1[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        re0[q] = xv[q].x;
        im0[q] = a.inverse ? -xv[q].y : xv[q].y;
        re1[q] = xv[q].z;
        im1[q] = a.inverse ? -xv[q].w : xv[q].w;
      }
      store_parts8_row(X, r1, 8 * g, re0);
      store_parts8_row(X, r1, 64 + 8 * g, im0);
      store_parts8_row(X, 64 + r1, 8 * g, re1);
      store_parts8_row(X, 64 + r1, 64 + 8 * g, im1);
    }
    for (int step = 0; step < 2 && ok; step++) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        bool go = true;
        if (!f_ready) {
          go = mbar_wait_bounded(smem_addr(fbar), 0);
          f_ready = go;
        }
        if (go) {
          tc_issue(A, X, tmem, smem_addr(bar));
        } else {
          // nothing issued: arrive on the barrier so that every thread leaves its wait
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
          ok = false;
          if (a.err) atomicExch(a.err, 1);
        }
      }
      if (!mbar_wait_bounded(smem_addr(bar), phase)) {
        ok = false;
        if (tid == 0 && a.err) atomicExch(a.err, 1);
      }
      ok = __syncthreads_and(ok) != 0;  // warp-collective TMEM loads below: all or none
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (!ok) break;
      if (step == 0) {
        // D1 lane (kc = k2, c), columns n = 64 jj + r1  ->  product 2 operand
#pragma unroll 1
        for (int c0 = 0; c0 < 64; c0 += 32) {
          float y[32];
          tmem_ld32(tq + (unsigned)(64 * jj + c0), y);
          float z[32];
#pragma unroll
          for (int i = 0; i < 32; i++) {
            const float other = __shfl_xor_sync(0xffffffffu, y[i], 1);
            const float yr = c ? other : y[i], yi = c ? y[i] : other;
            const float2 w = t4k[((c0 + i) * kc) & 4095];
            z[i] = c ? fmaf(yr, w.y, yi * w.x) : fmaf(yr, w.x, -(yi * w.y));
          }
#pragma unroll
          for (int grp = 0; grp < 4; grp++)
            store_parts8_row(X, 64 * jj + kc, (c ? 64 : 0) + c0 + 8 * grp, z + 8 * grp);
        }
      } else if (jj == 0 || two) {
        // D3 lane (kc = k1, c), columns (jj, k2): V[k2 + 64 k1]; this thread keeps k2 in [32 c, 32 c + 32)
        float2 v[32];
#pragma unroll 1
        for (int c0 = 0; c0 < 64; c0 += 32) {
          float y[32];
          tmem_ld32(tq + (unsigned)(64 * jj + c0), y);
          const bool keep = c0 == 32 * c;
#pragma unroll
          for (int i = 0; i < 32; i++) {
            const float other = __shfl_xor_sync(0xffffffffu, y[i], 1);
            if (keep) v[i] = c ? make_float2(other, y[i]) : make_float2(y[i], other);
          }
        }
        float2 *dp = out + b * a.bstride + (j + jj) * 4096 + 64 * kc + 32 * c;
#pragma unroll
        for (int i = 0; i < 32; i += 2) {
          const float s = a.inverse ? -1.f : 1.f;
          *reinterpret_cast<float4 *>(dp + i) = make_float4(v[i].x, s * v[i].y, v[i + 1].x, s * v[i + 1].y);
        }
      } else {
        // the second sub-transform of a tile with one: no outputs, but the
        // warp still took part in the collective loads of the other half
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // the operand buffer and TMEM are rewritten by the next tile
  }
  if (tid == 0 && !f_ready) (void)mbar_wait_bounded(smem_addr(fbar), 0);
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TP_N) : "memory");
}

}  // namespace

int launch_tc_dft64(const void *x, void *y, int nvec, int *err, cudaStream_t st) {
  static PerContext<int> attr;  // the kernel's dynamic shared memory limit, per context
  GS_CHECK(attr.ensure_at_least(TC_SMEM, [](int v) {
    if (cudaFuncSetAttribute(tc_dft64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, v) ==
        cudaSuccess)
      return (int)GSFFT_OK;
    set_last_error("tc_dft64_kernel: %d bytes of shared memory refused: %s", v,
                   cudaGetErrorString(cudaGetLastError()));
    return (int)GSFFT_ERR_CUDA;
  }));
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

namespace {
// Failure-detection self-check: one CTA waits on an mbarrier that nothing
// arrives on (no copy or product is ever issued against it), with the
// engine's bounded wait, and records that the wait gave up.
__global__ void bounded_wait_probe_kernel(long long limit, int *gave_up) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool done = mbar_wait_bounded(smem_addr(&bar), 0, limit);
  if (threadIdx.x == 0) *gave_up = done ? 0 : 1;
}
}  // namespace

int launch_bounded_wait_probe(long long limit, int *gave_up, cudaStream_t st) {
  bounded_wait_probe_kernel<<<1, 32, 0, st>>>(limit, gave_up);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int tc_build_F(void **F) {
  GS_CUDA(cudaMalloc(F, 3 * A_BYTES));
  tc_build_F_kernel<<<(TC_M * TC_K + 255) / 256, 256>>>(static_cast<unsigned char *>(*F));
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_tc4096_pass(const TcPassArgs &a, cudaStream_t st) {
  // first passes only (Ns = 1, outputs contiguous per sub-transform), an even
  // number of sub-transforms per row and 16-byte aligned element pairs
  if (a.logNs != 0 || a.logN < 13 || !a.tw_R || !a.F || a.samples || a.row_max || !a.write_complex)
    return GSFFT_ERR_UNSUPPORTED;
  if ((reinterpret_cast<uintptr_t>(a.in) & 15) || (reinterpret_cast<uintptr_t>(a.out) & 15) ||
      (a.bstride & 1) || (a.nsum > 1 && (a.sstride & 1)))
    return GSFFT_ERR_UNSUPPORTED;
  static PerContext<int> attr;  // the kernel's dynamic shared memory limit, per context
  GS_CHECK(attr.ensure_at_least(TC4K_SMEM, [](int v) {
    if (cudaFuncSetAttribute(tc4096_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, v) ==
        cudaSuccess)
      return (int)GSFFT_OK;
    set_last_error("tc4096_pass_kernel: %d bytes of shared memory refused: %s", v,
                   cudaGetErrorString(cudaGetLastError()));
    return (int)GSFFT_ERR_CUDA;
  }));
  int dev = 0, sms = 0;
  GS_CUDA(cudaGetDevice(&dev));
  GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const long long ntiles = (a.total + 1) / 2;
  const int grid = (int)(ntiles < sms ? ntiles : sms);
  if (grid < 1) return GSFFT_OK;
  tc4096_pass_kernel<<<grid, TP_THREADS, TC4K_SMEM, st>>>(a);
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
