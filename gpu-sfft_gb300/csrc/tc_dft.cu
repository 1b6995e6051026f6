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

// The three bf16 parts of F (real form of DFT_64) in the K-major layout,
// 3 x 32 KiB, built once per FFT plan.
__global__ void tc_build_F_kernel(unsigned char *F) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= TC_M * TC_K) return;
  const int m = e / TC_K, k = e % TC_K;
  const int o = m & 63, i = k & 63;
  double s, c;
  sincospi(-2.0 * (double)((o * i) & 63) / 64.0, &s, &c);
  float f;
  if (m < 64) f = (k < 64) ? (float)c : (float)(-s);
  else f = (k < 64) ? (float)s : (float)c;
  __nv_bfloat16 p0, p1, p2;
  split3(f, p0, p1, p2);
  const int off = kmajor_off(m, k, TC_K);
  *reinterpret_cast<__nv_bfloat16 *>(F + off) = p0;
  *reinterpret_cast<__nv_bfloat16 *>(F + A_BYTES + off) = p1;
  *reinterpret_cast<__nv_bfloat16 *>(F + 2 * A_BYTES + off) = p2;
}

constexpr int TP_THREADS = 256;  // two warpgroups: TMEM quadrant = warp % 4
constexpr int DP = 68;           // row pitch (floats) of the fp32 result staged in shared memory

constexpr int ST_BYTES = 128 * DP * 4;  // fp32 staging of a 128 x 64 result
constexpr int TC4K_SMEM = 3 * A_BYTES + 3 * B_BYTES + ST_BYTES + 64;

// issue the six bf16 products D = F * X (X parts at xb) and commit them to bar
__device__ __forceinline__ void tc_issue(unsigned char *A, unsigned char *xb, unsigned tmem, unsigned bar) {
  constexpr unsigned IDESC = idesc_bf16(TC_M, TC_N);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int pa[6] = {1, 0, 2, 0, 1, 0};
  const int pb[6] = {1, 2, 0, 1, 0, 0};
  for (int t = 0; t < 6; t++) {
    const unsigned abase = smem_addr(A + pa[t] * A_BYTES);
    const unsigned bbase = smem_addr(xb + pb[t] * B_BYTES);
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

// TMEM result (128 lanes x 64 columns) -> stg[m][c] (row pitch DP), by 8 warps
__device__ __forceinline__ void tmem_to_stage(unsigned tmem, float *stg, int warp, int lane) {
  const int q4 = warp & 3, h = warp >> 2;
  const int m = 32 * q4 + lane;
#pragma unroll
  for (int c = 0; c < 32; c += 8) {
    const int c0 = 32 * h + c;
    unsigned r[8];
    const unsigned taddr = tmem + ((unsigned)(32 * q4) << 16) + (unsigned)c0;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    uint4 *d4 = reinterpret_cast<uint4 *>(stg + m * DP + c0);
    d4[0] = make_uint4(r[0], r[1], r[2], r[3]);
    d4[1] = make_uint4(r[4], r[5], r[6], r[7]);
  }
}

// split eight complex values into the three bf16 parts of operand row `row`,
// columns kc..kc+7 (re) and 64+kc..64+kc+7 (im)
__device__ __forceinline__ void store_parts8(unsigned char *xb, int row, int kc, const float2 (&x)[8]) {
  unsigned wr[3][4], wi[3][4];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    __nv_bfloat16 r[3], im[3];
    split3(x[q].x, r[0], r[1], r[2]);
    split3(x[q].y, im[0], im[1], im[2]);
#pragma unroll
    for (int pp = 0; pp < 3; pp++) {
      const unsigned br = __bfloat16_as_ushort(r[pp]), bi = __bfloat16_as_ushort(im[pp]);
      if (q & 1) {
        wr[pp][q >> 1] |= br << 16;
        wi[pp][q >> 1] |= bi << 16;
      } else {
        wr[pp][q >> 1] = br;
        wi[pp][q >> 1] = bi;
      }
    }
  }
  const int offr = kmajor_off(row, kc, TC_K), offi = kmajor_off(row, 64 + kc, TC_K);
#pragma unroll
  for (int pp = 0; pp < 3; pp++) {
    *reinterpret_cast<uint4 *>(xb + pp * B_BYTES + offr) = make_uint4(wr[pp][0], wr[pp][1], wr[pp][2], wr[pp][3]);
    *reinterpret_cast<uint4 *>(xb + pp * B_BYTES + offi) = make_uint4(wi[pp][0], wi[pp][1], wi[pp][2], wi[pp][3]);
  }
}

// One radix-4096 Stockham pass of an FP32 FFT as a four-step transform on the
// tensor cores: one sub-transform per tile; with r = r1 + 64 r2 and
// k = k2 + 64 k1,
//   Y[r1][k2] = sum_r2 v[r1 + 64 r2] W64^(r2 k2)            (tensor cores)
//   V[k2 + 64 k1] = sum_r1 W64^(r1 k1) W4096^(r1 k2) Y[r1][k2] (tensor cores)
// where v[r] = in[j + r S] * w((j mod Ns) r / (Ns 4096)) and the result goes
// to out[(j / Ns) Ns 4096 + (j mod Ns) + k Ns].
__global__ void __launch_bounds__(TP_THREADS, 1) tc4096_pass_kernel(TcPassArgs a) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char *A = tsm;
  unsigned char *Bm = tsm + 3 * A_BYTES;
  float *stg = reinterpret_cast<float *>(tsm + 3 * A_BYTES + 3 * B_BYTES);  // [128][DP]
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(tsm + 3 * A_BYTES + 3 * B_BYTES + ST_BYTES);
  unsigned long long *fbar = bar + 1;
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bar + 2);
  unsigned *red = tmem_slot + 1;  // [8]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float2 *__restrict__ in = reinterpret_cast<const float2 *>(a.in);
  float2 *__restrict__ out = reinterpret_cast<float2 *>(a.out);
  float *__restrict__ smp = reinterpret_cast<float *>(a.samples);
  const float2 *__restrict__ thi = reinterpret_cast<const float2 *>(a.tw_hi);
  const float2 *__restrict__ tlo = reinterpret_cast<const float2 *>(a.tw_lo);
  const float2 *__restrict__ t4k = reinterpret_cast<const float2 *>(a.tw_R);  // exp(-2 pi i m / 4096)
  const int logS = a.logN - 12;
  const long long Smask = (1LL << logS) - 1;
  const int logNs = a.logNs;
  const long long Nsmask = (1LL << logNs) - 1;
  const int hmask = (1 << a.tw_h) - 1;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(TC_N)
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
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;
  unsigned phase = 0;
  bool ok = true, f_ready = false;

  for (long long u = blockIdx.x; u < a.total && ok; u += gridDim.x) {
    const long long b = u >> logS, j = u & Smask;
    const float2 *src = in + b * a.bstride + j;
    // ---- step 1 operand: row r1, columns r2 (eight per item)
    {
      float2 xv[2][8];
#pragma unroll
      for (int it = 0; it < 2; it++) {
        const int item = tid + it * TP_THREADS;
        const int r1 = item & 63, g = item >> 6;
#pragma unroll
        for (int q = 0; q < 8; q++) xv[it][q] = src[(long long)(r1 + 64 * (8 * g + q)) << logS];
        // row-group partial inputs (first pass after the streaming perm+filter),
        // added in group order
        for (int s2 = 1; s2 < a.nsum; s2++)
#pragma unroll
          for (int q = 0; q < 8; q++)
            xv[it][q] = cadd(xv[it][q], src[s2 * a.sstride + ((long long)(r1 + 64 * (8 * g + q)) << logS)]);
      }
#pragma unroll
      for (int it = 0; it < 2; it++) {
        const int item = tid + it * TP_THREADS;
        const int r1 = item & 63, g = item >> 6;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          float2 x = xv[it][q];
          if (a.inverse) x.y = -x.y;
          if (logNs > 0) {
            const long long mm = (j & Nsmask) * (long long)(r1 + 64 * (8 * g + q));
            x = cmul(x, cmul(thi[mm >> a.tw_h], tlo[mm & hmask]));
          }
          xv[it][q] = x;
        }
        store_parts8(Bm, r1, 8 * g, xv[it]);
      }
    }
    for (int step = 0; step < 2 && ok; step++) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        bool go = true;
        if (!f_ready) {
          go = mbar_wait_bounded(smem_addr(fbar), 0);
          f_ready = go;
        }
        if (go) {
          tc_issue(A, Bm, tmem, smem_addr(bar));
        } else {
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_addr(bar))
                       : "memory");
          ok = false;
          if (a.err) atomicExch(a.err, 1);
        }
      }
      if (!mbar_wait_bounded(smem_addr(bar), phase)) {
        ok = false;
        if (tid == 0 && a.err) atomicExch(a.err, 1);
      }
      ok = __syncthreads_and(ok) != 0;
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (!ok) break;
      tmem_to_stage(tmem, stg, warp, lane);  // stg[m][c]: m = output (re | im), c = vector
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (step == 0) {
        // step 3 operand: row k2, columns r1: Z = Y[r1][k2] * W4096^(r1 k2)
#pragma unroll
        for (int it = 0; it < 2; it++) {
          const int item = tid + it * TP_THREADS;
          const int k2 = item & 63, g = item >> 6;
          float2 z[8];
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const int r1 = 8 * g + q;
            const float2 y = make_float2(stg[k2 * DP + r1], stg[(64 + k2) * DP + r1]);
            z[q] = cmul(y, __ldg(&t4k[(r1 * k2) & 4095]));
          }
          store_parts8(Bm, k2, 8 * g, z);
        }
      }
    }
    if (!ok) break;
    // ---- outputs: k = k2 + 64 k1; stg[k1 (re) | 64 + k1 (im)][k2]
    float tmax = 0.f;
#pragma unroll 4
    for (int e = tid; e < 4096; e += TP_THREADS) {
      const int k2 = e & 63, k1 = e >> 6;
      const int k = k2 + 64 * k1;
      const float re = stg[k1 * DP + k2];
      float im = stg[(64 + k1) * DP + k2];
      if (a.inverse) im = -im;
      const long long dest = b * a.bstride + ((j >> logNs) << (logNs + 12)) + (j & Nsmask) +
                             ((long long)k << logNs);
      if (a.write_complex) out[dest] = make_float2(re, im);
      if (smp) {
        const float sq = __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
        smp[dest] = sq;
        tmax = sq > tmax ? sq : tmax;
      }
    }
    if (smp && a.row_max) {
      unsigned kmax = __float_as_uint(tmax);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned y = __shfl_xor_sync(0xffffffffu, kmax, o);
        kmax = y > kmax ? y : kmax;
      }
      if (lane == 0) red[warp] = kmax;
      __syncthreads();
      if (tid == 0) {
        unsigned m8 = red[0];
        for (int w2 = 1; w2 < TP_THREADS / 32; w2++) m8 = red[w2] > m8 ? red[w2] : m8;
        atomicMax(reinterpret_cast<unsigned *>(a.row_max) + b, m8);
      }
    }
    __syncthreads();  // the staging and operand buffers are rewritten by the next tile
  }
  if (tid == 0 && !f_ready) (void)mbar_wait_bounded(smem_addr(fbar), 0);
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N) : "memory");
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

int tc_build_F(void **F) {
  GS_CUDA(cudaMalloc(F, 3 * A_BYTES));
  tc_build_F_kernel<<<(TC_M * TC_K + 255) / 256, 256>>>(static_cast<unsigned char *>(*F));
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_tc4096_pass(const TcPassArgs &a, cudaStream_t st) {
  static PerContext<int> attr;  // the kernel's dynamic shared memory limit, per context
  GS_CHECK(attr.ensure_at_least(TC4K_SMEM, [](int v) {
    if (cudaFuncSetAttribute(tc4096_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, v) ==
        cudaSuccess)
      return (int)GSFFT_OK;
    set_last_error("tc4096_pass_kernel: %d bytes of shared memory refused: %s", v,
                   cudaGetErrorString(cudaGetLastError()));
    return (int)GSFFT_ERR_CUDA;
  }));
  if (a.logN < 12 || !a.tw_R) return GSFFT_ERR_UNSUPPORTED;
  int dev = 0, sms = 0;
  GS_CUDA(cudaGetDevice(&dev));
  GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = (int)(a.total < sms ? a.total : sms);
  if (grid < 1) return GSFFT_OK;
  tc4096_pass_kernel<<<grid, TP_THREADS, TC4K_SMEM, st>>>(a);
  GS_LAUNCHED();
  return GSFFT_OK;
}


}  // namespace gsfft
