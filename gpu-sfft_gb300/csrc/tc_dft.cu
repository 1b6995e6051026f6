// 64-point complex DFTs on the 5th-generation tensor cores (tcgen05): a
// building block over independent vectors (tc_dft64_kernel) and two FFT
// passes built from it -- a radix-4096 first pass (two DFT_64 stages, a
// warp-specialised two-tile pipeline) and a radix-64 last pass (one DFT_64
// stage per 128 sub-transforms, coalesced both ways).
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
// output o), built once per FFT plan in the tensor-memory layout of an A
// operand: part p, row m (a TMEM lane), 32-bit column c holding k = 2c in its
// low and k = 2c + 1 in its high half.  In global memory a part is 128 rows of
// 256 bytes whose 16-byte chunks are XOR-swizzled by the row (chunk ch of row
// m at (ch ^ (m & 15)) * 16), so that a warp reading chunk ch of 32 rows from
// a shared-memory copy touches every bank once per 128 bytes.
// With theta = 2 pi o i / 64 and W = e^{-i theta}:
//   Re(W x) = cos(theta) xr + sin(theta) xi,  Im(W x) = cos(theta) xi - sin(theta) xr.
constexpr int FT_ROW_BYTES = 256;                   // 64 columns x 4 bytes
constexpr int FT_PART_BYTES = TC_M * FT_ROW_BYTES;  // 32 KiB
__global__ void tc_build_F_kernel(unsigned char *F) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= TC_M * (TC_K / 2)) return;
  const int m = e / (TC_K / 2), col = e % (TC_K / 2);
  const int o = m >> 1;
  unsigned w[3] = {0u, 0u, 0u};
  for (int h = 0; h < 2; h++) {
    const int k = 2 * col + h, i = k & 63;
    double sn, cs;
    sincospi(2.0 * (double)((o * i) & 63) / 64.0, &sn, &cs);
    float f;
    if ((m & 1) == 0) f = (k < 64) ? (float)cs : (float)sn;
    else f = (k < 64) ? (float)(-sn) : (float)cs;
    __nv_bfloat16 p[3];
    split3(f, p[0], p[1], p[2]);
    for (int pp = 0; pp < 3; pp++) w[pp] |= (unsigned)__bfloat16_as_ushort(p[pp]) << (16 * h);
  }
  const int ch = col >> 2;
  const int off = m * FT_ROW_BYTES + ((ch ^ (m & 15)) << 4) + (col & 3) * 4;
  for (int pp = 0; pp < 3; pp++) *reinterpret_cast<unsigned *>(F + pp * FT_PART_BYTES + off) = w[pp];
}

// ---- radix-4096 pass ------------------------------------------------------
constexpr int TP_N = 128;                 // vectors per product: two sub-transforms x 64
constexpr int X_BYTES = TP_N * TC_K * 2;  // one bf16 part of an operand: 32 KiB
constexpr int TQ_XBUF = 3 * X_BYTES;      // one operand buffer (three parts): 96 KiB
constexpr int TQ_TW_BYTES = 64 * 64 * 8;  // W4096^(r1 k2) at [r1][k2]
constexpr int TQ_LD_WARPS = 8;            // loaders: global -> bf16 parts of product 1's operand
constexpr int TQ_EP_WARPS = 4;            // epilogue: TMEM read-back (warp w: lanes 32 (w % 4) ..)
constexpr int TQ_MMA_WARP = TQ_LD_WARPS + TQ_EP_WARPS;  // issues the products (one lane)
constexpr int TQ_THREADS = (TQ_MMA_WARP + 1) * 32;
constexpr int TQ_TMEM_COLS = 512;  // F' parts at columns 0, 64, 128; product buffers at 256, 384
constexpr unsigned TQ_D_COL = 256;
// mbarriers
enum {
  B_XFULL = 0,    // [2] loaders -> MMA: product 1's operand is in X[b]
  B_X2FULL = 2,   // [2] epilogue -> MMA: product 2's operand is in X[b]
  B_DFREE = 4,    // [2] epilogue -> MMA: D[b] has been read
  B_D1 = 6,       // [2] MMA -> epilogue: product 1 is in D[b]
  B_D2 = 8,       // [2] MMA -> epilogue: product 2 is in D[b]
  B_XFREE = 10,   // [2] MMA -> loaders: the products reading X[b] are done
  B_FCOPY = 12,   // the bulk copy of F' into X[1] has landed
  B_FREADY = 13,  // epilogue -> all: F' is in tensor memory, X[1] is free
  B_FIN = 14,     // every product issued has completed
  TQ_NBAR = 15
};
constexpr int TQ_SMEM = 2 * TQ_XBUF + TQ_TW_BYTES + TQ_NBAR * 8 + 16;
static_assert(TQ_SMEM <= 227 * 1024, "radix-4096 pass exceeds the shared memory of a CTA");
static_assert(3 * FT_PART_BYTES <= TQ_XBUF, "F' staging does not fit an operand buffer");

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// A pipeline wait: gives up at once when another role has given up, else
// after the engine's bound (and then makes every role give up).  The result
// is made uniform over the warp, whose TMEM accesses are collective.
__device__ __forceinline__ bool role_wait(unsigned bar, unsigned parity, volatile int *abort, int *err) {
  bool ok = *abort == 0;
  if (ok && !mbar_wait_bounded(bar, parity)) {
    ok = false;
    *abort = 1;
    if (err) atomicExch(err, 1);
  }
  return __all_sync(0xffffffffu, ok);
}

// issue the six bf16 products D = F' * X (A = the F' parts in tensor memory,
// B = the three parts of X in shared memory, N = TP_N vectors)
__device__ __forceinline__ void tq_issue(unsigned tmem, unsigned dcol, unsigned xbase) {
  constexpr unsigned IDESC = idesc_bf16(TC_M, TP_N);
  const int pa[6] = {1, 0, 2, 0, 1, 0};
  const int pb[6] = {1, 2, 0, 1, 0, 0};
#pragma unroll
  for (int t = 0; t < 6; t++) {
#pragma unroll
    for (int kk = 0; kk < TC_K / 16; kk++) {
      const unsigned at = tmem + (unsigned)(64 * pa[t] + 8 * kk);  // 16 bf16 of K = 8 columns
      const unsigned long long bd = smem_desc(xbase + pb[t] * X_BYTES + kk * 256, 128, (TC_K / 8) * 128);
      const unsigned acc = (t > 0 || kk > 0) ? 1u : 0u;
      asm volatile(
          "{ .reg .pred p; setp.ne.b32 p, %4, 0;\n"
          "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p; }" ::"r"(dcol),
          "r"(at), "l"(bd), "r"(IDESC), "r"(acc)
          : "memory");
    }
  }
}

// 16 consecutive TMEM columns of this warp's lane quadrant (no wait)
__device__ __forceinline__ void tmem_ld16_nowait(unsigned taddr, unsigned (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 consecutive TMEM columns of this warp's lane quadrant from registers
__device__ __forceinline__ void tmem_st32(unsigned taddr, const unsigned (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31, %32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]),
      "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]),
      "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
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
//
// The CTA is a two-tile pipeline.  F' lives in tensor memory (the A operand
// of every product; one bulk copy of the plan's prebuilt parts into X[1],
// which the epilogue warps move to tensor memory), which leaves shared memory
// for two operand buffers X[b]
// and tensor memory for two product buffers D[b]; tile i of the CTA uses
// buffer b = i & 1.  Loader warps fill X[b] with tile i + 1's operand while
// the tensor cores and the epilogue warps work on tile i.  The MMA warp
// issues, in this order, product 1 of tile i and product 2 of tile i - 1; the
// epilogue warps read back product 1 of tile i (writing product 2's operand
// into X[b]) and then product 2 of tile i - 1 (storing the outputs).  Every
// hand-over is an mbarrier, every wait is bounded: a wait that gives up flags
// the run (a.err) and makes every role stop at its next wait, and the CTA
// still waits (bounded) for the products it issued before freeing the
// tensor memory.
__global__ void __launch_bounds__(TQ_THREADS, 1) tc4096_pass_kernel(TcPassArgs a) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char *X = tsm;  // X[0], X[1]
  float2 *tw = reinterpret_cast<float2 *>(tsm + 2 * TQ_XBUF);
  unsigned long long *bars = reinterpret_cast<unsigned long long *>(tsm + 2 * TQ_XBUF + TQ_TW_BYTES);
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bars + TQ_NBAR);
  volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned bar0 = smem_addr(bars);
#define BAR(i) (bar0 + 8u * (unsigned)(i))
  const float2 *__restrict__ in = reinterpret_cast<const float2 *>(a.in);
  float2 *__restrict__ out = reinterpret_cast<float2 *>(a.out);
  const float2 *__restrict__ twg = reinterpret_cast<const float2 *>(a.tw_R);
  const int logS = a.logN - 12;
  const long long S = 1LL << logS;
  const long long ntiles = a.total >> 1;
  const int T = (int)((ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x);  // tiles of this CTA

  if (warp == TQ_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(TQ_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    *abort = 0;
    for (int b = 0; b < 2; b++) {
      mbar_init(BAR(B_XFULL + b), TQ_LD_WARPS * 32);
      mbar_init(BAR(B_X2FULL + b), TQ_EP_WARPS * 32);
      mbar_init(BAR(B_DFREE + b), TQ_EP_WARPS * 32);
      mbar_init(BAR(B_D1 + b), 1);
      mbar_init(BAR(B_D2 + b), 1);
      mbar_init(BAR(B_XFREE + b), 1);
    }
    mbar_init(BAR(B_FCOPY), 1);
    mbar_init(BAR(B_FREADY), TQ_EP_WARPS * 32);
    mbar_init(BAR(B_FIN), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // F' (three parts, 96 KiB) into X[1], where the epilogue warps move it to tensor memory
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(BAR(B_FCOPY)),
                 "r"(3 * FT_PART_BYTES)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(X + TQ_XBUF)),
        "l"(a.F), "r"(3 * FT_PART_BYTES), "r"(BAR(B_FCOPY))
        : "memory");
  }
  for (int e = tid; e < 64 * 64; e += TQ_THREADS) tw[e] = twg[((e >> 6) * (e & 63)) & 4095];
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;

  if (warp < TQ_LD_WARPS) {
    // ---- loaders: items (r1, g) and (r1, g + 4), r2 = 8 g + q
    const int r1 = tid & 63, g0 = tid >> 6;
    for (int i = 0; i < T; i++) {
      const int b = i & 1;
      const unsigned u = (unsigned)i >> 1;
      bool ok = true;
      if (i == 1) ok = role_wait(BAR(B_FREADY), 0, abort, a.err);  // X[1] held the F' copy
      if (ok && u > 0) ok = role_wait(BAR(B_XFREE + b), (u - 1) & 1, abort, a.err);
      if (!ok) break;
      const long long u0 = 2 * ((long long)blockIdx.x + (long long)i * gridDim.x);
      const long long row = u0 >> logS, j = u0 & (S - 1);  // j even: j and j + 1 share a row
      const float2 *src = in + row * a.bstride + j;
      float4 xv[2][8];
#pragma unroll
      for (int h = 0; h < 2; h++)
#pragma unroll
        for (int q = 0; q < 8; q++)
          xv[h][q] = __ldg(reinterpret_cast<const float4 *>(
              src + ((long long)(r1 + 64 * (8 * (g0 + 4 * h) + q)) << logS)));
      for (int s2 = 1; s2 < a.nsum; s2++) {
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(
                src + s2 * a.sstride + ((long long)(r1 + 64 * (8 * (g0 + 4 * h) + q)) << logS)));
            xv[h][q].x += v.x;
            xv[h][q].y += v.y;
            xv[h][q].z += v.z;
            xv[h][q].w += v.w;
          }
      }
      unsigned char *xb = X + b * TQ_XBUF;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int g = g0 + 4 * h;
        float re0[8], im0[8], re1[8], im1[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          re0[q] = xv[h][q].x;
          im0[q] = a.inverse ? -xv[h][q].y : xv[h][q].y;
          re1[q] = xv[h][q].z;
          im1[q] = a.inverse ? -xv[h][q].w : xv[h][q].w;
        }
        store_parts8_row(xb, r1, 8 * g, re0);
        store_parts8_row(xb, r1, 64 + 8 * g, im0);
        store_parts8_row(xb, 64 + r1, 8 * g, re1);
        store_parts8_row(xb, 64 + r1, 64 + 8 * g, im1);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(BAR(B_XFULL + b));
    }
  } else if (warp < TQ_MMA_WARP) {
    // ---- epilogue: TMEM lane L = 32 q + lane
    const int q = warp & 3;
    const int L = 32 * q + lane;
    const int kc = L >> 1, c = L & 1;
    const unsigned tq = tmem + ((unsigned)(32 * q) << 16);
    bool ok = role_wait(BAR(B_FCOPY), 0, abort, a.err);
    if (ok) {
      // F' row L of each part: shared staging -> tensor memory columns 64 p + 32 h ..
      const unsigned char *fs = X + TQ_XBUF;
#pragma unroll 1
      for (int p = 0; p < 3; p++)
#pragma unroll 1
        for (int h = 0; h < 2; h++) {
          unsigned r[32];
#pragma unroll
          for (int cc = 0; cc < 8; cc++) {
            const int ch = 8 * h + cc;
            const uint4 v = *reinterpret_cast<const uint4 *>(fs + p * FT_PART_BYTES + L * FT_ROW_BYTES +
                                                             ((ch ^ (L & 15)) << 4));
            r[4 * cc] = v.x;
            r[4 * cc + 1] = v.y;
            r[4 * cc + 2] = v.z;
            r[4 * cc + 3] = v.w;
          }
          tmem_st32(tq + (unsigned)(64 * p + 32 * h), r);
        }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(BAR(B_FREADY));
    }
    for (int s = 0; s <= T && ok; s++) {
      if (s < T) {
        // product 1 of tile s -> product 2's operand in X[b]
        const int b = s & 1;
        const unsigned u = (unsigned)s >> 1;
        ok = role_wait(BAR(B_D1 + b), u & 1, abort, a.err);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        unsigned char *xb = X + b * TQ_XBUF;
        const unsigned dcol = tq + TQ_D_COL + 128u * b;
#pragma unroll 1
        for (int n0 = 0; n0 < 128; n0 += 16) {  // columns n = 64 jj + r1
          const int jj = n0 >> 6, c0 = n0 & 63;
          unsigned yr_[16];
          tmem_ld16_nowait(dcol + (unsigned)n0, yr_);
          tmem_wait_ld();
          float z[16];
#pragma unroll
          for (int i = 0; i < 16; i++) {
            const float y = __uint_as_float(yr_[i]);
            const float other = __shfl_xor_sync(0xffffffffu, y, 1);
            const float yr = c ? other : y, yi = c ? y : other;
            const float2 w = tw[(c0 + i) * 64 + kc];
            z[i] = c ? fmaf(yr, w.y, yi * w.x) : fmaf(yr, w.x, -(yi * w.y));
          }
          store_parts8_row(xb, 64 * jj + kc, (c ? 64 : 0) + c0, z);
          store_parts8_row(xb, 64 * jj + kc, (c ? 64 : 0) + c0 + 8, z + 8);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(BAR(B_X2FULL + b));
      }
      if (s >= 1) {
        // product 2 of tile s - 1 -> outputs
        const int i = s - 1, b = i & 1;
        const unsigned u = (unsigned)i >> 1;
        ok = role_wait(BAR(B_D2 + b), u & 1, abort, a.err);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const unsigned dcol = tq + TQ_D_COL + 128u * b;
        const long long u0 = 2 * ((long long)blockIdx.x + (long long)i * gridDim.x);
        const long long row = u0 >> logS, j = u0 & (S - 1);
        const float sg = a.inverse ? -1.f : 1.f;
#pragma unroll 1
        for (int n0 = 0; n0 < 128; n0 += 64) {
          // lane (kc = k1, c), columns n0 + k2: V[k2 + 64 k1] of sub-transform jj = n0 / 64.
          // Thread c keeps k2 in [32 c, 32 c + 32): its own half (Re for c = 0,
          // Im for c = 1) of those columns and its partner's other half.
          const int jj = n0 >> 6;
          float2 *dp = out + row * a.bstride + (j + jj) * 4096 + 64 * kc + 32 * c;
#pragma unroll 1
          for (int h = 0; h < 32; h += 16) {
            unsigned ya[16], yb[16];
            tmem_ld16_nowait(dcol + (unsigned)(n0 + h), ya);       // k2 = h ..
            tmem_ld16_nowait(dcol + (unsigned)(n0 + 32 + h), yb);  // k2 = 32 + h ..
            tmem_wait_ld();
#pragma unroll
            for (int i2 = 0; i2 < 16; i2 += 2) {
              float re[2], im[2];
#pragma unroll
              for (int e = 0; e < 2; e++) {
                const float send = __uint_as_float(c ? ya[i2 + e] : yb[i2 + e]);
                const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
                const float own = __uint_as_float(c ? yb[i2 + e] : ya[i2 + e]);
                re[e] = c ? recv : own;
                im[e] = sg * (c ? own : recv);
              }
              *reinterpret_cast<float4 *>(dp + h + i2) = make_float4(re[0], im[0], re[1], im[1]);
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(BAR(B_DFREE + b));
      }
    }
  } else {
    // ---- MMA warp: product 1 of tile s, then product 2 of tile s - 1
    bool ok = role_wait(BAR(B_FREADY), 0, abort, a.err);
    bool issued = false;
    for (int s = 0; s <= T && ok; s++) {
      if (s < T) {
        const int b = s & 1;
        const unsigned u = (unsigned)s >> 1;
        ok = role_wait(BAR(B_XFULL + b), u & 1, abort, a.err);
        if (ok && u > 0) ok = role_wait(BAR(B_DFREE + b), (u - 1) & 1, abort, a.err);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (lane == 0) {
          tq_issue(tmem, tmem + TQ_D_COL + 128u * b, smem_addr(X + b * TQ_XBUF));
          tc_commit(BAR(B_D1 + b));
        }
        __syncwarp();
        issued = true;
      }
      if (s >= 1) {
        const int i = s - 1, b = i & 1;
        const unsigned u = (unsigned)i >> 1;
        ok = role_wait(BAR(B_X2FULL + b), u & 1, abort, a.err);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (lane == 0) {
          tq_issue(tmem, tmem + TQ_D_COL + 128u * b, smem_addr(X + b * TQ_XBUF));
          tc_commit(BAR(B_D2 + b));
          tc_commit(BAR(B_XFREE + b));
        }
        __syncwarp();
      }
    }
    if (lane == 0) {
      if (issued) {
        tc_commit(BAR(B_FIN));
        if (!mbar_wait_bounded(BAR(B_FIN), 0) && a.err) atomicExch(a.err, 1);
      }
      // the F' copy has landed (a no-op unless a wait gave up before it)
      (void)mbar_wait_bounded(BAR(B_FCOPY), 0);
    }
    __syncwarp();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == TQ_MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TQ_TMEM_COLS)
                 : "memory");
#undef BAR
}

// ---- radix-64 last pass ----------------------------------------------------
// The three bf16 parts of F' (as above: interleaved Re / Im rows) in the
// shared-memory layout of an A operand (K-major, no swizzle), 3 x 32 KiB.
__global__ void tc_build_F_smem_kernel(unsigned char *F) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= TC_M * TC_K) return;
  const int m = e / TC_K, k = e % TC_K;
  const int o = m >> 1, i = k & 63;
  double sn, cs;
  sincospi(2.0 * (double)((o * i) & 63) / 64.0, &sn, &cs);
  float f;
  if ((m & 1) == 0) f = (k < 64) ? (float)cs : (float)sn;
  else f = (k < 64) ? (float)(-sn) : (float)cs;
  __nv_bfloat16 p0, p1, p2;
  split3(f, p0, p1, p2);
  const int off = kmajor_off(m, k, TC_K);
  *reinterpret_cast<__nv_bfloat16 *>(F + off) = p0;
  *reinterpret_cast<__nv_bfloat16 *>(F + A_BYTES + off) = p1;
  *reinterpret_cast<__nv_bfloat16 *>(F + 2 * A_BYTES + off) = p2;
}

constexpr int T64_THREADS = 256;  // 8 warps: warp w reads TMEM lanes 32 (w % 4) .. + 31
constexpr int T64_SMEM = 3 * A_BYTES + 3 * X_BYTES + 64;
static_assert(T64_SMEM <= 227 * 1024, "radix-64 pass exceeds the shared memory of a CTA");

__device__ __forceinline__ float sq_sum_f(float x, float y) { return __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)); }

// The last Stockham pass (radix 64, Ns = S = N / 64) of an FP32 FFT on the
// tensor cores:
//   V_j[k] = sum_r in[j + r S] W_N^(j r) W_64^(r k),   out[j + k S] = V_j[k],
// one product D = F' X per tile of 128 consecutive sub-transforms j (one
// row).  X row n = j - j0, columns K = r (Re) and 64 + r (Im) of the
// twiddled inputs, split into three bf16 parts; D lane 2k + c (Re / Im of
// output k), column n.  Both sides move whole 1 KiB runs: a warp loads 32
// consecutive j of one r, and each thread pair stores 32 consecutive j of one
// k.  The epilogue can also write |V|^2 and the row maximum (the bucket
// cutoff's samples).  F' stays in shared memory (one bulk copy per CTA).
__global__ void __launch_bounds__(T64_THREADS, 1) tc64_last_pass_kernel(TcPassArgs a) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char *A = tsm;                // 3 parts of F'
  unsigned char *X = tsm + 3 * A_BYTES;  // 3 parts of the operand
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(tsm + 3 * A_BYTES + 3 * X_BYTES);
  unsigned long long *fbar = bar + 1;
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float2 *__restrict__ in = reinterpret_cast<const float2 *>(a.in);
  float2 *__restrict__ out = reinterpret_cast<float2 *>(a.out);
  float *__restrict__ smp = reinterpret_cast<float *>(a.samples);
  const float2 *__restrict__ thi = reinterpret_cast<const float2 *>(a.tw_hi);
  const float2 *__restrict__ tlo = reinterpret_cast<const float2 *>(a.tw_lo);
  const int logS = a.logN - 6;
  const long long tpr = 1LL << (logS - 7);  // tiles per row
  const long long ntiles = a.total >> 7;
  const int th = a.tw_h;
  const long long hmask = (1LL << th) - 1;

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
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;
  const int quad = warp & 3, half = warp >> 2;
  const unsigned tq = tmem + ((unsigned)(32 * quad) << 16);
  const int L = 32 * quad + lane;
  const int kc = L >> 1, c = L & 1;
  unsigned phase = 0;
  bool ok = true, f_ready = false;

  for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const long long row = t / tpr, j0 = (t % tpr) << 7;
    const float2 *src = in + row * a.bstride + j0;
    // ---- operand: items (n, g), r = 8 g + q; a warp covers 32 consecutive n.
    // All 32 loads of a thread's four items are issued before any is used.
    const int n = tid & 127, gb = tid >> 7;  // items (n, gb + 2 it), it < 4
    float2 xv[4][8];
#pragma unroll
    for (int it = 0; it < 4; it++)
#pragma unroll
      for (int q = 0; q < 8; q++) xv[it][q] = src[n + ((long long)(8 * (gb + 2 * it) + q) << logS)];
#pragma unroll
    for (int it = 0; it < 4; it++) {
      const int g = gb + 2 * it;
      const long long jn = j0 + n;
      float re[8], im[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float2 v = xv[it][q];
        if (a.inverse) v.y = -v.y;
        const long long mm = jn * (8 * g + q);  // < N
        const float2 w = cmul(__ldg(&thi[mm >> th]), __ldg(&tlo[mm & hmask]));
        v = cmul(v, w);
        re[q] = v.x;
        im[q] = v.y;
      }
      store_parts8_row(X, n, 8 * g, re);
      store_parts8_row(X, n, 64 + 8 * g, im);
    }
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
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        constexpr unsigned IDESC = idesc_bf16(TC_M, TP_N);
        const int pa[6] = {1, 0, 2, 0, 1, 0};
        const int pb[6] = {1, 2, 0, 1, 0, 0};
        for (int u = 0; u < 6; u++) {
          const unsigned abase = smem_addr(A + pa[u] * A_BYTES);
          const unsigned bbase = smem_addr(X + pb[u] * X_BYTES);
#pragma unroll
          for (int kk = 0; kk < TC_K / 16; kk++) {
            const unsigned long long ad = smem_desc(abase + kk * 256, 128, (TC_K / 8) * 128);
            const unsigned long long bd = smem_desc(bbase + kk * 256, 128, (TC_K / 8) * 128);
            const unsigned acc = (u > 0 || kk > 0) ? 1u : 0u;
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
    // ---- outputs: this warp reads columns [64 half, 64 half + 64) of its
    // lanes; thread c stores the 32 columns 64 half + 32 c .. of output kc
    float tmax = 0.f;
#pragma unroll 1
    for (int hh = 0; hh < 32; hh += 16) {
      unsigned ya[16], yb[16];
      tmem_ld16_nowait(tq + (unsigned)(64 * half + hh), ya);
      tmem_ld16_nowait(tq + (unsigned)(64 * half + 32 + hh), yb);
      tmem_wait_ld();
      const long long off = row * a.bstride + j0 + 64 * half + 32 * c + hh + ((long long)kc << logS);
#pragma unroll
      for (int i2 = 0; i2 < 16; i2 += 2) {
        float re[2], im[2];
#pragma unroll
        for (int e = 0; e < 2; e++) {
          const float send = __uint_as_float(c ? ya[i2 + e] : yb[i2 + e]);
          const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
          const float own = __uint_as_float(c ? yb[i2 + e] : ya[i2 + e]);
          re[e] = c ? recv : own;
          im[e] = c ? own : recv;
          if (a.inverse) im[e] = -im[e];
        }
        if (a.write_complex)
          *reinterpret_cast<float4 *>(out + off + i2) = make_float4(re[0], im[0], re[1], im[1]);
        if (smp) {
          const float s0 = sq_sum_f(re[0], im[0]), s1 = sq_sum_f(re[1], im[1]);
          *reinterpret_cast<float2 *>(smp + off + i2) = make_float2(s0, s1);
          tmax = fmaxf(tmax, fmaxf(s0, s1));
        }
      }
    }
    if (smp && a.row_max) {
      unsigned kmax = __float_as_uint(tmax);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned y = __shfl_down_sync(0xffffffffu, kmax, o);
        kmax = y > kmax ? y : kmax;
      }
      if (lane == 0) atomicMax(reinterpret_cast<unsigned *>(a.row_max) + row, kmax);
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
  GS_CUDA(cudaMalloc(F, 3 * FT_PART_BYTES));
  tc_build_F_kernel<<<(TC_M * (TC_K / 2) + 255) / 256, 256>>>(static_cast<unsigned char *>(*F));
  GS_LAUNCHED();
  return GSFFT_OK;
}

int tc_build_F_smem(void **F) {
  GS_CUDA(cudaMalloc(F, 3 * A_BYTES));
  tc_build_F_smem_kernel<<<(TC_M * TC_K + 255) / 256, 256>>>(static_cast<unsigned char *>(*F));
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_tc64_last_pass(const TcPassArgs &a, cudaStream_t st) {
  // the last pass (Ns = N / 64), at least 128 sub-transforms per row, the
  // inter-pass twiddle tables of the pass, 16-byte aligned rows
  if (a.logN < 13 || a.logNs != a.logN - 6 || !a.tw_hi || !a.tw_lo || !a.F || a.nsum > 1)
    return GSFFT_ERR_UNSUPPORTED;
  if ((reinterpret_cast<uintptr_t>(a.in) & 15) || (reinterpret_cast<uintptr_t>(a.out) & 15) ||
      (reinterpret_cast<uintptr_t>(a.samples) & 7) || (a.bstride & 1) || (a.row_max && !a.samples))
    return GSFFT_ERR_UNSUPPORTED;
  static PerContext<int> attr;  // the kernel's dynamic shared memory limit, per context
  GS_CHECK(attr.ensure_at_least(T64_SMEM, [](int v) {
    if (cudaFuncSetAttribute(tc64_last_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, v) ==
        cudaSuccess)
      return (int)GSFFT_OK;
    set_last_error("tc64_last_pass_kernel: %d bytes of shared memory refused: %s", v,
                   cudaGetErrorString(cudaGetLastError()));
    return (int)GSFFT_ERR_CUDA;
  }));
  int dev = 0, sms = 0;
  GS_CUDA(cudaGetDevice(&dev));
  GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const long long ntiles = a.total >> 7;
  const long long grid = ntiles < sms ? ntiles : sms;
  if (grid < 1) return GSFFT_OK;
  tc64_last_pass_kernel<<<(int)grid, T64_THREADS, T64_SMEM, st>>>(a);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_tc4096_pass(const TcPassArgs &a, cudaStream_t st) {
  // first passes only (Ns = 1, outputs contiguous per sub-transform), at
  // least two sub-transforms per row (so a tile's pair shares a row) and
  // 16-byte aligned element pairs
  if (a.logNs != 0 || a.logN < 13 || !a.tw_R || !a.F || a.samples || a.row_max || !a.write_complex)
    return GSFFT_ERR_UNSUPPORTED;
  if ((reinterpret_cast<uintptr_t>(a.in) & 15) || (reinterpret_cast<uintptr_t>(a.out) & 15) ||
      (a.bstride & 1) || (a.nsum > 1 && (a.sstride & 1)) || a.nsum < 1 || (a.total & 1))
    return GSFFT_ERR_UNSUPPORTED;
  static PerContext<int> attr;  // the kernel's dynamic shared memory limit, per context
  GS_CHECK(attr.ensure_at_least(TQ_SMEM, [](int v) {
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
  // one CTA per SM (its shared memory allows no second), so that each holds
  // all 512 tensor-memory columns of its SM
  const long long ntiles = a.total / 2;
  const long long grid = ntiles < sms ? ntiles : sms;
  if (grid < 1) return GSFFT_OK;
  tc4096_pass_kernel<<<(int)grid, TQ_THREADS, TQ_SMEM, st>>>(a);
  GS_LAUNCHED();
  return GSFFT_OK;
}

}  // namespace gsfft
