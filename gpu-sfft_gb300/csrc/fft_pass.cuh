// Power-of-two complex FFT for sm_103a, FP64 and FP32, batched.
//
// Replaces the cuFFT Z2Z plans of the reference (innerLoop.cu:144-152 for the
// W_RLFC-point RLFC transform, :252-256 for the B-point bucket transform,
// cuExperiment.cu:305-308 / :362-365 / :425-426 for the filter design).
//
// Algorithm: Stockham auto-sort with one large radix R = 2^LOGR per global
// pass (1 pass up to 2^13 (FP64) / 2^14 (FP32) points, 2 passes up to 2^24,
// 3 passes beyond).  Pass p with Ns = product of the earlier radices:
//   v[r] = in[j + r*N/R] * exp(-2 pi i (j mod Ns) r / (Ns R));  V = DFT_R(v);
//   out[(j / Ns) Ns R + (j mod Ns) + k Ns] = V[k]
// Each CTA runs G sub-transforms of size R in shared memory as a Stockham
// sequence of radix-16 register stages (one radix-2/4/8 stage for the
// remainder).  G >= 2 (FP64) / 4 (FP32) so every strided global access moves
// whole 32-byte sectors.  Twiddles come from exact-angle tables (sincospi in
// FP64); FP64 looks every one up, FP32 builds some as products of a few
// looked-up ones (at most about eight roundings, never a long recurrence).
// Inverse = conj(DFT(conj(x))).
//
// This header holds the pass kernel; its instantiations are spread over
// fft_pass_*.cu so that they compile in parallel.
#pragma once
#include "gsfft_internal.cuh"

namespace gsfft {

struct PassArgs {
  const void *in;
  void *out;
  long long N;        // transform size
  int logN;           // log2 N
  int logNs;          // log2 of the product of the earlier radices
  long long bstride;  // batch stride of in/out/samples (elements)
  int batch;
  long long total;    // sub-transforms over the whole batch
  int Ns;
  int inverse;
  const void *tw_hi, *tw_lo;
  int tw_h;
  const void *twR;
  const void *gx;     // gather source (first pass only) or null
  long long goffs[8];
  long long gstride;
  void *samples;      // last pass only, or null
  void *row_max;      // per batch row, with samples
  int nsum;           // first pass: add nsum partial inputs sstride apart
  long long sstride;
  int write_complex;
};

// Launch one pass of radix 2^logr (each covers the radices listed).
int fft_pass_f32_lo(int logr, const PassArgs &a, long long total_sub, cudaStream_t st);  // 5..10
int fft_pass_f32_hi(int logr, const PassArgs &a, long long total_sub, cudaStream_t st);  // 11..14
int fft_pass_f64_lo(int logr, const PassArgs &a, long long total_sub, cudaStream_t st);  // 5..9
int fft_pass_f64_hi(int logr, const PassArgs &a, long long total_sub, cudaStream_t st);  // 10..13

namespace {

// cos / sin of 2 pi m / 16
__device__ __forceinline__ double c16d(int m) {
  const double t[8] = {1.0, 0.92387953251128675613, 0.70710678118654752440, 0.38268343236508977173,
                       0.0, -0.38268343236508977173, -0.70710678118654752440, -0.92387953251128675613};
  return t[m];
}
__device__ __forceinline__ double s16d(int m) {
  const double t[8] = {0.0, 0.38268343236508977173, 0.70710678118654752440, 0.92387953251128675613,
                       1.0, 0.92387953251128675613, 0.70710678118654752440, 0.38268343236508977173};
  return t[m];
}

// a * exp(-2 pi i m / 16), m in [0, 8) (compile-time after unrolling)
template <typename V> __device__ __forceinline__ V tw16(V a, int m) {
  typedef decltype(a.x) T;
  if (m == 0) return a;
  if (m == 4) { V r; r.x = a.y; r.y = -a.x; return r; }
  T c = (T)c16d(m), s = (T)s16d(m);
  V r;
  r.x = fma(a.x, c, a.y * s);
  r.y = fma(a.y, c, -(a.x * s));
  return r;
}

template <int E> __device__ __forceinline__ constexpr int bitrev(int k) {
  int r = 0;
  for (int b = 1; b < E; b <<= 1) { r = (r << 1) | (k & 1); k >>= 1; }
  return r;
}

// In-register forward DFT of E = 2,4,8,16 points (radix-2 DIF); the result
// X[k] is left in v[bitrev(k)].
template <typename V, int E> __device__ __forceinline__ void dft_reg(V *v) {
#pragma unroll
  for (int half = E / 2; half >= 1; half >>= 1) {
#pragma unroll
    for (int blk = 0; blk < E; blk += 2 * half) {
#pragma unroll
      for (int j = 0; j < half; j++) {
        V a = v[blk + j], b = v[blk + j + half];
        v[blk + j] = cadd(a, b);
        v[blk + j + half] = tw16(csub(a, b), j * (8 / half));
      }
    }
  }
}

__host__ __device__ constexpr int imin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int imax(int a, int b) { return a > b ? a : b; }

// sub-transforms per CTA
template <typename T> __host__ __device__ constexpr int g_of(int logr);
template <> __host__ __device__ constexpr int g_of<double>(int logr) {
  return logr >= 13 ? 1 : imax(2, 2048 >> logr);
}
template <> __host__ __device__ constexpr int g_of<float>(int logr) {
  return logr >= 14 ? 1 : (logr == 13 ? 2 : imax(4, 4096 >> logr));
}
template <typename T> __host__ __device__ constexpr int nt_of(int logr) {
  return imin(((1 << logr) / 16) * g_of<T>(logr), 512);
}
// Resident CTAs per SM the register budget is sized for, so that the loads,
// shared-memory butterflies and stores of different CTAs overlap.  A thread
// holds one radix-16 butterfly when (R/16)*G <= 512 (Q = 1); then FP32 fits
// 64 registers (two 512-thread CTAs) and FP64 128 (two 256-thread CTAs).
template <typename T> __host__ __device__ constexpr int minb_of(int logr) {
  return ((1 << logr) / 16) * g_of<T>(logr) > 512
             ? 1
             : (sizeof(T) == 4 ? (nt_of<T>(logr) >= 512 ? 2 : 4) : (nt_of<T>(logr) >= 512 ? 1 : 2));
}
__host__ __device__ constexpr int padded(int i) { return i + (i >> 4); }
// Row stride in elements.  Rows start in different banks; when a warp's load
// or store phase interleaves G rows (FP32, 2 <= G <= 16, each row handled by
// whole warps in the butterfly stages), a pitch of 16/G 8-byte elements past
// a multiple of 16 puts the G rows' runs of consecutive elements on disjoint
// bank pairs within each half-warp (16 lanes x 8 bytes = one wavefront), and
// fills every bank pair exactly twice over the whole warp.
template <typename T> __host__ __device__ constexpr int rowpitch(int logr) {
  return padded(1 << logr) +
         ((sizeof(T) == 4 && g_of<T>(logr) >= 2 && g_of<T>(logr) <= 16 &&
           nt_of<T>(logr) / g_of<T>(logr) >= 32)
              ? 16 / g_of<T>(logr)
              : 1);
}
// twiddle table exp(-2 pi i m / R) copied into shared memory when it fits
template <typename T> __host__ __device__ constexpr int data_smem_of(int logr) {
  return g_of<T>(logr) * rowpitch<T>(logr) * (int)sizeof(typename Cx<T>::V);
}
template <typename T> __host__ __device__ constexpr bool tw_in_smem(int logr) {
  return data_smem_of<T>(logr) + (1 << logr) * (int)sizeof(typename Cx<T>::V) <= 220 * 1024;
}
template <typename T> __host__ __device__ constexpr int smem_of(int logr) {
  return data_smem_of<T>(logr) +
         (tw_in_smem<T>(logr) ? (1 << logr) * (int)sizeof(typename Cx<T>::V) : 0);
}

// Inter-pass twiddles folded into the first shared-memory stage (FP32 passes
// after the first): the stage's inputs are conjugated (inverse) and
// multiplied by W^(jm r) in registers instead of in a separate read-modify-
// write of shared memory.  Element r = t + e NB of the row takes
//   W^(jm t) (W^(4 jm NB))^a (W^(jm NB))^b,  e = 4a + b,
// from three two-level table look-ups per thread and running products (at
// most about eight roundings).
struct PreTw {
  const float2 *thi, *tlo;
  int h, hmask;
  long long u0, Smask, Nsmask;
  int inverse;
  bool on;
};

__device__ __forceinline__ float2 tw_look(const PreTw &pt, long long mm) {
  return cmul(__ldg(&pt.thi[mm >> pt.h]), __ldg(&pt.tlo[mm & pt.hmask]));
}

template <typename V, int E, int Q, int NB, int TPF>
__device__ __forceinline__ void apply_pretw(V (&v)[Q][E], const PreTw &pt, int g, int t0) {
  if constexpr (sizeof(decltype(V().x)) == 4) {
    if (!pt.on) return;
    const long long jm = ((pt.u0 + g) & pt.Smask) & pt.Nsmask;
    const float2 s1 = tw_look(pt, jm * NB);
    float2 s4 = make_float2(1.f, 0.f);
    if constexpr (E >= 8) s4 = tw_look(pt, jm * 4 * NB);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      float2 wa = tw_look(pt, jm * (t0 + q * TPF)), w = wa;
#pragma unroll
      for (int e = 0; e < E; e++) {
        if (e > 0) {
          if ((e & 3) == 0) {
            wa = cmul(wa, s4);
            w = wa;
          } else {
            w = cmul(w, s1);
          }
        }
        V x = v[q][e];
        if (pt.inverse) x.y = -x.y;
        v[q][e] = cmul(x, w);
      }
    }
  }
}

// Twiddles of one radix-E butterfly of a Stockham stage: v[e] *= twR[k e step]
// (twR[m] = exp(-2 pi i m / R)).
template <typename V, int E>
__device__ __forceinline__ void stage_twiddles(V (&v)[E], const V *__restrict__ twR, int k, int step) {
  if constexpr (sizeof(v[0].x) == 8 || E < 4) {
    // FP64: exact table entries (its FP64 pipe, not shared memory, is the limit)
#pragma unroll
    for (int e = 1; e < E; e++) v[e] = cmul(v[e], twR[k * e * step]);
  } else {
    // FP32: two table reads (w, w^4), other powers by products at most four
    // deep -- the strided table reads were the shared-memory bank hot spot
    V w[E];
    w[1] = twR[k * step];
    w[2] = cmul(w[1], w[1]);
    w[3] = cmul(w[2], w[1]);
    w[4] = twR[4 * k * step];
#pragma unroll
    for (int e = 5; e < 8 && e < E; e++) w[e] = cmul(w[4], w[e - 4]);
    if constexpr (E == 16) {
      w[8] = cmul(w[4], w[4]);
#pragma unroll
      for (int e = 9; e < 12; e++) w[e] = cmul(w[8], w[e - 8]);
      w[12] = cmul(w[8], w[4]);
#pragma unroll
      for (int e = 13; e < 16; e++) w[e] = cmul(w[12], w[e - 12]);
    }
#pragma unroll
    for (int e = 1; e < E; e++) v[e] = cmul(v[e], w[e]);
  }
}

// One Stockham stage of radix E inside shared memory, for all G rows, after
// stages whose radices multiply to Ns = 2^LOGNS.  All strides are compile-time
// constants: with padded(i) = i + i/16, NB = R/E and t < NB,
//   padded(t + e NB)            = padded(t) + e NB + (e NB)/16
//   padded(hi Ns E + k + e Ns)  = padded(hi Ns E) + padded(k) + e Ns + (e Ns)/16
// (k < Ns, powers of two), so every shared-memory access of a butterfly is one
// base address plus an immediate offset.
template <typename V, int LOGR, int G, int E, int LOGNS>
__device__ __forceinline__ void smem_stage(V *sm, const V *__restrict__ twR, const PreTw &pt) {
  constexpr int R = 1 << LOGR;
  constexpr int RP = rowpitch<decltype(V().x)>(LOGR);
  constexpr int NT = imin((R / 16) * G, 512);
  constexpr int TPF = NT / G;
  constexpr int NB = R / E;          // butterflies per row
  constexpr int Q = NB / TPF;        // butterflies per thread
  constexpr int Ns = 1 << LOGNS;
  constexpr int LOGE = E == 2 ? 1 : (E == 4 ? 2 : (E == 8 ? 3 : 4));
  constexpr int step = R / (Ns * E);
  const int g = threadIdx.x / TPF, t0 = threadIdx.x % TPF;
  V *s = sm + g * RP;
  V v[Q][E];
  // a first stage with folded inter-pass twiddles loads all its inputs first
  const bool fold = LOGNS == 0 && pt.on;
  if (fold) {
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const V *rp = s + padded(t0 + q * TPF);
#pragma unroll
      for (int e = 0; e < E; e++) v[q][e] = rp[e * NB + ((e * NB) >> 4)];
    }
    apply_pretw<V, E, Q, NB, TPF>(v, pt, g, t0);
  }
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int t = t0 + q * TPF;
    if (!fold) {
      const V *rp = s + padded(t);
#pragma unroll
      for (int e = 0; e < E; e++) v[q][e] = rp[e * NB + ((e * NB) >> 4)];
    }
    if constexpr (LOGNS > 0) stage_twiddles<V, E>(v[q], twR, t & (Ns - 1), step);
    dft_reg<V, E>(v[q]);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int t = t0 + q * TPF;
    const int hi = t >> LOGNS, k = t & (Ns - 1);
    V *wp = s + padded(hi << (LOGNS + LOGE)) + padded(k);
#pragma unroll
    for (int e = 0; e < E; e++) wp[e * Ns + ((e * Ns) >> 4)] = v[q][bitrev<E>(e)];
  }
  __syncthreads();
}

// Radices up to 2^9 (G >= 8 rows per CTA): the same stages with Ns at run time
// in one loop -- fully inlined compile-time stages spill there under the
// 64-register budget of four resident CTAs.
template <typename V, int LOGR, int G, int E>
__device__ __forceinline__ void rt_smem_stage(V *sm, const V *__restrict__ twR, int Ns) {
  constexpr int R = 1 << LOGR;
  constexpr int RP = rowpitch<decltype(V().x)>(LOGR);
  constexpr int NT = imin((R / 16) * G, 512);
  constexpr int TPF = NT / G;
  constexpr int NB = R / E;          // butterflies per row
  constexpr int Q = NB / TPF;        // butterflies per thread
  const int g = threadIdx.x / TPF, t0 = threadIdx.x % TPF;
  V *s = sm + g * RP;
  V v[Q][E];
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int t = t0 + q * TPF;
#pragma unroll
    for (int e = 0; e < E; e++) v[q][e] = s[padded(t + e * NB)];
    if (Ns > 1) {
      const int k = t % Ns;
      const int step = R / (Ns * E);
      if (sizeof(v[0][0].x) == 8 || E < 4) {
        // FP64: exact table entries (its FP64 pipe, not shared memory, is the limit)
#pragma unroll
        for (int e = 1; e < E; e++) v[q][e] = cmul(v[q][e], twR[k * e * step]);
      } else {
        // FP32: two table reads (w, w^4), other powers by products at most four
        // deep -- the strided table reads were the shared-memory bank hot spot
        V w[E];
        w[1] = twR[k * step];
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
        w[4] = twR[4 * k * step];
#pragma unroll
        for (int e = 5; e < 8 && e < E; e++) w[e] = cmul(w[4], w[e - 4]);
        if (E == 16) {
          w[8] = cmul(w[4], w[4]);
#pragma unroll
          for (int e = 9; e < 12; e++) w[e] = cmul(w[8], w[e - 8]);
          w[12] = cmul(w[8], w[4]);
#pragma unroll
          for (int e = 13; e < 16; e++) w[e] = cmul(w[12], w[e - 12]);
        }
#pragma unroll
        for (int e = 1; e < E; e++) v[q][e] = cmul(v[q][e], w[e]);
      }
    }
    dft_reg<V, E>(v[q]);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int t = t0 + q * TPF;
    const int base = (t / Ns) * Ns * E + (t % Ns);
#pragma unroll
    for (int e = 0; e < E; e++) s[padded(base + e * Ns)] = v[q][bitrev<E>(e)];
  }
  __syncthreads();
}

template <typename V, int LOGR, int G>
__device__ __forceinline__ void rt_cta_fft(V *sm, const V *__restrict__ twR) {
  constexpr int LEFT = LOGR % 4;
  int Ns = 1;
  if (LEFT == 1) { rt_smem_stage<V, LOGR, G, 2>(sm, twR, Ns); Ns <<= 1; }
  if (LEFT == 2) { rt_smem_stage<V, LOGR, G, 4>(sm, twR, Ns); Ns <<= 2; }
  if (LEFT == 3) { rt_smem_stage<V, LOGR, G, 8>(sm, twR, Ns); Ns <<= 3; }
#pragma unroll 1
  for (int s = 0; s < LOGR / 4; s++) { rt_smem_stage<V, LOGR, G, 16>(sm, twR, Ns); Ns <<= 4; }
}

template <typename V, int LOGR, int G, int LOGNS>
__device__ __forceinline__ void radix16_stages(V *sm, const V *__restrict__ twR, const PreTw &pt) {
  if constexpr (LOGNS + 4 <= LOGR) {
    smem_stage<V, LOGR, G, 16, LOGNS>(sm, twR, pt);
    radix16_stages<V, LOGR, G, LOGNS + 4>(sm, twR, pt);
  }
}

template <typename V, int LOGR, int G>
__device__ __forceinline__ void cta_fft(V *sm, const V *__restrict__ twR, const PreTw &pt) {
  constexpr int LEFT = LOGR % 4;
  if constexpr (LEFT == 1) smem_stage<V, LOGR, G, 2, 0>(sm, twR, pt);
  if constexpr (LEFT == 2) smem_stage<V, LOGR, G, 4, 0>(sm, twR, pt);
  if constexpr (LEFT == 3) smem_stage<V, LOGR, G, 8, 0>(sm, twR, pt);
  radix16_stages<V, LOGR, G, LEFT>(sm, twR, pt);
}

// FP32 inter-pass twiddles W^(jm r), r = r0 + q TPF, q = 0, 1, ... in order,
// of one thread: three two-level table look-ups -- W^(jm r0), W^(jm TPF),
// W^(4 jm TPF) -- instead of one per element, then
//   w_q = A_(q/4) B_(q mod 4),  A_0 = W^(jm r0), A_m = A_(m-1) W^(4 jm TPF),
//   B_i = W^(i jm TPF),
// so w_q is within about q/4 + 4 roundings of its exact value (q < 32).
// Scattered table reads were the L1 limit of the pass; FP64 keeps exact
// per-element look-ups.
struct TwRun {
  float2 a, s4, b1, b2, b3;
  __device__ __forceinline__ static float2 look(const float2 *thi, const float2 *tlo, int h,
                                                int hmask, long long mm) {
    return cmul(thi[mm >> h], tlo[mm & hmask]);
  }
  __device__ __forceinline__ void init(const float2 *thi, const float2 *tlo, int h, int hmask,
                                       long long jm, int r0, int tpf) {
    b1 = look(thi, tlo, h, hmask, jm * tpf);
    s4 = look(thi, tlo, h, hmask, jm * 4 * tpf);
    a = look(thi, tlo, h, hmask, jm * r0);
    b2 = cmul(b1, b1);
    b3 = cmul(b2, b1);
  }
  // call with q = 0, 1, 2, ... (compile-time after unrolling)
  __device__ __forceinline__ float2 next(int q) {
    const int i = q & 3;
    if (q > 0 && i == 0) a = cmul(a, s4);
    return i == 0 ? a : cmul(a, i == 1 ? b1 : (i == 2 ? b2 : b3));
  }
};

__device__ __forceinline__ double sq_sum(double2 v) { return __dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)); }
__device__ __forceinline__ float sq_sum(float2 v) { return __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)); }

__device__ __forceinline__ unsigned long long key_bits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}
__device__ __forceinline__ unsigned key_bits(float v) { return __float_as_uint(v); }

// atomic max of a non-negative sample over a warp segment of one batch row
__device__ __forceinline__ void row_max_update(void *rm, long long b, double v) {
  unsigned long long k = (unsigned long long)__double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long y = __shfl_down_sync(0xffffffffu, k, o);
    k = y > k ? y : k;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long *>(rm) + b, k);
}
__device__ __forceinline__ void row_max_update(void *rm, long long b, float v) {
  unsigned k = __float_as_uint(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned y = __shfl_down_sync(0xffffffffu, k, o);
    k = y > k ? y : k;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned *>(rm) + b, k);
}

// ---------------------------------------------------------------- fused I/O
// FP32 radix 2^11 and 2^12 (G = 4 sub-transforms of one batch row per CTA,
// plain loads): the first stage takes its inputs straight from global memory
// into registers and the last stage stores its outputs straight to global
// memory, so every element passes through shared memory twice (once per
// inner stage boundary) instead of four times, and the load and store phases
// with their barriers are gone.  In both fused stages the lanes take the G
// sub-transforms fastest (g = tid % G): each warp load or store moves whole
// 32-byte sectors (G consecutive sub-transforms are adjacent on input, and
// on output once Ns >= G; with Ns = 1 each sub-transform's outputs are
// contiguous and 8 lanes write 64 bytes of it).
template <typename T> __host__ __device__ constexpr bool fused_io(int logr) {
  return sizeof(T) == 4 && (logr == 11 || logr == 12);
}

// Radix of the first stage of a radix-2^LOGR transform (the remainder stage).
template <int LOGR> __host__ __device__ constexpr int first_radix() {
  return LOGR % 4 == 0 ? 16 : (1 << (LOGR % 4));
}

// First stage (Ns = 1, radix E = first_radix): butterfly t of row g reads
// r = t + e NB, e < E, from src[r S] (src = the row's sub-transform j,
// S = 2^logS), applies the conjugation and inter-pass twiddles in registers
// and writes its outputs to shared memory.  Butterflies go to lanes so that
// the shared-memory stores of each half-warp hit 16 distinct bank pairs with
// the 16/G pitch, i.e. the half-warp's four butterflies fall on four
// consecutive pairs: for E = 16 (padded(16 t + e) = 17 t + e) four consecutive
// t; for E = 8 (padded(8 t + e) = 8 t + t/2 + e) four t of one parity (with
// consecutive t, t and t + 2 would share a pair).
template <typename V, int LOGR, int G>
__device__ __forceinline__ void fused_first_stage(V *sm, const V *__restrict__ src, int logS, const PreTw &pt,
                                                  int inverse) {
  constexpr int R = 1 << LOGR, E = first_radix<LOGR>();
  constexpr int LOGE = E == 2 ? 1 : (E == 4 ? 2 : (E == 8 ? 3 : 4));
  constexpr int NT = nt_of<float>(LOGR), TPF = NT / G, RP = rowpitch<float>(LOGR);
  constexpr int NB = R / E, Q = NB / TPF;
  static_assert(G == 4 && E >= 8 && Q * TPF == NB, "fused first stage: G = 4, radix 8 or 16");
  const int tid = threadIdx.x, g = tid % G;
  int t0;
  if constexpr (E == 8) {
    const int tl = (tid >> 2) & 7;  // lane / G
    t0 = (tid >> 5) * 8 + (((tl & 3) << 1) | (tl >> 2));
  } else {
    t0 = tid / G;
  }
  V v[Q][E];
  const V *p = src + ((long long)t0 << logS);
  const long long sq = (long long)TPF << logS, se = (long long)NB << logS;
#pragma unroll
  for (int q = 0; q < Q; q++)
#pragma unroll
    for (int e = 0; e < E; e++) v[q][e] = __ldg(p + q * sq + e * se);
  if (pt.on) {
    apply_pretw<V, E, Q, NB, TPF>(v, pt, g, t0);  // conjugates too when inverse
  } else if (inverse) {
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
      for (int e = 0; e < E; e++) v[q][e].y = -v[q][e].y;
  }
  V *s = sm + g * RP;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    dft_reg<V, E>(v[q]);
    // Stockham output of butterfly t (Ns = 1): positions t E + e, all in one
    // run of 16 (padded adds (t E) / 16 to each)
    V *wp = s + padded((t0 + q * TPF) << LOGE);
#pragma unroll
    for (int e = 0; e < E; e++) wp[e] = v[q][bitrev<E>(e)];
  }
}

// Inner stages: radix 16 after Ns = 2^LOGNS, up to the last stage.
template <typename V, int LOGR, int G, int LOGNS>
__device__ __forceinline__ void fused_mid_stages(V *sm, const V *__restrict__ twR, const PreTw &pt) {
  if constexpr (LOGNS + 4 < LOGR) {
    smem_stage<V, LOGR, G, 16, LOGNS>(sm, twR, pt);
    fused_mid_stages<V, LOGR, G, LOGNS + 4>(sm, twR, pt);
  }
}

// Last stage (radix 16, Ns = R/16): butterfly t of row g reads t + e NB from
// shared memory and gives X[t + e NB] of sub-transform j, stored at
// d0 + (t + e NB) Ns_global (complex and / or |X|^2 with the row maximum).
template <typename T, typename V, int LOGR, int G>
__device__ __forceinline__ void fused_last_stage(const V *sm, const V *__restrict__ twR, const PassArgs &a,
                                                 long long b, long long d0, int logNs) {
  constexpr int R = 1 << LOGR, E = 16;
  constexpr int NT = nt_of<T>(LOGR), TPF = NT / G, RP = rowpitch<T>(LOGR);
  constexpr int NB = R / E, Q = NB / TPF;
  static_assert(Q * TPF == NB, "fused last stage: whole butterflies per thread");
  const int tid = threadIdx.x, g = tid % G, t0 = tid / G;
  const V *s = sm + g * RP;
  V *__restrict__ out = reinterpret_cast<V *>(a.out);
  T *__restrict__ smp = reinterpret_cast<T *>(a.samples);
  T tmax = 0;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int t = t0 + q * TPF;
    V v[E];
    const V *rp = s + padded(t);
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = rp[e * NB + ((e * NB) >> 4)];
    stage_twiddles<V, E>(v, twR, t, 1);  // k = t mod Ns = t, step R / (Ns E) = 1
    dft_reg<V, E>(v);
#pragma unroll
    for (int e = 0; e < E; e++) {
      V x = v[bitrev<E>(e)];
      if (a.inverse) x.y = -x.y;
      const long long d = d0 + ((long long)(t + e * NB) << logNs);
      if (a.write_complex) out[d] = x;
      if (smp) {
        const T sv = sq_sum(x);
        smp[d] = sv;
        tmax = sv > tmax ? sv : tmax;
      }
    }
  }
  if (smp && a.row_max) row_max_update(a.row_max, b, tmax);
}

template <typename T, int LOGR>
__global__ void __launch_bounds__(nt_of<T>(LOGR), minb_of<T>(LOGR)) fft_pass_kernel(PassArgs a) {
  pdl_enter();
  typedef typename Cx<T>::V V;
  constexpr int R = 1 << LOGR, G = g_of<T>(LOGR), NT = nt_of<T>(LOGR), RP = rowpitch<T>(LOGR);
  constexpr int ITER = R * G / NT;  // elements per thread in the load / store phases
  extern __shared__ __align__(16) unsigned char smraw[];
  V *sm = reinterpret_cast<V *>(smraw);
  const V *twR = reinterpret_cast<const V *>(a.twR);
  if (tw_in_smem<T>(LOGR)) {
    V *tws = reinterpret_cast<V *>(smraw + data_smem_of<T>(LOGR));
    for (int i = threadIdx.x; i < R; i += NT) tws[i] = twR[i];
    twR = tws;  // made visible by the barrier before the first butterfly stage
  }
  const V *__restrict__ in = reinterpret_cast<const V *>(a.in);
  const V *__restrict__ gx = reinterpret_cast<const V *>(a.gx);
  const V *__restrict__ thi = reinterpret_cast<const V *>(a.tw_hi);
  const V *__restrict__ tlo = reinterpret_cast<const V *>(a.tw_lo);
  // all sizes are powers of two: S = N/R sub-transforms per batch entry
  const int logS = a.logN - LOGR;
  const long long Smask = (1LL << logS) - 1;
  const int logNs = a.logNs;
  const long long Nsmask = (1LL << logNs) - 1;
  const long long u0 = (long long)blockIdx.x * G;
  const int hmask = (1 << a.tw_h) - 1;
  const bool g_fast_in = logS >= 0 && (1LL << logS) >= G;
  // Fast layouts (at least G sub-transforms per batch row on input, Ns >= G on
  // output): thread tid owns sub-transform g = tid % G and rows r = tid/G + q TPF,
  // so its global addresses advance by one fixed stride and its shared-memory
  // offsets padded(r) = padded(tid/G) + q TPF + q TPF/16 are compile-time.
  constexpr int TPF = NT / G;
  const int tid = threadIdx.x;
  PreTw pt;
  pt.thi = reinterpret_cast<const float2 *>(thi);
  pt.tlo = reinterpret_cast<const float2 *>(tlo);
  pt.h = a.tw_h;
  pt.hmask = hmask;
  pt.u0 = u0;
  pt.Smask = Smask;
  pt.Nsmask = Nsmask;
  pt.inverse = a.inverse;
  // FP32 passes after the first fold the conjugation and the inter-pass
  // twiddles into their first stage (fast load path; radix 2^11 to 2^13, where
  // the first stage keeps its inputs in registers without spilling)
  pt.on = LOGR >= 11 && LOGR <= 13 && sizeof(T) == 4 && g_fast_in && !gx && a.nsum <= 1 &&
          logNs > 0;
  if constexpr (fused_io<T>(LOGR)) {
    // S >= G with both powers of two: the grid covers the batch exactly and
    // all G sub-transforms of a CTA lie in one batch row
    if (g_fast_in && !gx && a.nsum <= 1) {
      const long long u = u0 + tid % G;
      const long long b = u >> logS, j = u & Smask;
      PreTw ptf = pt;  // inter-pass twiddles in registers wherever Ns > 1
      ptf.on = logNs > 0;
      fused_first_stage<V, LOGR, G>(sm, in + b * a.bstride + j, logS, ptf, a.inverse);
      __syncthreads();
      fused_mid_stages<V, LOGR, G, (LOGR % 4 == 0 ? 4 : LOGR % 4)>(sm, twR, pt);
      const long long d0 = b * a.bstride + ((j >> logNs) << (logNs + LOGR)) + (j & Nsmask);
      fused_last_stage<T, V, LOGR, G>(sm, twR, a, b, d0, logNs);
      return;
    }
  }
  if (g_fast_in && !gx) {
    const int g = tid % G, r0 = tid / G;
    const long long u = u0 + g;
    V *dst = sm + g * RP + padded(r0);
    if (u >= a.total) {
#pragma unroll
      for (int q = 0; q < ITER; q++) dst[q * TPF + ((q * TPF) >> 4)] = mk((T)0, (T)0);
    } else {
      const long long b = u >> logS, j = u & Smask;
      const V *src = in + b * a.bstride + j + ((long long)r0 << logS);
      const long long qs = (long long)TPF << logS;
      const long long jm = j & Nsmask;
      const long long mm0 = jm * r0, dmm = jm * TPF;  // twiddle exponents, < Ns * R
      if (a.nsum <= 1) {
#pragma unroll
        for (int q = 0; q < ITER; q++)
          asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(
                           (unsigned)__cvta_generic_to_shared(dst + q * TPF + ((q * TPF) >> 4))),
                       "l"(src + q * qs), "n"(sizeof(V))
                       : "memory");
        asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
        if ((a.inverse || logNs > 0) && !pt.on) {
          // each thread rewrites only the elements it loaded: no barrier needed here
          TwRun tr;
          if constexpr (sizeof(T) == 4)
            if (logNs > 0)
              tr.init(reinterpret_cast<const float2 *>(thi), reinterpret_cast<const float2 *>(tlo),
                      a.tw_h, hmask, jm, r0, TPF);
#pragma unroll
          for (int q = 0; q < ITER; q++) {
            V *p = dst + q * TPF + ((q * TPF) >> 4);
            V v = *p;
            if (a.inverse) v.y = -v.y;
            if (logNs > 0) {
              if constexpr (sizeof(T) == 4) {
                v = cmul(v, tr.next(q));
              } else {
                const long long mm = mm0 + q * dmm;
                v = cmul(v, cmul(thi[mm >> a.tw_h], tlo[mm & hmask]));
              }
            }
            *p = v;
          }
        }
      } else {
        // row-group partials added on load (first pass after the streaming perm+filter)
        // (a first pass: logNs = 0 in practice, so per-element look-ups stay)
        constexpr int LB = ITER < 4 ? ITER : 4;
#pragma unroll
        for (int q0 = 0; q0 < ITER; q0 += LB) {
          V vbuf[LB];
#pragma unroll
          for (int q = 0; q < LB; q++) {
            const V *p = src + (q0 + q) * qs;
            V v = p[0];
            for (int s2 = 1; s2 < a.nsum; s2++) v = cadd(v, p[s2 * a.sstride]);
            vbuf[q] = v;
          }
#pragma unroll
          for (int q = 0; q < LB; q++) {
            V v = vbuf[q];
            if (a.inverse) v.y = -v.y;
            if (logNs > 0) {
              const long long mm = mm0 + (q0 + q) * dmm;
              v = cmul(v, cmul(thi[mm >> a.tw_h], tlo[mm & hmask]));
            }
            dst[(q0 + q) * TPF + (((q0 + q) * TPF) >> 4)] = v;
          }
        }
      }
    }
  } else {
    if (a.nsum <= 1) {
      // every element straight into shared memory with cp.async: all ITER loads
      // of a thread in flight, no registers held
#pragma unroll
      for (int q = 0; q < ITER; q++) {
        const int lt = threadIdx.x + q * NT;
        int g, r;
        if (g_fast_in) { g = lt % G; r = lt / G; } else { r = lt % R; g = lt / R; }
        const long long u = u0 + g;
        const long long b = u >> logS, j = u & Smask;
        const long long m = j + ((long long)r << logS);
        V *dst = &sm[g * RP + padded(r)];
        if (u >= a.total) {
          *dst = mk((T)0, (T)0);
        } else {
          const V *src = gx ? &gx[a.goffs[b] + m * a.gstride] : &in[b * a.bstride + m];
          asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                       "l"(src), "n"(sizeof(V))
                       : "memory");
        }
      }
      asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
      if (a.inverse || logNs > 0) {
        // each thread rewrites only the elements it loaded: no barrier needed here
#pragma unroll
        for (int q = 0; q < ITER; q++) {
          const int lt = threadIdx.x + q * NT;
          int g, r;
          if (g_fast_in) { g = lt % G; r = lt / G; } else { r = lt % R; g = lt / R; }
          V *p = &sm[g * RP + padded(r)];
          V v = *p;
          if (a.inverse) v.y = -v.y;
          if (logNs > 0) {
            const long long j = (u0 + g) & Smask;
            const long long mm = (j & Nsmask) * r;  // < Ns * R
            V w = cmul(thi[mm >> a.tw_h], tlo[mm & hmask]);
            v = cmul(v, w);
          }
          *p = v;
        }
      }
    } else {
      // row-group partials added on load (first pass after the streaming perm+filter)
      constexpr int LB = ITER < 4 ? ITER : 4;
#pragma unroll
      for (int q0 = 0; q0 < ITER; q0 += LB) {
        V vbuf[LB];
#pragma unroll
        for (int q = 0; q < LB; q++) {
          const int lt = threadIdx.x + (q0 + q) * NT;
          int g, r;
          if (g_fast_in) { g = lt % G; r = lt / G; } else { r = lt % R; g = lt / R; }
          const long long u = u0 + g;
          const long long b = u >> logS, j = u & Smask;
          const long long m = j + ((long long)r << logS);
          V v = mk((T)0, (T)0);
          if (u < a.total) {
            const long long idx = b * a.bstride + m;
            v = in[idx];
            for (int s2 = 1; s2 < a.nsum; s2++) v = cadd(v, in[idx + s2 * a.sstride]);
          }
          vbuf[q] = v;
        }
#pragma unroll
        for (int q = 0; q < LB; q++) {
          const int lt = threadIdx.x + (q0 + q) * NT;
          int g, r;
          if (g_fast_in) { g = lt % G; r = lt / G; } else { r = lt % R; g = lt / R; }
          V v = vbuf[q];
          if (a.inverse) v.y = -v.y;
          if (logNs > 0) {
            const long long j = (u0 + g) & Smask;
            const long long mm = (j & Nsmask) * r;
            V w = cmul(thi[mm >> a.tw_h], tlo[mm & hmask]);
            v = cmul(v, w);
          }
          sm[g * RP + padded(r)] = v;
        }
      }
    }
  }
  __syncthreads();
  if constexpr (LOGR <= 9) rt_cta_fft<V, LOGR, G>(sm, twR);
  else cta_fft<V, LOGR, G>(sm, twR, pt);
  V *__restrict__ out = reinterpret_cast<V *>(a.out);
  T *__restrict__ smp = reinterpret_cast<T *>(a.samples);
  const bool g_fast_out = logNs >= 0 && (1LL << logNs) >= G;
  // All G sub-transforms of the CTA lie in one batch row when S >= G; then each
  // thread keeps its own maximum and the CTA reduces once.  Otherwise every
  // warp's lanes hold one row per iteration (R >= 128 > 32).
  const bool one_row = (1LL << logS) >= G;
  const bool want_max = smp && a.row_max;
  if (g_fast_out && (one_row || !want_max)) {
    const int g = tid % G, k0 = tid / G;
    const long long u = u0 + g;
    T tmax = 0;
    if (u < a.total) {
      const long long b = u >> logS, j = u & Smask;
      const long long d0 = b * a.bstride + ((j >> logNs) << (logNs + LOGR)) + (j & Nsmask) +
                           ((long long)k0 << logNs);
      const long long ds = (long long)TPF << logNs;
      const V *sp = sm + g * RP + padded(k0);
#pragma unroll 4
      for (int q = 0; q < ITER; q++) {
        V v = sp[q * TPF + ((q * TPF) >> 4)];
        if (a.inverse) v.y = -v.y;
        const long long d = d0 + q * ds;
        if (a.write_complex) out[d] = v;
        if (smp) {
          const T sv = sq_sum(v);
          smp[d] = sv;
          tmax = sv > tmax ? sv : tmax;
        }
      }
    }
    if (want_max && u0 < a.total) row_max_update(a.row_max, u0 >> logS, tmax);
  } else {
    T tmax = 0;
#pragma unroll 4
    for (int q = 0; q < ITER; q++) {
      const int lt = threadIdx.x + q * NT;
      int g, k;
      if (g_fast_out) { g = lt % G; k = lt / G; } else { k = lt % R; g = lt / R; }
      const long long u = u0 + g;
      const bool live = u < a.total;
      const long long b = u >> logS, j = u & Smask;
      T sv = 0;
      if (live) {
        const long long dest = ((j >> logNs) << (logNs + LOGR)) + (j & Nsmask) + ((long long)k << logNs);
        V v = sm[g * RP + padded(k)];
        if (a.inverse) v.y = -v.y;
        if (a.write_complex) out[b * a.bstride + dest] = v;
        if (smp) {
          sv = sq_sum(v);
          smp[b * a.bstride + dest] = sv;
        }
      }
      if (smp && a.row_max) {
        if (one_row) {
          tmax = sv > tmax ? sv : tmax;
        } else {
          const long long bb = __shfl_sync(0xffffffffu, b, 0);
          const bool uniform = __all_sync(0xffffffffu, b == bb && live);
          if (uniform) row_max_update(a.row_max, bb, sv);
          else if (live) atomicMax(reinterpret_cast<typename KeyOf<T>::K *>(a.row_max) + b, key_bits(sv));
        }
      }
    }
    if (smp && a.row_max && one_row && u0 < a.total) row_max_update(a.row_max, u0 >> logS, tmax);
  }
}
template <typename T, int LOGR>
int launch_pass(const PassArgs &a, long long total_sub, cudaStream_t st) {
  constexpr int G = g_of<T>(LOGR), NT = nt_of<T>(LOGR), SM = smem_of<T>(LOGR);
  static PerContext<int> attr;  // per instantiation and CUDA context
  GS_CHECK(attr.ensure_at_least(SM, [](int v) {
    if (cudaFuncSetAttribute(fft_pass_kernel<T, LOGR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             v) == cudaSuccess)
      return (int)GSFFT_OK;
    set_last_error("fft_pass_kernel: %d bytes of shared memory refused: %s", v,
                   cudaGetErrorString(cudaGetLastError()));
    return (int)GSFFT_ERR_CUDA;
  }));
  long long grid = (total_sub + G - 1) / G;
  if (grid > 0x7fffffffLL) return GSFFT_ERR_UNSUPPORTED;
  GS_CUDA(launch_pdl(fft_pass_kernel<T, LOGR>, dim3((unsigned)grid), dim3(NT), SM, st, a));
  GS_LAUNCHED();
  return GSFFT_OK;
}
}  // namespace

}  // namespace gsfft
