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
// FP64), never from recurrences.  Inverse = conj(DFT(conj(x))).
#include "gsfft_internal.cuh"

#include <algorithm>

namespace gsfft {

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
// whole warps in the butterfly stages), a pitch of 32/G 8-byte elements past
// a multiple of 16 makes the G x (32/G) lanes fill every bank pair exactly
// twice (two wavefronts) instead of colliding.
template <typename T> __host__ __device__ constexpr int rowpitch(int logr) {
  return padded(1 << logr) +
         ((sizeof(T) == 4 && g_of<T>(logr) >= 2 && g_of<T>(logr) <= 16 &&
           nt_of<T>(logr) / g_of<T>(logr) >= 32)
              ? 32 / g_of<T>(logr)
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

// One Stockham stage of radix E inside shared memory, for all G rows.
template <typename V, int LOGR, int G, int E>
__device__ __forceinline__ void smem_stage(V *sm, const V *__restrict__ twR, int Ns) {
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
__device__ __forceinline__ void cta_fft(V *sm, const V *__restrict__ twR) {
  constexpr int LEFT = LOGR % 4;
  int Ns = 1;
  if (LEFT == 1) { smem_stage<V, LOGR, G, 2>(sm, twR, Ns); Ns <<= 1; }
  if (LEFT == 2) { smem_stage<V, LOGR, G, 4>(sm, twR, Ns); Ns <<= 2; }
  if (LEFT == 3) { smem_stage<V, LOGR, G, 8>(sm, twR, Ns); Ns <<= 3; }
#pragma unroll 1
  for (int s = 0; s < LOGR / 4; s++) { smem_stage<V, LOGR, G, 16>(sm, twR, Ns); Ns <<= 4; }
}

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

template <typename T, int LOGR>
__global__ void __launch_bounds__(nt_of<T>(LOGR), minb_of<T>(LOGR)) fft_pass_kernel(PassArgs a) {
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
  __syncthreads();
  cta_fft<V, LOGR, G>(sm, twR);
  V *__restrict__ out = reinterpret_cast<V *>(a.out);
  T *__restrict__ smp = reinterpret_cast<T *>(a.samples);
  const bool g_fast_out = logNs >= 0 && (1 << logNs) >= G;
  // All G sub-transforms of the CTA lie in one batch row when S >= G; then each
  // thread keeps its own maximum and the CTA reduces once.  Otherwise every
  // warp's lanes hold one row per iteration (R >= 128 > 32).
  const bool one_row = (1LL << logS) >= G;
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

// exp(-2 pi i m / Np) for m in [0, count) at spacing `mul`
template <typename V>
__global__ void twiddle_table_kernel(V *t, long long count, long long mul, long long Np) {
  long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= count) return;
  double s, c;
  // angle 2*pi*(m*mul)/Np, reduced exactly in integers
  long long num = (m * mul) % Np;
  sincospi(2.0 * (double)num / (double)Np, &s, &c);
  t[m].x = (decltype(t[m].x))c;
  t[m].y = (decltype(t[m].y))(-s);
}

template <typename T>
int make_table(void **dst, long long count, long long mul, long long Np) {
  typedef typename Cx<T>::V V;
  GS_CUDA(cudaMalloc(dst, sizeof(V) * count));
  twiddle_table_kernel<V><<<(unsigned)((count + 255) / 256), 256>>>((V *)*dst, count, mul, Np);
  GS_LAUNCHED();
  return GSFFT_OK;
}

template <typename T, int LOGR>
int launch_pass(const PassArgs &a, long long total_sub, cudaStream_t st) {
  constexpr int G = g_of<T>(LOGR), NT = nt_of<T>(LOGR), SM = smem_of<T>(LOGR);
  static bool attr_done = false;  // per instantiation; idempotent if raced
  if (!attr_done) {
    GS_CUDA(cudaFuncSetAttribute(fft_pass_kernel<T, LOGR>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SM));
    attr_done = true;
  }
  long long grid = (total_sub + G - 1) / G;
  if (grid > 0x7fffffffLL) return GSFFT_ERR_UNSUPPORTED;
  fft_pass_kernel<T, LOGR><<<(unsigned)grid, NT, SM, st>>>(a);
  GS_LAUNCHED();
  return GSFFT_OK;
}

template <typename T>
int dispatch_pass(int logr, const PassArgs &a, long long total_sub, cudaStream_t st) {
  switch (logr) {
    case 5: return launch_pass<T, 5>(a, total_sub, st);
    case 6: return launch_pass<T, 6>(a, total_sub, st);
    case 7: return launch_pass<T, 7>(a, total_sub, st);
    case 8: return launch_pass<T, 8>(a, total_sub, st);
    case 9: return launch_pass<T, 9>(a, total_sub, st);
    case 10: return launch_pass<T, 10>(a, total_sub, st);
    case 11: return launch_pass<T, 11>(a, total_sub, st);
    case 12: return launch_pass<T, 12>(a, total_sub, st);
    case 13: return launch_pass<T, 13>(a, total_sub, st);
    case 14:
      if constexpr (sizeof(T) == 4) return launch_pass<T, 14>(a, total_sub, st);
      break;
    default: break;
  }
  return GSFFT_ERR_UNSUPPORTED;
}

}  // namespace

int fft_plan_init(FftPlan &p, long long n, int precision, int max_batch) {
  fft_plan_free(p);
  if (n < 256 || (n & (n - 1)) != 0) return GSFFT_ERR_UNSUPPORTED;
  int L = 0;
  while ((1LL << L) < n) L++;
  const int one_pass_max = precision == GSFFT_FP64 ? 13 : 14;
  p.n = n;
  p.L = L;
  p.precision = precision;
  if (L <= one_pass_max) {
    p.npass = 1;
    p.logR[0] = L;
  } else if (L <= 24) {
    p.npass = 2;
    p.logR[0] = (L + 1) / 2;
    p.logR[1] = L - p.logR[0];
  } else if (L <= 36) {
    p.npass = 3;
    p.logR[0] = (L + 2) / 3;
    p.logR[1] = (L - p.logR[0] + 1) / 2;
    p.logR[2] = L - p.logR[0] - p.logR[1];
  } else {
    return GSFFT_ERR_UNSUPPORTED;
  }
  for (int i = 0; i < p.npass; i++)
    if (p.logR[i] < 7 || p.logR[i] > one_pass_max) return GSFFT_ERR_UNSUPPORTED;
  const bool dbl = precision == GSFFT_FP64;
  long long Np = 1;
  for (int i = 0; i < p.npass; i++) {
    const long long R = 1LL << p.logR[i];
    Np *= R;
    int lg = 0;
    while ((1LL << lg) < Np) lg++;
    const int h = (lg + 1) / 2;
    p.tw_h[i] = h;
    const long long nlo = 1LL << h, nhi = (Np + nlo - 1) / nlo;
    if (dbl) {
      GS_CHECK(make_table<double>(&p.tw_lo[i], nlo, 1, Np));
      GS_CHECK(make_table<double>(&p.tw_hi[i], nhi, nlo, Np));
      GS_CHECK(make_table<double>(&p.tw_R[i], R, 1, R));
    } else {
      GS_CHECK(make_table<float>(&p.tw_lo[i], nlo, 1, Np));
      GS_CHECK(make_table<float>(&p.tw_hi[i], nhi, nlo, Np));
      GS_CHECK(make_table<float>(&p.tw_R[i], R, 1, R));
    }
  }
  if (p.npass > 1) {
    const size_t es = dbl ? 16 : 8;
    p.scratch_elems = (long long)n * max_batch * (p.npass == 3 ? 2 : 1);
    GS_CUDA(cudaMalloc(&p.scratch, es * p.scratch_elems));
  }
  GS_CUDA(cudaDeviceSynchronize());
  return GSFFT_OK;
}

// FP32 plan whose first pass is a radix-4096 tensor-core pass (two DFT_64
// stages; its outputs are then contiguous) and whose second is a CUDA-core
// pass of radix 2^(L-12): n = 2^L, 5 <= L-12 <= 14.
int fft_plan_init_tc(FftPlan &p, long long n, int max_batch) {
  fft_plan_free(p);
  if (n < 256 || (n & (n - 1)) != 0) return GSFFT_ERR_UNSUPPORTED;
  int L = 0;
  while ((1LL << L) < n) L++;
  if (L - 12 < 5 || L - 12 > 14) return GSFFT_ERR_UNSUPPORTED;
  p.n = n;
  p.L = L;
  p.precision = GSFFT_MIXED;
  p.npass = 2;
  p.logR[0] = 12;
  p.logR[1] = L - 12;
  p.tc[0] = true;
  p.tc[1] = false;
  long long Np = 1;
  for (int i = 0; i < p.npass; i++) {
    const long long R = 1LL << p.logR[i];
    Np *= R;
    int lg = 0;
    while ((1LL << lg) < Np) lg++;
    const int h = (lg + 1) / 2;
    p.tw_h[i] = h;
    const long long nlo = 1LL << h, nhi = (Np + nlo - 1) / nlo;
    GS_CHECK(make_table<float>(&p.tw_lo[i], nlo, 1, Np));
    GS_CHECK(make_table<float>(&p.tw_hi[i], nhi, nlo, Np));
    GS_CHECK(make_table<float>(&p.tw_R[i], R, 1, R));
  }
  GS_CHECK(tc_build_F(&p.tc_F));
  p.scratch_elems = (long long)n * max_batch;
  GS_CUDA(cudaMalloc(&p.scratch, sizeof(float2) * p.scratch_elems));
  GS_CUDA(cudaDeviceSynchronize());
  return GSFFT_OK;
}

void fft_plan_free(FftPlan &p) {
  for (int i = 0; i < 3; i++) {
    if (p.tw_hi[i]) cudaFree(p.tw_hi[i]);
    if (p.tw_lo[i]) cudaFree(p.tw_lo[i]);
    if (p.tw_R[i]) cudaFree(p.tw_R[i]);
    p.tw_hi[i] = p.tw_lo[i] = p.tw_R[i] = nullptr;
  }
  if (p.scratch) cudaFree(p.scratch);
  p.scratch = nullptr;
  if (p.tc_F) cudaFree(p.tc_F);
  p.tc_F = nullptr;
  for (int i = 0; i < 3; i++) p.tc[i] = false;
  p.npass = 0;
}

int fft_launches(const FftPlan &p) { return p.npass; }

int fft_exec(const FftPlan &p, const void *in, void *out, int batch, int sign,
             const FftIo &io, cudaStream_t st) {
  if (p.npass == 0) return GSFFT_ERR_STATE;
  const bool dbl = p.precision == GSFFT_FP64;
  const size_t es = dbl ? 16 : 8;
  if (p.npass > 1 && (long long)batch * p.n * (p.npass == 3 ? 2 : 1) > p.scratch_elems)
    return GSFFT_ERR_PARAM;
  if (io.gather_x && batch > 8) return GSFFT_ERR_PARAM;
  const void *src = in;
  char *scr = (char *)p.scratch;
  long long Ns = 1;
  for (int i = 0; i < p.npass; i++) {
    const bool last = i == p.npass - 1;
    void *dst;
    if (last) dst = out;
    else dst = scr + (size_t)(i == 1 ? 1 : 0) * es * p.n * batch;
    PassArgs a;
    a.in = src;
    a.out = dst;
    a.N = p.n;
    a.logN = p.L;
    {
      int l = 0;
      while ((1LL << l) < Ns) l++;
      a.logNs = l;
    }
    a.bstride = p.n;
    a.batch = batch;
    a.Ns = (int)Ns;
    a.inverse = sign > 0;
    a.tw_hi = p.tw_hi[i];
    a.tw_lo = p.tw_lo[i];
    a.tw_h = p.tw_h[i];
    a.twR = p.tw_R[i];
    a.gx = (i == 0) ? io.gather_x : nullptr;
    for (int q = 0; q < 8; q++) a.goffs[q] = io.gather_offsets[q];
    a.gstride = io.gather_stride;
    a.samples = last ? io.samples : nullptr;
    a.row_max = last ? io.row_max : nullptr;
    a.nsum = (i == 0) ? io.sum_rows : 1;
    a.sstride = io.sum_stride;
    a.write_complex = last ? (io.write_complex ? 1 : 0) : 1;
    const long long total_sub = (p.n >> p.logR[i]) * batch;
    a.total = total_sub;
    int s;
    if (p.tc[i]) {
      if (dbl || a.gx || p.logR[i] != 12) return GSFFT_ERR_UNSUPPORTED;  // partial sums, no gather
      TcPassArgs t;
      t.in = a.in;
      t.out = a.out;
      t.logN = a.logN;
      t.logNs = a.logNs;
      t.bstride = a.bstride;
      t.total = total_sub;
      t.inverse = a.inverse;
      t.tw_hi = a.tw_hi;
      t.tw_lo = a.tw_lo;
      t.tw_h = a.tw_h;
      t.F = p.tc_F;
      t.tw_R = p.tw_R[i];
      t.samples = a.samples;
      t.row_max = a.row_max;
      t.write_complex = a.write_complex;
      t.err = io.err;
      t.nsum = a.nsum;
      t.sstride = a.sstride;
      s = launch_tc4096_pass(t, st);
    } else {
      s = dbl ? dispatch_pass<double>(p.logR[i], a, total_sub, st)
              : dispatch_pass<float>(p.logR[i], a, total_sub, st);
    }
    if (s != GSFFT_OK) return s;
    src = dst;
    Ns <<= p.logR[i];
  }
  return GSFFT_OK;
}

}  // namespace gsfft
