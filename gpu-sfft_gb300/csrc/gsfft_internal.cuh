// Internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <mutex>

#include "gsfft.h"

namespace gsfft {

// ---------------------------------------------------------------- per-context set-up
// The calling thread's current CUDA context: its device ordinal and the
// driver's context id, which is unique for the life of the process (a context
// made after cudaDeviceReset gets a new one).
struct CtxKey {
  int dev = -1;
  unsigned long long id = 0;
  bool operator==(const CtxKey &o) const { return dev == o.dev && id == o.id; }
};
int current_ctx_key(CtxKey *out);

// One value per CUDA context, computed on first use in that context under a
// lock.  Function attributes, occupancy figures and symbol addresses belong
// to a context, so caching them process-wide would skip the set-up on a
// second device, or after a device reset.
template <typename T>
class PerContext {
 public:
  template <typename F>
  T get(F &&compute) {
    CtxKey k;
    if (current_ctx_key(&k) != 0) return compute();
    std::lock_guard<std::mutex> lock(mu_);
    for (int i = 0; i < n_; i++)
      if (keys_[i] == k) return vals_[i];
    const T v = compute();
    if (n_ < kSlots) {
      keys_[n_] = k;
      vals_[n_] = v;
      n_++;
    }
    return v;
  }
  // Calls set(want) unless this context already recorded a value >= want;
  // records want when set returns 0.  For grow-only attributes such as the
  // dynamic shared memory limit of a kernel.
  template <typename F>
  int ensure_at_least(T want, F &&set) {
    CtxKey k;
    if (current_ctx_key(&k) != 0) return set(want);
    std::lock_guard<std::mutex> lock(mu_);
    int i = 0;
    for (; i < n_; i++)
      if (keys_[i] == k) break;
    if (i < n_ && !(vals_[i] < want)) return 0;
    const int rc = set(want);
    if (rc == 0) {
      if (i < n_) {
        vals_[i] = want;
      } else if (n_ < kSlots) {
        keys_[n_] = k;
        vals_[n_] = want;
        n_++;
      }
    }
    return rc;
  }

 private:
  static constexpr int kSlots = 64;
  std::mutex mu_;
  CtxKey keys_[kSlots];
  T vals_[kSlots] = {};
  int n_ = 0;
};

// ---------------------------------------------------------------- errors
void set_last_error(const char *fmt, ...);

#define GS_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      ::gsfft::set_last_error("%s:%d %s: %s", __FILE__, __LINE__, #call,     \
                              cudaGetErrorString(e_));                       \
      return GSFFT_ERR_CUDA;                                                 \
    }                                                                        \
  } while (0)

#define GS_CHECK(call)                        \
  do {                                        \
    int s_ = (call);                          \
    if (s_ != GSFFT_OK) return s_;            \
  } while (0)

// Every kernel launch goes through this: checks the launch and counts it.
extern thread_local int g_launch_counter;
#define GS_LAUNCHED()                                                         \
  do {                                                                        \
    ++::gsfft::g_launch_counter;                                              \
    cudaError_t e_ = cudaGetLastError();                                      \
    if (e_ != cudaSuccess) {                                                  \
      ::gsfft::set_last_error("%s:%d launch: %s", __FILE__, __LINE__,         \
                              cudaGetErrorString(e_));                        \
      return GSFFT_ERR_CUDA;                                                  \
    }                                                                         \
  } while (0)

// ---------------------------------------------------------------- bounded waits
// Every wait of a kernel on an mbarrier (a TMA copy's or a tensor-core
// product's completion) gives up after `limit` SM clock cycles -- by default
// 2^30, about half a second at 2 GHz, far above any real completion -- and
// returns false, so that a kernel whose producer never arrives records an
// error and returns instead of hanging the GPU.
constexpr long long kWaitLimitCycles = 1LL << 30;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar_smem_addr, unsigned parity,
                                                  long long limit = kWaitLimitCycles) {
  const long long t0 = clock64();
  while (true) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(bar_smem_addr), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}
// launches the failure-detection self-check kernel (capi.cu: gsfft_check_bounded_wait)
int launch_bounded_wait_probe(long long limit, int *gave_up, cudaStream_t st);

// ---------------------------------------------------------------- launches
// Programmatic dependent launch.  The kernels of a run begin with pdl_enter():
// griddepcontrol.wait returns once the preceding grid of the stream has
// completed and its writes are visible (at once when the kernel was launched
// normally), then launch_dependents lets the next kernel be scheduled as soon
// as every block of this grid has passed its wait.  So only the launch of the
// next kernel overlaps this one; its blocks wait before touching memory, and a
// waiting grid never holds resources its predecessor still needs (all of the
// predecessor's blocks have started by then).
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch `kernel` as a programmatic dependent of the stream's previous kernel.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// ---------------------------------------------------------------- complex
template <typename T> struct Cx;
template <> struct Cx<double> { typedef double2 V; };
template <> struct Cx<float> { typedef float2 V; };

__host__ __device__ __forceinline__ double2 mk(double x, double y) { return make_double2(x, y); }
__host__ __device__ __forceinline__ float2 mk(float x, float y) { return make_float2(x, y); }

template <typename V> __device__ __forceinline__ V cadd(V a, V b) { V c; c.x = a.x + b.x; c.y = a.y + b.y; return c; }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { V c; c.x = a.x - b.x; c.y = a.y - b.y; return c; }
template <typename V> __device__ __forceinline__ V cconj(V a) { a.y = -a.y; return a; }
// (a.x b.x - a.y b.y, a.x b.y + a.y b.x), two fused operations per component.
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  V c;
  c.x = fma(a.x, b.x, -(a.y * b.y));
  c.y = fma(a.x, b.y, a.y * b.x);
  return c;
}

// Keys whose unsigned order equals the order of non-negative floats.
template <typename T> struct KeyOf;
template <> struct KeyOf<double> { typedef unsigned long long K; };
template <> struct KeyOf<float> { typedef unsigned int K; };

// ---------------------------------------------------------------- FFT
struct FftPlan {
  long long n = 0;         // transform size (power of two)
  int L = 0;               // log2 n
  int precision = 0;       // GSFFT_FP64 / GSFFT_MIXED (float)
  int npass = 0;
  int logR[3] = {0, 0, 0}; // radix of each pass (log2)
  // per pass: twiddle tables for exp(-2 pi i m / Np) with Np = prod radices
  // up to and including the pass, split as hi[m >> h] * lo[m & (2^h - 1)].
  void *tw_hi[3] = {nullptr, nullptr, nullptr};
  void *tw_lo[3] = {nullptr, nullptr, nullptr};
  int tw_h[3] = {0, 0, 0};
  void *tw_R[3] = {nullptr, nullptr, nullptr};  // exp(-2 pi i m / R) for the pass radix
  bool tc[3] = {false, false, false};  // pass runs on the tensor cores (radix 4096 or 64, FP32)
  void *tc_F = nullptr;                // DFT_64 operand of the tensor-core pass (its layout
                                       // follows the pass: tc_build_F / tc_build_F_smem)
  void *scratch = nullptr; // one transform-sized buffer per batch entry (multi-pass)
  long long scratch_elems = 0;
};

// One tensor-core pass of an FP32 FFT (tc_dft.cu): the radix-4096 first
// pass or the radix-64 last pass.
struct TcPassArgs {
  const void *in;       // float2
  void *out;            // float2
  int logN, logNs;
  long long bstride, total;  // row stride; sub-transforms over the batch
  int inverse;
  const void *tw_hi, *tw_lo;
  int tw_h;
  const void *F;        // three bf16 parts of the DFT_64 real form (tc_build_F)
  const void *tw_R;     // exp(-2 pi i m / 4096) for the radix-4096 form
  void *samples;        // float |X|^2 or null
  void *row_max;        // u32 bit pattern per row, with samples
  int write_complex;
  int *err;             // set when a completion wait timed out (may be null)
  int nsum = 1;         // radix-4096 form: add nsum partial inputs sstride apart
  long long sstride = 0;
};
int tc_build_F(void **F);
// radix 64 as the last pass (one DFT_64 product per 128 sub-transforms)
int tc_build_F_smem(void **F);
int launch_tc64_last_pass(const TcPassArgs &a, cudaStream_t st);
// radix 4096 = 64 x 64 in one pass (four-step, both DFT_64 stages on the tensor cores)
int launch_tc4096_pass(const TcPassArgs &a, cudaStream_t st);

// Optional fused prologue/epilogue of an FFT execution.
struct FftIo {
  // gather loader (first pass): element m of batch b is x[offs[b] + m * stride]
  const void *gather_x = nullptr;
  long long gather_offsets[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // one per batch entry (batch <= 8)
  long long gather_stride = 0;
  // first-pass loader alternative: element = sum over s < sum_rows of
  // in[s * sum_stride + index], added in s order (row-group partials)
  int sum_rows = 1;
  long long sum_stride = 0;
  // epilogue: |X|^2 (same precision) written to samples[b * n + k]
  void *samples = nullptr;
  // optional: per-row maximum of the samples (bit pattern, u64 for double /
  // u32 for float) accumulated with atomicMax; the caller zeroes it first
  void *row_max = nullptr;
  bool write_complex = true;
  // tensor-core passes: set when a completion wait timed out (may be null)
  int *err = nullptr;
};

// first_logr: log2 of the first pass's radix for two-pass sizes (0: ceil(L/2))
int fft_plan_init(FftPlan &p, long long n, int precision, int max_batch, int first_logr = 0);
// FP32 plan: radix-4096 tensor-core pass, then a CUDA-core pass of radix
// n / 4096; GSFFT_ERR_UNSUPPORTED unless n = 2^(17..26)
int fft_plan_init_tc(FftPlan &p, long long n, int max_batch);
// FP32 plan: CUDA-core radix-2^(L-6) first pass, tensor-core radix-64 last pass (13 <= L <= 20)
int fft_plan_init_tc64(FftPlan &p, long long n, int max_batch);
void fft_plan_free(FftPlan &p);
// in: batch entries at in + b*n; out: out + b*n.  sign -1 forward, +1 inverse.
int fft_exec(const FftPlan &p, const void *in, void *out, int batch, int sign,
             const FftIo &io, cudaStream_t st);
int fft_launches(const FftPlan &p);

// ---------------------------------------------------------------- select
// Top-`num` of each row by key (ties at the threshold: lowest index first),
// indices written ascending.  keys: double or float samples (bit patterns of
// non-negative values).  size either fixed (size_dev == nullptr) or read from
// *size_dev (rows then have capacity `size`, only the first *size_dev used;
// batch must be 1).  When the live size <= num, all live indices are taken.
struct SelectScratch {
  void *hist = nullptr;        // batch * 2048 uint32
  void *state = nullptr;       // batch * SelState
  void *tiles = nullptr;       // batch * max_tiles * 4 uint32
  void *coop_hist = nullptr;   // single-launch form: 6 passes x 8 rows x 2048 bins, zero between calls
  int max_batch = 0, max_tiles = 0;
  bool single_launch = true;   // cluster / cooperative form allowed (else multi-launch)
};
// Byte sizes of the SelectScratch regions for max_batch rows of at most
// max_size samples (what select_scratch_init allocates); state and coop_hist
// must hold zeros when a selection starts.
struct SelectScratchBytes {
  size_t hist, state, tiles, coop_hist;
  int max_tiles;
};
SelectScratchBytes select_scratch_bytes(int max_batch, long long max_size);
int select_scratch_init(SelectScratch &s, int max_batch, long long max_size);
void select_scratch_free(SelectScratch &s);
// row_max (optional, per row, bit pattern of the largest sample) with
// floor_rel > 0: samples below floor_rel * max are taken as exact zeros, so
// rounding-level samples tie and resolve by ascending index.
int select_top(const void *keys, int key_bytes, long long size, const int *size_dev,
               int num, int batch, long long row_stride, int *out, long long out_stride,
               int *count_out, SelectScratch &s, cudaStream_t st,
               const void *row_max = nullptr, double floor_rel = 0.0);

}  // namespace gsfft
