// gsfft_cutoff_noalloc: the cutoff of gsfft_cutoff with its scratch in a
// fixed device array of this library instead of cudaMalloc'd buffers.
//
// Who needs it: a caller that must not allocate device memory while it runs.
// cudaMalloc / cudaFree can block until the whole device is idle (stalling
// every other stream of the process), and an allocation can fail when another
// allocator of the process (a framework's caching pool, for instance) already
// holds the free HBM.  Serving loops with latency budgets and callers whose
// memory is fully reserved up front cannot take either risk; they pass their
// own input and output buffers and this entry point touches nothing else but
// the array below.
//
// The array is shared by every call in the process on a device and keeps
// whatever the previous call left in it.  Each call clears the parts that the
// selection needs to start at zero (the per-row state and the single-launch
// histograms) on the caller's stream before its kernels run.  Calls on one
// stream are ordered; calls that can overlap in time (different streams,
// different host threads without ordering) race on the array and give
// undefined results.
#include "gsfft_internal.cuh"

#include <mutex>

namespace gsfft {

size_t select_state_bytes();

namespace {

// Scratch layout (bytes), sized for GSFFT_NOALLOC_MAX_BATCH rows of at most
// GSFFT_NOALLOC_MAX_SIZE samples:
//   hist       rows x 2048 bins x 4             (multi-launch radix passes)
//   state      rows x per-row selection state   (1 KiB reserved)
//   coop_hist  6 passes x 8 rows x 2048 x 4     (single-launch form; zero on entry)
//   tiles      rows x (max_size / 4096) x 4 x 4 (per-tile counts)
constexpr size_t kTile = 4096;  // samples per selection tile
constexpr size_t kMaxTiles = (GSFFT_NOALLOC_MAX_SIZE + kTile - 1) / kTile;
constexpr size_t kHistOff = 0;
constexpr size_t kHistBytes = (size_t)GSFFT_NOALLOC_MAX_BATCH * 2048 * 4;
constexpr size_t kStateOff = kHistOff + kHistBytes;
constexpr size_t kStateBytes = 1024;
constexpr size_t kCoopOff = kStateOff + kStateBytes;
constexpr size_t kCoopBytes = (size_t)6 * 8 * 2048 * 4;
constexpr size_t kTilesOff = kCoopOff + kCoopBytes;
constexpr size_t kTilesBytes = (size_t)GSFFT_NOALLOC_MAX_BATCH * kMaxTiles * 4 * 4;
constexpr size_t kScratchBytes = kTilesOff + kTilesBytes;
static_assert(kScratchBytes <= (size_t)1 << 20, "no-alloc scratch exceeds 1 MiB");
static_assert(kStateOff % 256 == 0 && kCoopOff % 256 == 0 && kTilesOff % 256 == 0,
              "scratch regions must stay 256-byte aligned");

// One copy per device (a __device__ variable lives in every device's module).
static __device__ __align__(256) unsigned char g_cutoff_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_cutoff_scratch on the current device, looked up once per
// device (the first call on a device makes the lookup, which may load this
// library's device code onto that device).
int scratch_address(void **out) {
  int dev = 0;
  GS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_last_error("gsfft_cutoff_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
    return GSFFT_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_cutoff_scratch);
    if (e != cudaSuccess || !p) {
      set_last_error("gsfft_cutoff_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                     cudaGetErrorString(e));
      return GSFFT_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return GSFFT_OK;
}

}  // namespace

}  // namespace gsfft

using namespace gsfft;

extern "C" int gsfft_cutoff_noalloc(const void *d_samples, int size, int num, int batch,
                                    int precision, int *d_out, void *stream) {
  if (!d_samples || !d_out || size < 1 || num < 1 || num >= size || batch < 1 ||
      (precision != GSFFT_FP64 && precision != GSFFT_MIXED))
    return GSFFT_ERR_PARAM;
  if (size > GSFFT_NOALLOC_MAX_SIZE || batch > GSFFT_NOALLOC_MAX_BATCH) {
    set_last_error("gsfft_cutoff_noalloc: %d rows of %d samples exceed the fixed scratch "
                   "(at most %d rows of %d samples)",
                   batch, size, GSFFT_NOALLOC_MAX_BATCH, GSFFT_NOALLOC_MAX_SIZE);
    return GSFFT_ERR_CAPACITY;
  }
  if (select_state_bytes() * GSFFT_NOALLOC_MAX_BATCH > kStateBytes) {
    set_last_error("gsfft_cutoff_noalloc: selection state outgrew its scratch region");
    return GSFFT_ERR_UNSUPPORTED;
  }
  void *base = nullptr;
  GS_CHECK(scratch_address(&base));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  unsigned char *b = static_cast<unsigned char *>(base);
  SelectScratch ss;
  ss.hist = b + kHistOff;
  ss.state = b + kStateOff;
  ss.coop_hist = b + kCoopOff;
  ss.tiles = b + kTilesOff;
  ss.max_batch = GSFFT_NOALLOC_MAX_BATCH;
  ss.max_tiles = (int)kMaxTiles;
  // what the selection expects to find zeroed; the rest is written before it is read
  GS_CUDA(cudaMemsetAsync(ss.state, 0, kStateBytes, st));
  GS_CUDA(cudaMemsetAsync(ss.coop_hist, 0, kCoopBytes, st));
  // The SelectScratch does not own the array: it is never passed to
  // select_scratch_free.
  return select_top(d_samples, precision == GSFFT_FP64 ? 8 : 4, size, nullptr, num, batch, size,
                    d_out, num, nullptr, ss, st);
}
