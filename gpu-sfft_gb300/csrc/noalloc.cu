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

namespace gsfft {

namespace {

// The array is sized for GSFFT_NOALLOC_MAX_BATCH rows of at most
// GSFFT_NOALLOC_MAX_SIZE samples.  Its regions are laid out at run time from
// the selection's own size query (select_scratch_bytes), and every call
// checks that they fit, so a change to the selection's scratch needs cannot
// overrun the array: such a call returns GSFFT_ERR_UNSUPPORTED instead.
constexpr size_t kScratchBytes = (size_t)1 << 20;
constexpr size_t kAlign = 256;

// One copy per device (a __device__ variable lives in every device's module).
static __device__ __align__(256) unsigned char g_cutoff_scratch[kScratchBytes];

struct Layout {
  size_t hist, state, coop, tiles, end;
  SelectScratchBytes b;
};

size_t round_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

Layout layout() {
  Layout L;
  L.b = select_scratch_bytes(GSFFT_NOALLOC_MAX_BATCH, GSFFT_NOALLOC_MAX_SIZE);
  L.hist = 0;
  L.state = round_up(L.hist + L.b.hist);
  L.coop = round_up(L.state + L.b.state);
  L.tiles = round_up(L.coop + L.b.coop_hist);
  L.end = L.tiles + L.b.tiles;
  return L;
}

// Device address of g_cutoff_scratch in the current context, looked up once
// per context (the first call in a context makes the lookup, which may load
// this library's device code there).  Keyed by context, not only by device,
// so that a context made after cudaDeviceReset gets its own address.
int scratch_address(void **out) {
  static PerContext<void *> cache;
  const char *err = nullptr;
  cudaError_t e = cudaSuccess;
  void *p = cache.get([&]() -> void * {
    void *a = nullptr;
    e = cudaGetSymbolAddress(&a, g_cutoff_scratch);
    if (e != cudaSuccess || !a) {
      err = "cudaGetSymbolAddress failed";
      return nullptr;
    }
    return a;
  });
  if (!p) {
    // a failed lookup is cached as nullptr for that context: report it
    set_last_error("gsfft_cutoff_noalloc: %s: %s", err ? err : "no device address for the scratch",
                   cudaGetErrorString(e));
    return GSFFT_ERR_CUDA;
  }
  *out = p;
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
  const Layout L = layout();
  if (L.end > kScratchBytes) {
    set_last_error("gsfft_cutoff_noalloc: the selection needs %zu bytes of scratch, the fixed "
                   "array holds %zu", L.end, kScratchBytes);
    return GSFFT_ERR_UNSUPPORTED;
  }
  void *base = nullptr;
  GS_CHECK(scratch_address(&base));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  unsigned char *b = static_cast<unsigned char *>(base);
  SelectScratch ss;
  ss.hist = b + L.hist;
  ss.state = b + L.state;
  ss.coop_hist = b + L.coop;
  ss.tiles = b + L.tiles;
  ss.max_batch = GSFFT_NOALLOC_MAX_BATCH;
  ss.max_tiles = L.b.max_tiles;
  // what the selection expects to find zeroed; the rest is written before it is read
  GS_CUDA(cudaMemsetAsync(ss.state, 0, L.b.state, st));
  GS_CUDA(cudaMemsetAsync(ss.coop_hist, 0, L.b.coop_hist, st));
  // The SelectScratch does not own the array: it is never passed to
  // select_scratch_free.
  return select_top(d_samples, precision == GSFFT_FP64 ? 8 : 4, size, nullptr, num, batch, size,
                    d_out, num, nullptr, ss, st);
}
