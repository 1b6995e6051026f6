// Signal ingest, device memory helpers and device-side evaluation.
//
// Ingest (the H2D path of cuExperiment.cu:113-122): the reference copies the
// FP64 signal with one synchronous cudaMemcpy from pageable memory.  Here a
// host signal is moved through two pinned staging chunks (the CPU fills one
// while the copy engine drains the other) and, for the mixed engine,
// converted to {float, float} on the device chunk by chunk, all on the
// caller's stream so it can overlap the previous signal's sparse FFT.
//
// Evaluation (run_experiment, cuExperiment.cu:178-216): MISSED (estimation,
// result) and MSE*k = sum_i |xhat_k[i] - x_f[i]|^2 over all n bins, where
// xhat_k holds the k largest estimates and x_f is the normalised DFT of the
// signal, computed on the device from the plan's last run instead of dense
// host arrays.
#include "engine.cuh"

#include <string.h>

#include <mutex>

namespace gsfft {

namespace {

constexpr size_t CHUNK = (size_t)2 << 20;  // complex_t samples per staging chunk (32 MiB)

__global__ void to_float_kernel(const double2 *__restrict__ in, float2 *out, long long n) {
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i < n) {
    const double2 v = in[i];
    out[i] = make_float2((float)v.x, (float)v.y);
  }
}

// Pinned staging ring and device-side FP64 staging, created on first use.
struct Staging {
  std::mutex mu;
  complex_t *host[2] = {nullptr, nullptr};
  double2 *dev[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  int device = -1;
};
Staging g_stage;

int staging_init(Staging &s) {
  int dev = 0;
  GS_CUDA(cudaGetDevice(&dev));
  if (s.device == dev && s.host[0]) return GSFFT_OK;
  if (s.device >= 0 && s.device != dev) {
    set_last_error("gsfft_ingest: staging buffers belong to device %d", s.device);
    return GSFFT_ERR_UNSUPPORTED;
  }
  for (int b = 0; b < 2; b++) {
    GS_CUDA(cudaHostAlloc(&s.host[b], CHUNK * sizeof(complex_t), cudaHostAllocPortable));
    GS_CUDA(cudaMalloc(&s.dev[b], CHUNK * sizeof(double2)));
    GS_CUDA(cudaEventCreateWithFlags(&s.done[b], cudaEventDisableTiming));
  }
  s.device = dev;
  return GSFFT_OK;
}

bool is_pinned(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Deterministic sum of |x_f[i]|^2 (block partials, then one block).
__global__ void energy_partial_kernel(const double2 *__restrict__ xf, long long n, double *part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n; i += (long long)gridDim.x * 256) {
    const double2 v = xf[i];
    s += v.x * v.x + v.y * v.y;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// One block: top-k hits, the top-k correction of the energy, and the
// candidate hits read from the vote table (epoch-tagged entries, or 2-bit
// counters when packed).
__global__ void evaluate_kernel(const DevNode *__restrict__ topk, const int *n_topk,
                                const int *__restrict__ tloc, int k_true, const double2 *__restrict__ xf,
                                const unsigned *__restrict__ vote, unsigned epoch, unsigned thresh,
                                int packed /* n when packed, else 0 */, const double *part, int nparts,
                                double *out /* err, found_est, found_res */) {
  __shared__ double sd[1024];
  __shared__ int si[1024], sr[1024];
  const int t = threadIdx.x;
  double e = 0.0;
  for (int i = t; i < nparts; i += 1024) e += part[i];
  int found_res = 0;
  const int nt = *n_topk;
  for (int i = t; i < nt; i += 1024) {
    const DevNode nd = topk[i];
    const double2 x = xf[nd.key];
    const double dx = nd.x - x.x, dy = nd.y - x.y;
    e += dx * dx + dy * dy - (x.x * x.x + x.y * x.y);
    // binary search of the key among the sorted true locations
    int lo = 0, hi = k_true;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (tloc[mid] < (int)nd.key) lo = mid + 1;
      else hi = mid;
    }
    found_res += (lo < k_true && tloc[lo] == (int)nd.key) ? 1 : 0;
  }
  int found_est = 0;
  for (int i = t; i < k_true; i += 1024) {
    const unsigned loc = (unsigned)tloc[i];
    if (packed) {
      // this run's table of the two (epoch & 1)
      const unsigned *tab = vote + ((epoch & 1u) ? ((unsigned)packed >> 4) : 0u);
      found_est += ((tab[loc >> 4] >> (2 * (loc & 15u))) & 3u) >= thresh ? 1 : 0;
    } else {
      const unsigned v = vote[loc];
      found_est += ((v >> 8) == epoch && (v & 255u) >= thresh) ? 1 : 0;
    }
  }
  sd[t] = e;
  si[t] = found_est;
  sr[t] = found_res;
  __syncthreads();
  for (int o = 512; o > 0; o >>= 1) {
    if (t < o) {
      sd[t] += sd[t + o];
      si[t] += si[t + o];
      sr[t] += sr[t + o];
    }
    __syncthreads();
  }
  if (t == 0) {
    out[0] = sd[0];
    out[1] = (double)si[0];
    out[2] = (double)sr[0];
  }
}

}  // namespace

int launch_to_float(const complex_t *in, void *out, long long n, cudaStream_t st) {
  if (n <= 0) return GSFFT_OK;
  to_float_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const double2 *)in, (float2 *)out, n);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int ingest(const complex_t *h_x, long long n, int precision, void *d_x, cudaStream_t st) {
  if (precision == GSFFT_FP64 && is_pinned(h_x)) {
    GS_CUDA(cudaMemcpyAsync(d_x, h_x, sizeof(complex_t) * (size_t)n, cudaMemcpyHostToDevice, st));
    return GSFFT_OK;
  }
  std::lock_guard<std::mutex> lock(g_stage.mu);
  GS_CHECK(staging_init(g_stage));
  for (long long off = 0, c = 0; off < n; off += (long long)CHUNK, c++) {
    const int b = (int)(c & 1);
    const size_t len = (size_t)((n - off) < (long long)CHUNK ? (n - off) : (long long)CHUNK);
    // the copy that last used this staging pair must be done before refilling it
    GS_CUDA(cudaEventSynchronize(g_stage.done[b]));
    memcpy(g_stage.host[b], h_x + off, len * sizeof(complex_t));
    if (precision == GSFFT_FP64) {
      GS_CUDA(cudaMemcpyAsync(reinterpret_cast<complex_t *>(d_x) + off, g_stage.host[b],
                              len * sizeof(complex_t), cudaMemcpyHostToDevice, st));
    } else {
      GS_CUDA(cudaMemcpyAsync(g_stage.dev[b], g_stage.host[b], len * sizeof(complex_t),
                              cudaMemcpyHostToDevice, st));
      GS_CHECK(launch_to_float((const complex_t *)g_stage.dev[b],
                               reinterpret_cast<float2 *>(d_x) + off, (long long)len, st));
    }
    GS_CUDA(cudaEventRecord(g_stage.done[b], st));
  }
  return GSFFT_OK;
}

int plan_evaluate(Plan *P, const complex_t *d_xf, const int *d_true_loc, int k_true,
                  int *missed_est, int *missed_res, double *err, cudaStream_t st) {
  if (!P->ran) return GSFFT_ERR_STATE;
  const long long n = P->p.n;
  const int parts = 152 * 8;
  double *buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * (parts + 3)) != cudaSuccess) return GSFFT_ERR_ALLOC;
  int s = GSFFT_OK;
  energy_partial_kernel<<<parts, 256, 0, st>>>((const double2 *)d_xf, n, buf);
  if (cudaGetLastError() != cudaSuccess) s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) {
    evaluate_kernel<<<1, 1024, 0, st>>>(P->topk, &P->ctl->n_topk, d_true_loc, k_true,
                                        (const double2 *)d_xf, P->vote, P->epoch,
                                        (unsigned)P->p.loops_thresh, P->packed_vote ? P->p.n : 0, buf,
                                        parts, buf + parts);
    if (cudaGetLastError() != cudaSuccess) s = GSFFT_ERR_CUDA;
  }
  double h[3] = {0, 0, 0};
  if (s == GSFFT_OK &&
      cudaMemcpyAsync(h, buf + parts, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK && cudaStreamSynchronize(st) != cudaSuccess) s = GSFFT_ERR_CUDA;
  if (s == GSFFT_ERR_CUDA) set_last_error("gsfft_evaluate: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(buf);
  if (s != GSFFT_OK) return s;
  if (err) *err = h[0];
  if (missed_est) *missed_est = k_true - (int)h[1];
  if (missed_res) *missed_res = k_true - (int)h[2];
  return GSFFT_OK;
}

}  // namespace gsfft
