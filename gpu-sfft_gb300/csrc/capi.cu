// extern "C" entry points (include/gsfft.h).
#include "engine.cuh"

#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <vector>

namespace gsfft {

thread_local int g_launch_counter = 0;
static thread_local char g_err[512] = "";

void set_last_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int current_ctx_key(CtxKey *out) {
  typedef int (*CtxGetCurrent)(void **);
  typedef int (*CtxGetId)(void *, unsigned long long *);
  static CtxGetCurrent get_current = nullptr;
  static CtxGetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetId>(f);
  });
  int dev = -1;
  if (!get_current || !get_id || cudaGetDevice(&dev) != cudaSuccess) return GSFFT_ERR_CUDA;
  void *ctx = nullptr;
  if (get_current(&ctx) != 0) return GSFFT_ERR_CUDA;
  if (!ctx) {
    // no context yet on this thread: the runtime makes the device's primary
    // context current on its first real call
    if (cudaFree(nullptr) != cudaSuccess || get_current(&ctx) != 0 || !ctx) return GSFFT_ERR_CUDA;
  }
  unsigned long long id = 0;
  if (get_id(ctx, &id) != 0) return GSFFT_ERR_CUDA;
  out->dev = dev;
  out->id = id;
  return GSFFT_OK;
}

}  // namespace gsfft

using namespace gsfft;

struct gsfft_plan_s {
  Plan *impl;
};

static cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

namespace {
// Largest sample of each row as a bit pattern (samples are non-negative, so
// their bit patterns order like their values); out[] must start at zero.
template <typename K>
__global__ void row_max_kernel(const K *__restrict__ keys, long long size, int chunks,
                               K *__restrict__ out) {
  const int row = blockIdx.x / chunks, chunk = blockIdx.x % chunks;
  const long long per = (size + chunks - 1) / chunks;
  const long long lo = (long long)chunk * per;
  const long long hi = lo + per < size ? lo + per : size;
  K m = 0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const K v = keys[(long long)row * size + i];
    m = v > m ? v : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const K v = __shfl_down_sync(0xffffffffu, m, o);
    m = v > m ? v : m;
  }
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out + row, m);
}
}  // namespace

extern "C" {

const char *gsfft_version(void) { return GSFFT_VERSION_STRING; }
const char *gsfft_last_error(void) { return g_err; }

const char *gsfft_status_string(int status) {
  switch (status) {
    case GSFFT_OK: return "ok";
    case GSFFT_ERR_PARAM: return "invalid parameter";
    case GSFFT_ERR_CAPACITY: return "candidate capacity exceeded";
    case GSFFT_ERR_ALLOC: return "allocation failed";
    case GSFFT_ERR_CUDA: return "CUDA error";
    case GSFFT_ERR_UNSUPPORTED: return "unsupported size or mode";
    case GSFFT_ERR_STATE: return "invalid plan state";
    case GSFFT_ERR_TIMEOUT: return "a bounded device-side wait gave up";
    default: return "unknown status";
  }
}

/* utils.c:180-185 */
static int floor_to_pow2(double x) {
  unsigned int ans;
  for (ans = 1; ans <= x; ans <<= 1) {
  }
  return (int)(ans / 2);
}

int gsfft_derive_params(int q, int k, double Bcst, int loops_loc, int loops_thresh, int loops_est,
                        double RLFC_cst, int RLFC_loops, double tolerance, gsfft_params *p) {
  if (!p) return GSFFT_ERR_PARAM;
  memset(p, 0, sizeof(*p));
  if (q < 8 || q > 30 || k < 1 || tolerance <= 0 || tolerance >= 1) return GSFFT_ERR_PARAM;
  // experiment.c:54-84, evaluated in the reference's order
  int n = (int)pow(2, q);
  n = floor_to_pow2(n);
  p->q = q;
  p->n = n;
  p->k = k;
  p->Bcst = Bcst;
  p->RLFC_cst = RLFC_cst;
  p->loops_loc = loops_loc;
  p->loops_thresh = loops_thresh;
  p->loops_est = loops_est;
  p->loops = loops_loc + loops_est;
  p->RLFC_loops = RLFC_loops;
  p->tolerance = tolerance;
  p->BB = (unsigned)(Bcst * sqrt((double)n * k / (log2(n))));
  p->lobefrac = 0.5 / (p->BB);
  p->b_f = (int)(1.2 * 1.1 * ((double)n / p->BB));
  p->B = floor_to_pow2(p->BB);
  p->B_thresh = 2 * k;
  p->W_RLFC = floor_to_pow2(RLFC_cst * n / p->B);
  // cuExperiment.cu:279-284
  int w = (int)((1 / M_PI) * (1 / p->lobefrac) * acosh(1. / tolerance));
  if (!(w % 2)) w--;
  p->w = w;
  p->t0 = cosh(acosh(1 / tolerance) / (w - 1));
  if (!(p->b_f <= n) || !(p->B_thresh < p->W_RLFC) || !(p->B_thresh < p->B) ||
      !(loops_thresh <= loops_loc) || !(w <= n))
    return GSFFT_ERR_PARAM;
  return validate_params(*p);
}

int gsfft_design_filter(const gsfft_params *p, complex_t *d_filter_time, complex_t *d_filter_freq,
                        void *stream) {
  if (!p || !d_filter_time) return GSFFT_ERR_PARAM;
  return design_filter(*p, reinterpret_cast<double2 *>(d_filter_time),
                       reinterpret_cast<double2 *>(d_filter_freq), S(stream));
}

int gsfft_plan_create(const gsfft_params *p, int precision, unsigned flags, int max_candidates,
                      gsfft_plan *out) {
  return gsfft_plan_create_tuned(p, precision, flags, max_candidates, nullptr, out);
}

int gsfft_plan_get_tuning(gsfft_plan plan, gsfft_plan_tuning *out) {
  if (!plan || !out) return GSFFT_ERR_PARAM;
  *out = plan->impl->tuning;
  return GSFFT_OK;
}

int gsfft_plan_create_tuned(const gsfft_params *p, int precision, unsigned flags,
                            int max_candidates, const gsfft_plan_tuning *t, gsfft_plan *out) {
  if (!p || !out) return GSFFT_ERR_PARAM;
  *out = nullptr;
  Plan *impl = nullptr;
  int s = plan_create(*p, precision, flags, max_candidates, &impl, t);
  if (s != GSFFT_OK) return s;
  gsfft_plan h = (gsfft_plan)malloc(sizeof(gsfft_plan_s));
  if (!h) {
    plan_destroy(impl);
    return GSFFT_ERR_ALLOC;
  }
  h->impl = impl;
  *out = h;
  return GSFFT_OK;
}

int gsfft_plan_destroy(gsfft_plan plan) {
  if (!plan) return GSFFT_ERR_PARAM;
  plan_destroy(plan->impl);
  free(plan);
  return GSFFT_OK;
}

int gsfft_plan_set_filter(gsfft_plan plan, const complex_t *d_ft, const complex_t *d_ff,
                          void *stream) {
  if (!plan) return GSFFT_ERR_PARAM;
  return plan_set_filter(plan->impl, d_ft, d_ff, S(stream));
}

int gsfft_run(gsfft_plan plan, const void *d_x, const int *h_offs, const int *h_a, const int *h_ai,
              void *stream) {
  if (!plan || !d_x || !h_offs || !h_a || !h_ai) return GSFFT_ERR_PARAM;
  return plan_run(plan->impl, d_x, h_offs, h_a, h_ai, S(stream));
}

int gsfft_get_results(gsfft_plan plan, Node *h_nodes, int nodes_cap, int *I_F, Node *h_topk,
                      int topk_cap, int *n_topk, void *stream) {
  if (!plan) return GSFFT_ERR_PARAM;
  return plan_results(plan->impl, h_nodes, nodes_cap, I_F, h_topk, topk_cap, n_topk, S(stream));
}

int gsfft_device_results(gsfft_plan plan, const Node **d_nodes, const int **d_I_F,
                         const Node **d_topk, const int **d_n_topk) {
  if (!plan) return GSFFT_ERR_PARAM;
  Plan *P = plan->impl;
  if (d_nodes) *d_nodes = reinterpret_cast<const Node *>(P->nodes);
  if (d_I_F) *d_I_F = &P->ctl->cand_count;
  if (d_topk) *d_topk = reinterpret_cast<const Node *>(P->topk);
  if (d_n_topk) *d_n_topk = &P->ctl->n_topk;
  return GSFFT_OK;
}

int gsfft_debug_stages(gsfft_plan plan, int *h_J2, int *num_RLFC, int *h_J, void *h_bins,
                       void *stream) {
  if (!plan) return GSFFT_ERR_PARAM;
  return plan_debug(plan->impl, h_J2, num_RLFC, h_J, h_bins, S(stream));
}

int gsfft_plan_enable_timing(gsfft_plan plan, int on) {
  if (!plan) return GSFFT_ERR_PARAM;
  return plan_enable_timing(plan->impl, on != 0);
}

int gsfft_plan_stage_times(gsfft_plan plan, float *ms_avg, int max_stages, int *runs) {
  if (!plan || !ms_avg) return GSFFT_ERR_PARAM;
  return plan_stage_times(plan->impl, ms_avg, max_stages, runs);
}

const char *gsfft_stage_name(int stage) { return stage_name(stage); }

int gsfft_plan_launches_per_run(gsfft_plan plan) {
  return plan ? plan->impl->launches_per_run : -1;
}

/* ---------------------------------------------------------------- batches */

struct gsfft_batch_s {
  Batch *impl;
};

int gsfft_batch_create(const gsfft_plan *plans, int count, int streams, gsfft_batch *out) {
  if (!plans || count < 1 || !out) return GSFFT_ERR_PARAM;
  std::vector<Plan *> ps((size_t)count);
  for (int i = 0; i < count; i++) {
    if (!plans[i]) return GSFFT_ERR_PARAM;
    ps[(size_t)i] = plans[i]->impl;
  }
  Batch *b = nullptr;
  const int s = batch_create(ps.data(), count, streams, &b);
  if (s != GSFFT_OK) return s;
  *out = new gsfft_batch_s{b};
  return GSFFT_OK;
}

int gsfft_batch_destroy(gsfft_batch batch) {
  if (!batch) return GSFFT_ERR_PARAM;
  batch_destroy(batch->impl);
  delete batch;
  return GSFFT_OK;
}

int gsfft_run_batched(gsfft_batch batch, const void *const *d_x, const int *h_rlfc_offsets,
                      const int *h_a, const int *h_ai, void *stream) {
  if (!batch) return GSFFT_ERR_PARAM;
  return batch_run(batch->impl, d_x, h_rlfc_offsets, h_a, h_ai, S(stream));
}

int gsfft_batch_capture(gsfft_batch batch, const void *const *d_x, const int *h_rlfc_offsets,
                        const int *h_a, const int *h_ai) {
  if (!batch) return GSFFT_ERR_PARAM;
  return batch_capture(batch->impl, d_x, h_rlfc_offsets, h_a, h_ai);
}

int gsfft_batch_set_persistent_tail(gsfft_batch batch, int on) {
  if (!batch) return GSFFT_ERR_PARAM;
  return batch_set_persistent_tail(batch->impl, on != 0);
}

int gsfft_batch_launch(gsfft_batch batch, void *stream) {
  if (!batch) return GSFFT_ERR_PARAM;
  return batch_launch(batch->impl, S(stream));
}

/* ---------------------------------------------------------------- tensor cores */

static int sync_check(cudaStream_t st, const char *what);

int gsfft_tc_dft64(const void *d_in, void *d_out, int nvec, void *stream) {
  if (!d_in || !d_out || nvec < 0) return GSFFT_ERR_PARAM;
  if (nvec == 0) return GSFFT_OK;
  int *err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return GSFFT_ERR_ALLOC;
  int s = cudaMemsetAsync(err, 0, sizeof(int), S(stream)) == cudaSuccess ? GSFFT_OK : GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) s = launch_tc_dft64(d_in, d_out, nvec, err, S(stream));
  if (s == GSFFT_OK) s = sync_check(S(stream), "gsfft_tc_dft64");
  int herr = 0;
  if (s == GSFFT_OK && cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK && herr) {
    set_last_error("gsfft_tc_dft64: a tensor-core completion wait timed out");
    s = GSFFT_ERR_TIMEOUT;
  }
  cudaFree(err);
  return s;
}

/* ---------------------------------------------------------------- host I/O */


int gsfft_alloc(void **d_ptr, size_t bytes) {
  if (!d_ptr) return GSFFT_ERR_PARAM;
  *d_ptr = nullptr;
  if (bytes == 0) return GSFFT_OK;
  const cudaError_t e = cudaMalloc(d_ptr, bytes);
  if (e != cudaSuccess) {
    set_last_error("gsfft_alloc(%zu): %s", bytes, cudaGetErrorString(e));
    *d_ptr = nullptr;
    return GSFFT_ERR_ALLOC;
  }
  return GSFFT_OK;
}

int gsfft_free(void *d_ptr) {
  if (d_ptr && cudaFree(d_ptr) != cudaSuccess) {
    set_last_error("gsfft_free: %s", cudaGetErrorString(cudaGetLastError()));
    return GSFFT_ERR_CUDA;
  }
  return GSFFT_OK;
}

int gsfft_copy(void *dst, const void *src, size_t bytes, void *stream) {
  if ((!dst || !src) && bytes) return GSFFT_ERR_PARAM;
  if (bytes == 0) return GSFFT_OK;
  GS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, S(stream)));
  return sync_check(S(stream), "gsfft_copy");
}

int gsfft_ingest(const complex_t *h_x, long long n, int precision, void *d_x, void *stream) {
  if (!h_x || !d_x || n < 1 || (precision != GSFFT_FP64 && precision != GSFFT_MIXED))
    return GSFFT_ERR_PARAM;
  return ingest(h_x, n, precision, d_x, S(stream));
}

int gsfft_convert_signal(const complex_t *d_in, void *d_out, long long n, void *stream) {
  if (!d_in || !d_out || n < 1) return GSFFT_ERR_PARAM;
  return launch_to_float(d_in, d_out, n, S(stream));
}

int gsfft_sync(void *stream) { return sync_check(S(stream), "gsfft_sync"); }

int gsfft_evaluate(gsfft_plan plan, const complex_t *d_x_f, const int *d_true_loc, int k_true,
                   int *missed_estimation, int *missed_result, double *mse_k, void *stream) {
  if (!plan || !d_x_f || (!d_true_loc && k_true) || k_true < 0) return GSFFT_ERR_PARAM;
  return plan_evaluate(plan->impl, d_x_f, d_true_loc, k_true, missed_estimation, missed_result,
                       mse_k, S(stream));
}

int gsfft_plan_describe(gsfft_plan plan, int *streaming, int *row_groups) {
  if (!plan || !streaming || !row_groups) return GSFFT_ERR_PARAM;
  *streaming = plan->impl->use_stream ? 1 : 0;
  *row_groups = plan->impl->use_stream ? plan->impl->groups : 0;
  return GSFFT_OK;
}

int gsfft_plan_tensor_core_ffts(gsfft_plan plan, int *bucket, int *rlfc) {
  if (!plan || !bucket || !rlfc) return GSFFT_ERR_PARAM;
  *bucket = plan->impl->tc_bucket ? 1 : 0;
  *rlfc = plan->impl->tc_rlfc ? 1 : 0;
  return GSFFT_OK;
}

int gsfft_fft(const void *d_in, void *d_out, long long n_fft, int batch, int sign, int precision,
              void *stream) {
  if (!d_in || !d_out || batch < 1 || (sign != 1 && sign != -1)) return GSFFT_ERR_PARAM;
  if (precision != GSFFT_FP64 && precision != GSFFT_MIXED) return GSFFT_ERR_PARAM;
  FftPlan fp;
  int s = fft_plan_init(fp, n_fft, precision, batch);
  if (s == GSFFT_OK) {
    FftIo io;
    s = fft_exec(fp, d_in, d_out, batch, sign, io, S(stream));
    if (s == GSFFT_OK && cudaStreamSynchronize(S(stream)) != cudaSuccess) {
      set_last_error("gsfft_fft: %s", cudaGetErrorString(cudaGetLastError()));
      s = GSFFT_ERR_CUDA;
    }
  }
  fft_plan_free(fp);
  return s;
}

int gsfft_check_bounded_wait(long long limit_cycles, void *stream) {
  if (limit_cycles < 1 || limit_cycles > (1LL << 31)) return GSFFT_ERR_PARAM;
  int *flag = nullptr;
  if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) return GSFFT_ERR_ALLOC;
  int s = cudaMemsetAsync(flag, 0, sizeof(int), S(stream)) == cudaSuccess ? GSFFT_OK : GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) s = launch_bounded_wait_probe(limit_cycles, flag, S(stream));
  int gave_up = 0;
  if (s == GSFFT_OK &&
      (cudaMemcpyAsync(&gave_up, flag, sizeof(int), cudaMemcpyDeviceToHost, S(stream)) != cudaSuccess ||
       cudaStreamSynchronize(S(stream)) != cudaSuccess)) {
    set_last_error("gsfft_check_bounded_wait: %s", cudaGetErrorString(cudaGetLastError()));
    s = GSFFT_ERR_CUDA;
  }
  cudaFree(flag);
  if (s != GSFFT_OK) return s;
  if (gave_up) {
    set_last_error("bounded wait gave up after %lld cycles", limit_cycles);
    return GSFFT_ERR_TIMEOUT;
  }
  return GSFFT_OK;
}

// an FP32 FFT with one of the tensor-core plans (its completion waits checked)
static int fft_tc_run(int (*init)(FftPlan &, long long, int), const char *what, const void *d_in,
                      void *d_out, long long n_fft, int batch, int sign, void *stream) {
  if (!d_in || !d_out || batch < 1 || (sign != 1 && sign != -1)) return GSFFT_ERR_PARAM;
  FftPlan fp;
  int s = init(fp, n_fft, batch);
  if (s == GSFFT_OK) {
    int *err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
      s = GSFFT_ERR_ALLOC;
    } else {
      FftIo io;
      io.err = err;
      if (cudaMemsetAsync(err, 0, sizeof(int), S(stream)) != cudaSuccess) s = GSFFT_ERR_CUDA;
      if (s == GSFFT_OK) s = fft_exec(fp, d_in, d_out, batch, sign, io, S(stream));
      int h = 0;
      if (s == GSFFT_OK &&
          (cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, S(stream)) != cudaSuccess ||
           cudaStreamSynchronize(S(stream)) != cudaSuccess)) {
        set_last_error("%s: %s", what, cudaGetErrorString(cudaGetLastError()));
        s = GSFFT_ERR_CUDA;
      }
      if (s == GSFFT_OK && h) {
        set_last_error("%s: a tensor-core completion wait timed out", what);
        s = GSFFT_ERR_TIMEOUT;
      }
      cudaFree(err);
    }
  }
  fft_plan_free(fp);
  return s;
}

int gsfft_fft_tc(const void *d_in, void *d_out, long long n_fft, int batch, int sign,
                 void *stream) {
  return fft_tc_run(fft_plan_init_tc, "gsfft_fft_tc", d_in, d_out, n_fft, batch, sign, stream);
}

int gsfft_fft_tc64(const void *d_in, void *d_out, long long n_fft, int batch, int sign,
                   void *stream) {
  return fft_tc_run(fft_plan_init_tc64, "gsfft_fft_tc64", d_in, d_out, n_fft, batch, sign, stream);
}

int gsfft_cutoff(const void *d_samples, int size, int num, int batch, int precision, int *d_out,
                 void *stream) {
  if (!d_samples || !d_out || size < 1 || num < 1 || num >= size || batch < 1 ||
      (precision != GSFFT_FP64 && precision != GSFFT_MIXED))
    return GSFFT_ERR_PARAM;
  SelectScratch ss;
  int s = select_scratch_init(ss, batch, size);
  if (s == GSFFT_OK)
    s = select_top(d_samples, precision == GSFFT_FP64 ? 8 : 4, size, nullptr, num, batch, size,
                   d_out, num, nullptr, ss, S(stream));
  if (s == GSFFT_OK && cudaStreamSynchronize(S(stream)) != cudaSuccess) {
    set_last_error("gsfft_cutoff: %s", cudaGetErrorString(cudaGetLastError()));
    s = GSFFT_ERR_CUDA;
  }
  select_scratch_free(ss);
  return s;
}


int gsfft_cutoff_floor(const void *d_samples, int size, int num, int batch, int precision,
                       double floor_rel, const void *d_row_max, int *d_out, void *stream) {
  if (!d_samples || !d_out || size < 1 || num < 1 || num >= size || batch < 1 ||
      !(floor_rel >= 0.0 && floor_rel < 1.0) ||
      (precision != GSFFT_FP64 && precision != GSFFT_MIXED))
    return GSFFT_ERR_PARAM;
  const int kb = precision == GSFFT_FP64 ? 8 : 4;
  cudaStream_t st = S(stream);
  void *rmax = nullptr;
  SelectScratch ss;
  int s = select_scratch_init(ss, batch, size);
  if (s == GSFFT_OK && !d_row_max && floor_rel > 0.0) {
    if (cudaMalloc(&rmax, (size_t)kb * batch) != cudaSuccess) {
      s = GSFFT_ERR_ALLOC;
    } else if (cudaMemsetAsync(rmax, 0, (size_t)kb * batch, st) != cudaSuccess) {
      s = GSFFT_ERR_CUDA;
    } else {
      const int chunks = (int)((size + 65535) / 65536);
      if (kb == 8)
        row_max_kernel<unsigned long long><<<batch * chunks, 256, 0, st>>>(
            (const unsigned long long *)d_samples, size, chunks, (unsigned long long *)rmax);
      else
        row_max_kernel<unsigned><<<batch * chunks, 256, 0, st>>>((const unsigned *)d_samples, size,
                                                                  chunks, (unsigned *)rmax);
      if (cudaGetLastError() != cudaSuccess) s = GSFFT_ERR_CUDA;
    }
  }
  if (s == GSFFT_OK)
    s = select_top(d_samples, kb, size, nullptr, num, batch, size, d_out, num, nullptr, ss, st,
                   d_row_max ? d_row_max : rmax, floor_rel);
  if (s == GSFFT_OK && cudaStreamSynchronize(st) != cudaSuccess) {
    set_last_error("gsfft_cutoff_floor: %s", cudaGetErrorString(cudaGetLastError()));
    s = GSFFT_ERR_CUDA;
  }
  if (rmax) cudaFree(rmax);
  select_scratch_free(ss);
  return s;
}

/* ---------------------------------------------------------------- stages */

static int sync_check(cudaStream_t st, const char *what) {
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_last_error("%s: %s", what, cudaGetErrorString(e));
    return GSFFT_ERR_CUDA;
  }
  return GSFFT_OK;
}

int gsfft_stage_perm_filter(int precision, const void *d_x, int n, const complex_t *d_filter_time,
                            int w, int B, int loops, const int *h_ai, int quirk_residue,
                            void *d_bins, void *stream) {
  if (!d_x || !d_filter_time || !d_bins || !h_ai || loops < 1 || loops > MAX_LOOPS) return GSFFT_ERR_PARAM;
  if (n < 2 || (n & (n - 1)) || B < 1 || (B & (B - 1)) || B > n || w < 1 || w > n) return GSFFT_ERR_PARAM;
  Draws d;
  memset(&d, 0, sizeof(d));
  for (int l = 0; l < loops; l++) d.ai[l] = h_ai[l];
  const bool fl = precision == GSFFT_MIXED;
  void *taps = nullptr;
  if (fl) {
    if (cudaMalloc(&taps, sizeof(float2) * (size_t)w) != cudaSuccess) return GSFFT_ERR_ALLOC;
  }
  int s = GSFFT_OK;
  if (fl) s = launch_convert_taps((const double2 *)d_filter_time, taps, w, true, S(stream));
  if (s == GSFFT_OK)
    s = launch_perm_filter(precision, d_x, n, fl ? taps : (const void *)d_filter_time, w, B, loops, d,
                           quirk_residue != 0, d_bins, S(stream));
  if (s == GSFFT_OK) s = sync_check(S(stream), "gsfft_stage_perm_filter");
  if (taps) cudaFree(taps);
  return s;
}

int gsfft_stage_perm_filter_stream(int precision, const void *d_x, int n,
                                   const complex_t *d_filter_time, int w, int B, int loops,
                                   const int *h_a, void *d_bins, void *stream) {
  if (!d_x || !d_filter_time || !d_bins || !h_a || loops < 2 || loops > 16) return GSFFT_ERR_PARAM;
  if (n < 2 || (n & (n - 1)) || B < 1 || (B & (B - 1)) || B > n / 2 || w < 1 || w > n)
    return GSFFT_ERR_PARAM;
  if (!stream_pf_supported(n, B, loops, n, 0) || w / B >= 32) return GSFFT_ERR_UNSUPPORTED;
  Draws d;
  memset(&d, 0, sizeof(d));
  for (int l = 0; l < loops; l++) d.a[l] = h_a[l];
  const bool fl = precision == GSFFT_MIXED;
  void *taps = nullptr, *part = nullptr, *tbm = nullptr;
  int *err = nullptr;
  const int groups = stream_pf_groups(n, B, w, loops, precision);
  const size_t es = fl ? sizeof(float2) : sizeof(double2);
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return GSFFT_ERR_ALLOC;
  if (cudaMalloc(&part, es * (size_t)groups * loops * B) != cudaSuccess ||
      cudaMalloc(&tbm, es * (size_t)stream_taps_count(w, B)) != cudaSuccess ||
      (fl && cudaMalloc(&taps, sizeof(float2) * (size_t)w) != cudaSuccess)) {
    cudaFree(err);
    if (part) cudaFree(part);
    if (tbm) cudaFree(tbm);
    return GSFFT_ERR_ALLOC;
  }
  int s = cudaMemsetAsync(err, 0, sizeof(int), S(stream)) == cudaSuccess ? GSFFT_OK : GSFFT_ERR_CUDA;
  if (s == GSFFT_OK && fl) s = launch_convert_taps((const double2 *)d_filter_time, taps, w, true, S(stream));
  if (s == GSFFT_OK)
    s = launch_stream_taps(precision, fl ? taps : (const void *)d_filter_time, w, B, tbm, S(stream));
  if (s == GSFFT_OK)
    s = launch_perm_filter_stream(precision, d_x, n, tbm, w, B, loops, d, part, 0, nullptr, n, err,
                                  S(stream));
  if (s == GSFFT_OK)
    s = launch_sum_partials(precision, part, groups, (long long)loops * B, d_bins, S(stream));
  if (s == GSFFT_OK) s = sync_check(S(stream), "gsfft_stage_perm_filter_stream");
  int herr = 0;
  if (s == GSFFT_OK && cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK && herr) {
    set_last_error("gsfft_stage_perm_filter_stream: a copy-completion wait timed out");
    s = GSFFT_ERR_TIMEOUT;
  }
  if (taps) cudaFree(taps);
  cudaFree(tbm);
  cudaFree(part);
  cudaFree(err);
  return s;
}

int gsfft_stage_reverse_hash(const int *d_J, int B_thresh, const int *d_J2, int num_RLFC, int n,
                             int B, int W_RLFC, int a, int ai, int loops_thresh, unsigned epoch,
                             unsigned *d_vote, int *d_cand, int cap, int *h_count, void *stream) {
  if (!d_J || !d_J2 || !d_vote || !d_cand || !h_count || num_RLFC < 1 || B_thresh < 1)
    return GSFFT_ERR_PARAM;
  if (n < 2 || (n & (n - 1)) || W_RLFC >= n || W_RLFC <= n / B || (W_RLFC & (W_RLFC - 1)) ||
      W_RLFC < 32 || loops_thresh < 1 || loops_thresh > 255 || epoch >= (1u << 24))
    return GSFFT_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  const int words = W_RLFC / 32;
  unsigned *bm = nullptr, *d_ep = nullptr;
  int *cnt = nullptr, *blk = nullptr;
  RunCtl *ctl = nullptr;
  int s = GSFFT_OK;
  if (cudaMalloc(&bm, sizeof(unsigned) * words) != cudaSuccess ||
      cudaMalloc(&cnt, sizeof(int) * B_thresh) != cudaSuccess ||
      cudaMalloc(&blk, sizeof(int) * vote_block_ints(B_thresh)) != cudaSuccess ||
      cudaMalloc(&ctl, sizeof(RunCtl)) != cudaSuccess ||
      cudaMalloc(&d_ep, sizeof(unsigned)) != cudaSuccess)
    s = GSFFT_ERR_ALLOC;
  Draws d;
  memset(&d, 0, sizeof(d));
  d.a[0] = a;
  d.ai[0] = ai;
  RunCtl c;
  memset(&c, 0, sizeof(c));
  c.cand_count = *h_count;
  c.num_rlfc = num_RLFC;
  if (s == GSFFT_OK && (cudaMemcpyAsync(ctl, &c, sizeof(c), cudaMemcpyHostToDevice, st) != cudaSuccess ||
                        cudaMemcpyAsync(d_ep, &epoch, sizeof(unsigned), cudaMemcpyHostToDevice, st) !=
                            cudaSuccess))
    s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) s = launch_sigma_bitmaps(d_J2, ctl, num_RLFC, W_RLFC, 1, d, bm, ctl, st);
  if (s == GSFFT_OK)
    s = launch_vote_loop(0, d_J, B_thresh, n, B, W_RLFC, bm, d, loops_thresh, d_ep, d_vote, d_cand,
                         cap, cnt, blk, ctl, true, st);
  if (s == GSFFT_OK && cudaMemcpyAsync(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) s = sync_check(st, "gsfft_stage_reverse_hash");
  if (s == GSFFT_OK) {
    *h_count = c.cand_count;
    if (c.overflow) s = GSFFT_ERR_CAPACITY;
  }
  cudaFree(bm);
  cudaFree(cnt);
  cudaFree(blk);
  cudaFree(ctl);
  cudaFree(d_ep);
  return s;
}

int gsfft_stage_estimate(int precision, const int *d_cand, int num, const void *d_bins, int loops,
                         int n, int B, const int *h_ai, const complex_t *d_filter_freq, Node *d_out,
                         void *stream) {
  if (!d_cand || !d_bins || !h_ai || !d_filter_freq || !d_out || num < 0 || loops < 1 ||
      loops > MAX_LOOPS)
    return GSFFT_ERR_PARAM;
  if (n < 2 || (n & (n - 1)) || B < 1 || (B & (B - 1)) || B > n / 2) return GSFFT_ERR_PARAM;
  if (num == 0) return GSFFT_OK;
  cudaStream_t st = S(stream);
  const int nb = n / B;
  double2 *hinv = nullptr;
  double *mag2 = nullptr;
  RunCtl *ctl = nullptr;
  int s = GSFFT_OK;
  if (cudaMalloc(&hinv, hinv_bytes(nb)) != cudaSuccess ||
      cudaMalloc(&mag2, sizeof(double) * num) != cudaSuccess ||
      cudaMalloc(&ctl, sizeof(RunCtl)) != cudaSuccess)
    s = GSFFT_ERR_ALLOC;
  Draws d;
  memset(&d, 0, sizeof(d));
  for (int l = 0; l < loops; l++) d.ai[l] = h_ai[l];
  RunCtl c;
  memset(&c, 0, sizeof(c));
  c.cand_count = num;
  if (s == GSFFT_OK && cudaMemcpyAsync(ctl, &c, sizeof(c), cudaMemcpyHostToDevice, st) != cudaSuccess)
    s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) s = launch_hinv((const double2 *)d_filter_freq, n, nb, hinv, st);
  if (s == GSFFT_OK)
    s = launch_estimate(precision, d_cand, ctl, num, num, d_bins, loops, n, B, d, hinv,
                        reinterpret_cast<DevNode *>(d_out), mag2, st);
  if (s == GSFFT_OK) s = sync_check(st, "gsfft_stage_estimate");
  cudaFree(hinv);
  cudaFree(mag2);
  cudaFree(ctl);
  return s;
}

/* ------------------------------------------------------------------------
 * Drop-in entry points with the reference's signatures.
 * ---------------------------------------------------------------------- */

/* outerLoop.cu:65-190 */
Node *outer_loop(complex_t *d_x, int n, complex_t *d_filter_time, complex_t *d_filter_freq,
                 int d_filter_size, int B, int B_thresh, int W_RLFC, int RLFC_loops,
                 int loop_threshold, int loops_loc, int loops, int *I_F, float t_H_to_D) {
  (void)t_H_to_D;
  if (!I_F) return nullptr;
  gsfft_params p;
  memset(&p, 0, sizeof(p));
  int q = 0;
  while ((1 << q) < n) q++;
  p.q = q;
  p.n = n;
  p.k = B_thresh / 2;
  p.B = B;
  p.B_thresh = B_thresh;
  p.W_RLFC = W_RLFC;
  p.RLFC_loops = RLFC_loops;
  p.loops_loc = loops_loc;
  p.loops_thresh = loop_threshold;
  p.loops_est = loops - loops_loc;
  p.loops = loops;
  p.w = d_filter_size;
  p.b_f = 1;
  // random draws in the reference's order (innerLoop.cu:122-123, outerLoop.cu:128-134)
  int offs[MAX_RLFC_LOOPS], a[MAX_LOOPS], ai[MAX_LOOPS];
  if (RLFC_loops > MAX_RLFC_LOOPS || loops > MAX_LOOPS || W_RLFC <= 0 || n <= 0) {
    set_last_error("outer_loop: unsupported sizes");
    return nullptr;
  }
  const int sigma = n / W_RLFC;
  for (int r = 0; r < RLFC_loops; r++) offs[r] = (int)(unsigned)floor(drand48() * sigma);
  for (int i = 0; i < loops; i++) {
    int av = 0;
    // gcd(av, n) == 1 with n a power of two <=> av odd
    while ((av & 1) == 0) av = (int)(random() % n);
    a[i] = av;
    // modular inverse of an odd number mod 2^q by Newton iteration
    unsigned inv = (unsigned)av;
    for (int it = 0; it < 5; it++) inv *= 2u - (unsigned)av * inv;
    ai[i] = (int)(inv & (unsigned)(n - 1));
  }
  // the reference's own selection rule (raw |X|^2 threshold, innerLoop.cu:551-642) and,
  // below n = 2^27, its residue tap index (innerLoop.cu:230-237, :745-754)
  const unsigned flags =
      GSFFT_FLAG_RAW_SELECTION | (n < (1 << 27) ? GSFFT_FLAG_QUIRK_RESIDUE : 0u);
  gsfft_plan plan = nullptr;
  Node *out = nullptr;
  int s = gsfft_plan_create(&p, GSFFT_FP64, flags, 524288, &plan);
  if (s == GSFFT_OK) s = gsfft_plan_set_filter(plan, d_filter_time, d_filter_freq, nullptr);
  if (s == GSFFT_OK) s = gsfft_run(plan, d_x, offs, a, ai, nullptr);
  int count = 0;
  if (s == GSFFT_OK) s = gsfft_get_results(plan, nullptr, 0, &count, nullptr, 0, nullptr, nullptr);
  if (s == GSFFT_OK) {
    out = (Node *)malloc(sizeof(Node) * (count > 0 ? count : 1));
    if (!out) {
      set_last_error("outer_loop: host allocation of %d nodes failed", count);
      s = GSFFT_ERR_ALLOC;
    }
    if (s == GSFFT_OK) s = gsfft_get_results(plan, out, count, &count, nullptr, 0, nullptr, nullptr);
    if (s == GSFFT_OK) *I_F += count;
  }
  if (s != GSFFT_OK && out) {
    free(out);
    out = nullptr;
  }
  if (plan) gsfft_plan_destroy(plan);
  return out;
}

/* ---- stage drop-ins (innerLoop.h:32-50) ---- */

namespace {
__global__ void samples_kernel(const double2 *__restrict__ v, int size, double *s) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i < size) s[i] = __dadd_rn(__dmul_rn(v[i].x, v[i].x), __dmul_rn(v[i].y, v[i].y));
}

struct EvTimer {  // adds the elapsed seconds of a section to *acc
  cudaEvent_t a = nullptr, b = nullptr;
  double *acc;
  explicit EvTimer(double *acc_) : acc(acc_) {
    if (acc) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a);
    }
  }
  ~EvTimer() {
    if (acc) {
      float ms = 0.f;
      cudaEventRecord(b);
      cudaEventSynchronize(b);
      cudaEventElapsedTime(&ms, a, b);
      *acc += ms / 1.0e3;
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  }
};

int cutoff_device(const double *d_s, int size, int num, int *d_out) {
  SelectScratch ss;
  int s = select_scratch_init(ss, 1, size);
  if (s == GSFFT_OK) s = select_top(d_s, 8, size, nullptr, num, 1, size, d_out, num, nullptr, ss, 0);
  if (s == GSFFT_OK) s = sync_check(0, "cutoff");
  select_scratch_free(ss);
  return s;
}
}  // namespace

/* innerLoop.cu:112-177: one RLFC block of B_thresh ids into d_J2. */
int restr_loc_freq_coeff(complex_t *d_x, int n, int B_thresh, int W_RLFC, int *d_J2,
                         double *RLFC_Time) {
  EvTimer tm(RLFC_Time);
  if (!d_x || !d_J2 || W_RLFC < 256 || n % W_RLFC || B_thresh >= W_RLFC) return GSFFT_ERR_PARAM;
  const int sigma = n / W_RLFC;
  const int offset = (int)(unsigned)floor(drand48() * sigma);  /* innerLoop.cu:123 */
  FftPlan fp;
  double *s_d = nullptr;
  int s = fft_plan_init(fp, W_RLFC, GSFFT_FP64, 1);
  if (s == GSFFT_OK && cudaMalloc(&s_d, sizeof(double) * W_RLFC) != cudaSuccess) s = GSFFT_ERR_ALLOC;
  if (s == GSFFT_OK) {
    FftIo io;
    io.gather_x = d_x;
    io.gather_offsets[0] = offset;
    io.gather_stride = sigma;
    io.samples = s_d;
    io.write_complex = false;
    s = fft_exec(fp, nullptr, s_d, 1, -1, io, 0);
  }
  if (s == GSFFT_OK) s = cutoff_device(s_d, W_RLFC, B_thresh, d_J2);
  fft_plan_free(fp);
  cudaFree(s_d);
  return s;
}

/* innerLoop.cu:484-539: indices of the B largest |d_samp|^2, ascending. */
int samples_indices(complex_t *d_samp, int B, int samp_size, int *d_output, double *CTime) {
  EvTimer tm(CTime);
  if (!d_samp || !d_output || B < 1 || samp_size < B + 1) return GSFFT_ERR_PARAM;
  double *s_d = nullptr;
  if (cudaMalloc(&s_d, sizeof(double) * samp_size) != cudaSuccess) return GSFFT_ERR_ALLOC;
  samples_kernel<<<(samp_size + 255) / 256, 256>>>((const double2 *)d_samp, samp_size, s_d);
  int s = cudaGetLastError() == cudaSuccess ? GSFFT_OK : GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) s = cutoff_device(s_d, samp_size, B, d_output);
  cudaFree(s_d);
  return s;
}

/* innerLoop.cu:194-286: perm+filter, B-point FFT into d_bins_f, cutoff into d_J. */
int perm_filter_cutoff(complex_t *d_x, int n, complex_t *d_filter_time, int d_filter_size,
                       int B_thresh, int B, int a, int ai, complex_t *d_bins_f, int *d_J,
                       double *PF_T, double *BC_T) {
  (void)a;
  if (!d_x || !d_filter_time || !d_bins_f || !d_J || B < 256 || B_thresh >= B) return GSFFT_ERR_PARAM;
  int s;
  {
    EvTimer tm(PF_T);
    s = gsfft_stage_perm_filter(GSFFT_FP64, d_x, n, d_filter_time, d_filter_size, B, 1, &ai,
                                n < (1 << 27) ? 1 : 0, d_bins_f, nullptr);
  }
  if (s != GSFFT_OK) return s;
  EvTimer tm(BC_T);
  FftPlan fp;
  double *s_d = nullptr;
  s = fft_plan_init(fp, B, GSFFT_FP64, 1);
  if (s == GSFFT_OK && cudaMalloc(&s_d, sizeof(double) * B) != cudaSuccess) s = GSFFT_ERR_ALLOC;
  if (s == GSFFT_OK) {
    FftIo io;
    io.samples = s_d;
    s = fft_exec(fp, d_bins_f, d_bins_f, 1, -1, io, 0);
  }
  if (s == GSFFT_OK) s = cutoff_device(s_d, B, B_thresh, d_J);
  fft_plan_free(fp);
  cudaFree(s_d);
  return s;
}

/* innerLoop.cu:300-384: votes into the int table d_vote, appends to d_I from *I_F. */
int reverse_hash(int *d_J, int n, int B_thresh, int B, int a, int ai, int loop_thresh, int *d_vote,
                 int *d_I, int *I_F, double *G_T, int *d_J2, int num_RLFC, int W_RLFC,
                 int RLFC_loops) {
  (void)RLFC_loops;
  EvTimer tm(G_T);
  if (!I_F) return GSFFT_ERR_PARAM;
  return gsfft_stage_reverse_hash(d_J, B_thresh, d_J2, num_RLFC, n, B, W_RLFC, a, ai, loop_thresh,
                                  0u, reinterpret_cast<unsigned *>(d_vote), d_I, 524288, I_F,
                                  nullptr);
}

/* innerLoop.cu:396-466: malloc'ed host array of *I_F estimates (caller frees). */
Node *estimate_values(int *d_I, int *I_F, complex_t *d_bins_f, int loops, int n, int *permute, int B,
                      complex_t *d_filter_freq, int loops_loc) {
  (void)loops_loc;
  if (!I_F || *I_F < 0) return nullptr;
  const int num = *I_F;
  Node *h = (Node *)malloc(sizeof(Node) * (num > 0 ? num : 1));
  if (!h || num == 0) return h;
  Node *d = nullptr;
  if (cudaMalloc(&d, sizeof(Node) * num) != cudaSuccess) {
    free(h);
    return nullptr;
  }
  int s = gsfft_stage_estimate(GSFFT_FP64, d_I, num, d_bins_f, loops, n, B, permute, d_filter_freq,
                               d, nullptr);
  if (s == GSFFT_OK && cudaMemcpy(h, d, sizeof(Node) * num, cudaMemcpyDeviceToHost) != cudaSuccess)
    s = GSFFT_ERR_CUDA;
  cudaFree(d);
  if (s != GSFFT_OK) {
    free(h);
    return nullptr;
  }
  return h;
}

/* innerLoop.cu:647-649 */
int timesmod(const int x, const int a, const int n) {
  return (int)((((long long)(x)) * a) % n);
}

}  // extern "C"
