// Autotuner of a plan's stage shapes (gsfft_autotune_plan) and the entry
// points that create plans with explicit shapes.
//
// The shapes (gsfft_plan_tuning): the perm+filter form (one ordered pass over
// the signal or random gathers) and, for the ordered pass, the number of row
// groups with their own partial bins; the first-pass radix of the bucket and
// RLFC FFTs (two-pass sizes); the form of the cutoffs (one cluster or
// cooperative launch per cutoff, or the multi-launch radix passes).  The rules
// gsfft_plan_create applies fit the headline sizes; across the batched
// configurations (n from 2^18 to 2^24, k from 50 to 4000) other shapes can be
// faster, so the tuner measures them: coordinate descent over the knobs,
// each candidate plan timed with CUDA events over a few runs on the caller's
// signal, filter and draws.  Results are kept in a plain text file, one line
// per (device, precision, flags, sizes) key.
#include "engine.cuh"

#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>

namespace gsfft {

namespace {

std::mutex g_cache_mu;

// the flags that change a plan's pipeline, and so belong to the cache key
constexpr unsigned kTuneFlags = GSFFT_FLAG_QUIRK_RESIDUE | GSFFT_FLAG_RAW_SELECTION |
                                GSFFT_FLAG_TC_BUCKET_FFT | GSFFT_FLAG_TC_RLFC_FFT |
                                GSFFT_FLAG_CC_BUCKET_FFT;

int cache_key(const gsfft_params &p, int precision, unsigned flags, std::string *key) {
  int dev = 0;
  GS_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  GS_CUDA(cudaGetDeviceProperties(&prop, dev));
  std::string name = prop.name;
  for (char &c : name)
    if (c == ' ' || c == '\t') c = '_';
  char buf[512];
  snprintf(buf, sizeof(buf), "%s|sms=%d|prec=%d|flags=%u|n=%d|B=%d|W=%d|w=%d|Bt=%d|loops=%d|ll=%d|R=%d",
           name.c_str(), prop.multiProcessorCount, precision, flags & kTuneFlags, p.n, p.B,
           p.W_RLFC, p.w, p.B_thresh, p.loops, p.loops_loc, p.RLFC_loops);
  *key = buf;
  return GSFFT_OK;
}

bool cache_lookup(const char *path, const std::string &key, gsfft_plan_tuning *t, float *ms) {
  if (!path) return false;
  std::lock_guard<std::mutex> lock(g_cache_mu);
  FILE *f = fopen(path, "r");
  if (!f) return false;
  char line[1024], k[600];
  bool found = false;
  while (fgets(line, sizeof(line), f)) {
    gsfft_plan_tuning c = {};
    float m = 0.f;
    if (sscanf(line, "gsfft-tune-v1 %599s pf=%d groups=%d br=%d rr=%d sel=%d ms=%f", k,
               &c.perm_filter_form, &c.row_groups, &c.bucket_first_radix, &c.rlfc_first_radix,
               &c.select_form, &m) == 7 &&
        key == k) {
      *t = c;  // the last line for a key wins
      *ms = m;
      found = true;
    }
  }
  fclose(f);
  return found;
}

void cache_store(const char *path, const std::string &key, const gsfft_plan_tuning &t, float ms) {
  if (!path) return;
  std::lock_guard<std::mutex> lock(g_cache_mu);
  FILE *f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "gsfft-tune-v1 %s pf=%d groups=%d br=%d rr=%d sel=%d ms=%.5f\n", key.c_str(),
          t.perm_filter_form, t.row_groups, t.bucket_first_radix, t.rlfc_first_radix,
          t.select_form, ms);
  fclose(f);
}

struct Bench {
  const gsfft_params *p;
  int precision;
  unsigned flags;
  const void *d_x;
  const complex_t *ft, *ff;
  const int *offs, *a, *ai;
  int reps;
  cudaStream_t st;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};

// mean ms of one candidate (negative: the shape does not apply); *used: the
// shapes the plan actually took
int measure(Bench &b, const gsfft_plan_tuning &t, float *ms, gsfft_plan_tuning *used) {
  Plan *P = nullptr;
  int s = plan_create(*b.p, b.precision, b.flags, 0, &P, &t);
  if (s == GSFFT_ERR_PARAM || s == GSFFT_ERR_UNSUPPORTED) {
    *ms = -1.f;
    return GSFFT_OK;
  }
  GS_CHECK(s);
  s = plan_set_filter(P, b.ft, b.ff, b.st);
  if (s == GSFFT_OK) s = plan_run(P, b.d_x, b.offs, b.a, b.ai, b.st);  // warm-up
  if (s == GSFFT_OK && cudaEventRecord(b.e0, b.st) != cudaSuccess) s = GSFFT_ERR_CUDA;
  for (int r = 0; r < b.reps && s == GSFFT_OK; r++) s = plan_run(P, b.d_x, b.offs, b.a, b.ai, b.st);
  if (s == GSFFT_OK && cudaEventRecord(b.e1, b.st) != cudaSuccess) s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK && cudaEventSynchronize(b.e1) != cudaSuccess) s = GSFFT_ERR_CUDA;
  float total = 0.f;
  if (s == GSFFT_OK && cudaEventElapsedTime(&total, b.e0, b.e1) != cudaSuccess) s = GSFFT_ERR_CUDA;
  if (s == GSFFT_OK) {
    RunCtl c;
    if (cudaMemcpy(&c, P->ctl, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) s = GSFFT_ERR_CUDA;
    else if (c.err) {
      set_last_error("gsfft_autotune_plan: a bounded device-side wait gave up");
      s = GSFFT_ERR_TIMEOUT;
    }
  }
  if (s == GSFFT_OK) {
    *ms = total / (float)b.reps;
    *used = P->tuning;
  }
  plan_destroy(P);
  return s;
}

// log2 radices of a two-pass first pass for a transform of 2^L points
void radix_range(int L, int precision, int *lo, int *hi) {
  const int one = precision == GSFFT_FP64 ? 13 : 14;
  *lo = L - one > 7 ? L - one : 7;
  *hi = L - 7 < one ? L - 7 : one;
}

int ilog2i(long long v) {
  int l = 0;
  while ((1LL << l) < v) l++;
  return l;
}

}  // namespace

}  // namespace gsfft

using namespace gsfft;

extern "C" {

int gsfft_autotune_plan(const gsfft_params *p, int precision, unsigned flags, const void *d_x,
                        const complex_t *d_filter_time, const complex_t *d_filter_freq,
                        const int *h_rlfc_offsets, const int *h_a, const int *h_ai, int reps,
                        const char *cache_path, gsfft_plan_tuning *best, float *best_ms,
                        void *stream) {
  if (!p || !d_x || !d_filter_time || !d_filter_freq || !h_rlfc_offsets || !h_a || !h_ai ||
      !best || reps < 1 || reps > 1000)
    return GSFFT_ERR_PARAM;
  GS_CHECK(validate_params(*p));
  std::string key;
  GS_CHECK(cache_key(*p, precision, flags, &key));
  float cms = 0.f;
  if (cache_lookup(cache_path, key, best, &cms)) {
    if (best_ms) *best_ms = cms;
    return GSFFT_OK;
  }
  Bench b;
  b.p = p;
  b.precision = precision;
  b.flags = flags & ~(GSFFT_FLAG_FORCE_GATHER | GSFFT_FLAG_FORCE_STREAM);
  b.d_x = d_x;
  b.ft = d_filter_time;
  b.ff = d_filter_freq;
  b.offs = h_rlfc_offsets;
  b.a = h_a;
  b.ai = h_ai;
  b.reps = reps;
  b.st = reinterpret_cast<cudaStream_t>(stream);
  GS_CUDA(cudaEventCreate(&b.e0));
  if (cudaEventCreate(&b.e1) != cudaSuccess) {
    cudaEventDestroy(b.e0);
    return GSFFT_ERR_CUDA;
  }
  gsfft_plan_tuning cur = {}, used = {};
  float cur_ms = -1.f;
  int s = measure(b, cur, &cur_ms, &used);
  if (s == GSFFT_OK && cur_ms < 0.f) s = GSFFT_ERR_UNSUPPORTED;
  if (s == GSFFT_OK) cur = used;  // the rules' shapes, explicit
  auto consider = [&](const gsfft_plan_tuning &cand) {
    if (s != GSFFT_OK) return;
    float ms = -1.f;
    gsfft_plan_tuning u = {};
    s = measure(b, cand, &ms, &u);
    if (s == GSFFT_OK && ms >= 0.f && ms < cur_ms) {
      cur = u;
      cur_ms = ms;
    }
  };
  // 1. perm+filter form and row groups
  {
    gsfft_plan_tuning c = cur;
    c.perm_filter_form = 2;
    c.row_groups = 0;
    consider(c);
    for (int g = 1; g <= 32; g *= 2) {
      gsfft_plan_tuning d = cur;
      d.perm_filter_form = 1;
      d.row_groups = g;
      if (!(cur.perm_filter_form == 1 && cur.row_groups == g)) consider(d);
    }
  }
  // 2. first-pass radices of the two FFTs
  if (cur.bucket_first_radix > 0) {
    int lo, hi;
    radix_range(ilog2i(p->B), precision, &lo, &hi);
    const int keep = cur.bucket_first_radix;
    for (int r = lo; r <= hi; r++) {
      if (r == keep) continue;
      gsfft_plan_tuning c = cur;
      c.bucket_first_radix = r;
      consider(c);
    }
  }
  if (cur.rlfc_first_radix > 0) {
    int lo, hi;
    radix_range(ilog2i(p->W_RLFC), precision, &lo, &hi);
    const int keep = cur.rlfc_first_radix;
    for (int r = lo; r <= hi; r++) {
      if (r == keep) continue;
      gsfft_plan_tuning c = cur;
      c.rlfc_first_radix = r;
      consider(c);
    }
  }
  // 3. cutoff form
  {
    gsfft_plan_tuning c = cur;
    c.select_form = cur.select_form == 2 ? 1 : 2;
    consider(c);
  }
  cudaEventDestroy(b.e0);
  cudaEventDestroy(b.e1);
  if (s != GSFFT_OK) return s;
  *best = cur;
  if (best_ms) *best_ms = cur_ms;
  cache_store(cache_path, key, cur, cur_ms);
  return GSFFT_OK;
}

}  // extern "C"
