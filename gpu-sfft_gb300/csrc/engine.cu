// Plan and run orchestration: the outer loop of outerLoop.cu:65-190 as one
// stream-ordered sequence of kernels with every buffer allocated at plan time.
//
// Data layout in HBM (T = double in FP64 mode, float in MIXED mode):
//   x            n complex T (caller)             signal
//   filt         w complex T                      filter taps
//   filt_bm      B x TT complex T                 the taps bucket-major (streaming form),
//                                                TT = w/B + 1 rounded up to even
//   hinv         n/B + 1 complex double           conj(H)/|H|^2 around bin 0
//   rsamp        RLFC_loops x W_RLFC T            |FFT_W(restricted x)|^2
//   J2b / J2     RLFC_loops x B_thresh int        RLFC blocks / merged ids
//   bins         loops x B complex T              bucket spectra (in place FFT)
//   bsamp        loops x B T                      |bins|^2
//   J            loops_loc x B_thresh int         heavy buckets per location loop
//   bm_j2, bm_sig  W/32 and loops_loc x W/32 u32  residue bitmaps
//   vote         n u32                            epoch << 8 | count, or (at most 3
//                                                location loops) two n/16-word
//                                                tables of 2-bit counters
//   cand, nodes, mag2, topk_idx, topk             candidate list and results
#include "engine.cuh"

#include <stdlib.h>
#include <string.h>

#include <algorithm>

namespace gsfft {

namespace {

__global__ void convert_taps_kernel(const double2 *__restrict__ src, void *dst, int w, int to_float) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= w) return;
  const double2 v = src[i];
  if (to_float) reinterpret_cast<float2 *>(dst)[i] = make_float2((float)v.x, (float)v.y);
  else reinterpret_cast<double2 *>(dst)[i] = v;
}

// First kernel of a run (launched normally, after everything before it):
// block 0 clears the control block and the row maxima and advances the device
// epoch (a graph replay of the run advances it too); every block zeroes part
// of the residue bitmaps F_l.
__global__ void run_begin_kernel(RunCtl *ctl, unsigned long long *rmax, int nrmax, unsigned *epoch,
                                 unsigned *bm, long long bm_words) {
  pdl_enter();
  if (blockIdx.x == 0) {
    int *c = reinterpret_cast<int *>(ctl);
    for (int i = threadIdx.x; i < (int)(sizeof(RunCtl) / sizeof(int)); i += blockDim.x) c[i] = 0;
    for (int i = threadIdx.x; i < nrmax; i += blockDim.x) rmax[i] = 0ull;
    if (threadIdx.x == 0) *epoch = *epoch + 1u;
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < bm_words;
       i += (long long)gridDim.x * blockDim.x)
    bm[i] = 0u;
}

// the draws of a phased run, for the batch tail (batch_tail.cu)
__global__ void store_draws_kernel(Draws d, Draws *out) {
  if (threadIdx.x == 0) *out = d;
}

// hinv[idx] = conj(H)/|H|^2 with H = filter_freq[(n - d) mod n], d = idx - nb/2,
// followed by the same nb + 1 values rounded to float (the mixed estimate's
// ranking table)
__global__ void hinv_kernel(const double2 *__restrict__ ff, int n, int nb, double2 *hinv) {
  const int idx = blockIdx.x * 256 + threadIdx.x;
  if (idx > nb) return;
  const int d = idx - nb / 2;
  const int dist = (int)(((long long)n - d) & (long long)(n - 1));
  const double2 H = ff[dist];
  const double a2 = __dadd_rn(__dmul_rn(H.x, H.x), __dmul_rn(H.y, H.y));
  const double2 v = make_double2(H.x / a2, -H.y / a2);
  hinv[idx] = v;
  reinterpret_cast<float2 *>(hinv + nb + 1)[idx] = make_float2((float)v.x, (float)v.y);
}

template <typename P> int alloc(P **p, size_t bytes) {
  cudaError_t e = cudaMalloc((void **)p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    set_last_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    return GSFFT_ERR_ALLOC;
  }
  return GSFFT_OK;
}

}  // namespace

int validate_params(const gsfft_params &p) {
  auto pow2 = [](long long v) { return v > 0 && (v & (v - 1)) == 0; };
  if (!pow2(p.n) || p.n < 256 || p.n > (1 << 30)) return GSFFT_ERR_PARAM;
  if (!pow2(p.B) || p.B > p.n || !pow2(p.W_RLFC) || p.W_RLFC > p.n) return GSFFT_ERR_PARAM;
  if (p.B_thresh < 1 || p.B_thresh >= p.B || p.B_thresh >= p.W_RLFC) return GSFFT_ERR_PARAM;
  if (p.loops_loc < 1 || p.loops_thresh < 1 || p.loops_thresh > p.loops_loc) return GSFFT_ERR_PARAM;
  if (p.loops != p.loops_loc + p.loops_est || p.loops > MAX_LOOPS || p.loops_loc > 255)
    return GSFFT_ERR_PARAM;
  if (p.RLFC_loops < 1 || p.RLFC_loops > MAX_RLFC_LOOPS) return GSFFT_ERR_PARAM;
  if (p.w < 1 || p.w > p.n) return GSFFT_ERR_PARAM;
  // the window of a bucket must be shorter than W_RLFC, and W_RLFC < n
  if (p.W_RLFC >= p.n || p.W_RLFC <= p.n / p.B || p.W_RLFC < 256) return GSFFT_ERR_UNSUPPORTED;
  if (p.B < 256) return GSFFT_ERR_UNSUPPORTED;
  return GSFFT_OK;
}

int plan_create(const gsfft_params &pp, int precision, unsigned flags, int max_candidates,
                Plan **out, const gsfft_plan_tuning *tuning) {
  *out = nullptr;
  GS_CHECK(validate_params(pp));
  if (precision != GSFFT_FP64 && precision != GSFFT_MIXED) return GSFFT_ERR_PARAM;
  gsfft_plan_tuning tn = {};
  if (tuning) tn = *tuning;
  if (tn.perm_filter_form < 0 || tn.perm_filter_form > 2 || tn.select_form < 0 ||
      tn.select_form > 2 || tn.row_groups < 0 || tn.bucket_first_radix < 0 ||
      tn.rlfc_first_radix < 0)
    return GSFFT_ERR_PARAM;
  if (tn.perm_filter_form == 1) flags = (flags | GSFFT_FLAG_FORCE_STREAM) & ~GSFFT_FLAG_FORCE_GATHER;
  if (tn.perm_filter_form == 2) flags = (flags | GSFFT_FLAG_FORCE_GATHER) & ~GSFFT_FLAG_FORCE_STREAM;
  Plan *P = new Plan();
  P->p = pp;
  P->precision = precision;
  P->flags = flags;
  P->cap = max_candidates > 0 ? max_candidates : 524288;
  const gsfft_params &p = P->p;
  const size_t T = precision == GSFFT_FP64 ? 8 : 4, V = 2 * T;
  P->es = V;
  int s = GSFFT_OK;
  const int nb = p.n / p.B;
  const size_t wW = (size_t)p.W_RLFC / 32;
#define A(ptr, bytes) \
  if (s == GSFFT_OK) s = alloc(&P->ptr, (bytes))
  A(filt, V * p.w);
  A(hinv, hinv_bytes(nb));
  A(rsamp, T * (size_t)p.RLFC_loops * p.W_RLFC);
  A(J2b, sizeof(int) * (size_t)p.RLFC_loops * p.B_thresh);
  A(J2, sizeof(int) * (size_t)p.RLFC_loops * p.B_thresh);
  A(bins, V * (size_t)p.loops * p.B);
  A(bsamp, T * (size_t)p.loops * p.B);
  A(J, sizeof(int) * (size_t)p.loops_loc * p.B_thresh);
  A(bm_j2, sizeof(unsigned) * wW);
  A(bm_sig, sizeof(unsigned) * wW * p.loops_loc);
  A(tile_tmp, sizeof(unsigned) * (wW / 2048 + 2));
  A(vote, sizeof(unsigned) * (size_t)p.n);
  A(cand, sizeof(int) * (size_t)P->cap);
  A(cnt, sizeof(int) * (size_t)p.B_thresh);
  A(blk, sizeof(int) * (size_t)vote_block_ints(p.B_thresh));
  A(nodes, sizeof(DevNode) * (size_t)P->cap);
  A(mag2, sizeof(double) * (size_t)P->cap);
  A(topk_idx, sizeof(int) * (size_t)p.k + 16);
  A(topk, sizeof(DevNode) * (size_t)p.k + 16);
  A(ctl, sizeof(RunCtl));
  A(d_epoch, sizeof(unsigned) * 4);
  A(d_draws, sizeof(Draws));
  A(rmax, sizeof(unsigned long long) * (size_t)(p.RLFC_loops + p.loops));
  // perm+filter form: one ordered pass over x when that moves fewer DRAM bytes
  // than loops*w + RLFC_loops*W random reads (~80 bytes per random read)
  {
    const double stream_bytes = (double)p.n * V + 2.0 * p.RLFC_loops * p.W_RLFC * V;
    const double gather_bytes = 80.0 * ((double)p.loops * p.w + (double)p.RLFC_loops * p.W_RLFC);
    const bool ok = stream_pf_supported(p.n, p.B, p.loops, p.W_RLFC, p.RLFC_loops) &&
                    p.w / p.B < 32 && !(flags & GSFFT_FLAG_QUIRK_RESIDUE);
    P->use_stream = ok && !(flags & GSFFT_FLAG_FORCE_GATHER) &&
                    ((flags & GSFFT_FLAG_FORCE_STREAM) ||
                     (precision == GSFFT_MIXED && stream_bytes < gather_bytes));
  }
  if (tn.perm_filter_form == 1 && !P->use_stream) {
    plan_destroy(P);
    return GSFFT_ERR_PARAM;  // the ordered pass does not support these sizes
  }
  if (P->use_stream) {
    P->groups = stream_pf_groups(p.n, p.B, p.w, p.loops, precision);
    if (tn.row_groups > 0) {
      if (!stream_pf_groups_valid(p.n, p.B, tn.row_groups, precision)) {
        plan_destroy(P);
        return GSFFT_ERR_PARAM;
      }
      P->groups = tn.row_groups;
    }
    A(ybuf, V * (size_t)p.RLFC_loops * p.W_RLFC);
    A(bpart, V * (size_t)P->groups * p.loops * p.B);
    A(filt_bm, V * (size_t)stream_taps_count(p.w, p.B));
  }
#undef A
  P->floor_rel = (flags & GSFFT_FLAG_RAW_SELECTION) ? 0.0 : 1e-10;
  // 2-bit vote counters (n/4 bytes, L2-resident) when no count can pass 3
  P->packed_vote = p.loops_loc <= 3;
  if (s == GSFFT_OK) {
    int t = GSFFT_ERR_UNSUPPORTED;
    // tensor-core bucket FFT: the radix-64 last pass where B allows it
    // (2^13 .. 2^20), else the radix-4096 first pass.  By default MIXED
    // plans take it for 2^17 <= B <= 2^20: on the n = 2^27, k = 16000 step it
    // measured 0.5007 against 0.5124 ms, while the batch of small signals
    // (smaller B, one tile per CTA) ran slower with it.
    const bool tc_asked = (flags & GSFFT_FLAG_TC_BUCKET_FFT) != 0;
    const bool tc_default = !(flags & GSFFT_FLAG_CC_BUCKET_FFT) && p.B >= (1 << 17) && p.B <= (1 << 20);
    if (precision == GSFFT_MIXED && (tc_asked || tc_default)) {
      t = fft_plan_init_tc64(P->fftB, p.B, p.loops);
      if (t == GSFFT_ERR_UNSUPPORTED && tc_asked) t = fft_plan_init_tc(P->fftB, p.B, p.loops);
    }
    P->tc_bucket = t == GSFFT_OK;
    if (!P->tc_bucket) s = fft_plan_init(P->fftB, p.B, precision, p.loops, tn.bucket_first_radix);
  }
  if (s == GSFFT_OK) {
    // the RLFC transform reads the streaming pass's sub-samples; its first
    // pass can then run on the tensor cores (the gather form fuses a strided
    // gather into that pass instead)
    int t = GSFFT_ERR_UNSUPPORTED;
    if (precision == GSFFT_MIXED && (flags & GSFFT_FLAG_TC_RLFC_FFT) && P->use_stream)
      t = fft_plan_init_tc(P->fftW, p.W_RLFC, p.RLFC_loops);
    P->tc_rlfc = t == GSFFT_OK;
    if (!P->tc_rlfc)
      s = fft_plan_init(P->fftW, p.W_RLFC, precision, p.RLFC_loops, tn.rlfc_first_radix);
  }
  if (s == GSFFT_OK) s = select_scratch_init(P->selB, p.loops_loc, p.B);
  if (s == GSFFT_OK) s = select_scratch_init(P->selW, p.RLFC_loops, p.W_RLFC);
  if (s == GSFFT_OK) s = select_scratch_init(P->selK, 1, P->cap);
  P->selB.single_launch = P->selW.single_launch = P->selK.single_launch = tn.select_form != 2;
  // record the shapes in use
  P->tuning.perm_filter_form = P->use_stream ? 1 : 2;
  P->tuning.row_groups = P->use_stream ? P->groups : 0;
  P->tuning.bucket_first_radix = P->fftB.npass == 2 && !P->tc_bucket ? P->fftB.logR[0] : 0;
  P->tuning.rlfc_first_radix = P->fftW.npass == 2 && !P->tc_rlfc ? P->fftW.logR[0] : 0;
  P->tuning.select_form = tn.select_form == 2 ? 2 : 1;
  if (s == GSFFT_OK &&
      (cudaStreamCreateWithFlags(&P->side, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&P->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&P->ev_join, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&P->ev_bins, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&P->ev_rsel, cudaEventDisableTiming) != cudaSuccess ||
       cudaStreamCreateWithFlags(&P->aux, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&P->ev_vclr, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&P->ev_voted, cudaEventDisableTiming) != cudaSuccess)) {
    set_last_error("plan init: %s", cudaGetErrorString(cudaGetLastError()));
    s = GSFFT_ERR_CUDA;
  }
  if (s == GSFFT_OK) {
    cudaError_t e = cudaMemset(P->vote, 0, sizeof(unsigned) * (size_t)p.n);
    if (e == cudaSuccess) e = cudaMemset(P->ctl, 0, sizeof(RunCtl));
    if (e == cudaSuccess) e = cudaMemset(P->d_epoch, 0, sizeof(unsigned) * 4);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      set_last_error("plan init: %s", cudaGetErrorString(e));
      s = GSFFT_ERR_CUDA;
    }
  }
  if (s != GSFFT_OK) {
    plan_destroy(P);
    return s;
  }
  P->epoch = 0;
  *out = P;
  return GSFFT_OK;
}

void plan_destroy(Plan *P) {
  if (!P) return;
  void *ptrs[] = {P->filt, P->hinv, P->rsamp, P->J2b, P->J2, P->bins, P->bsamp, P->J,
                  P->bm_j2, P->bm_sig, P->tile_tmp, P->vote, P->cand, P->cnt, P->blk,
                  P->nodes, P->mag2, P->topk_idx, P->topk, P->ctl, P->rmax, P->ybuf, P->bpart,
                  P->filt_bm, P->d_epoch, P->d_draws};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  for (cudaEvent_t e : P->events) cudaEventDestroy(e);
  if (P->ev_fork) cudaEventDestroy(P->ev_fork);
  if (P->ev_join) cudaEventDestroy(P->ev_join);
  if (P->ev_bins) cudaEventDestroy(P->ev_bins);
  if (P->ev_rsel) cudaEventDestroy(P->ev_rsel);
  if (P->ev_vclr) cudaEventDestroy(P->ev_vclr);
  if (P->ev_voted) cudaEventDestroy(P->ev_voted);
  if (P->aux) cudaStreamDestroy(P->aux);
  if (P->side) cudaStreamDestroy(P->side);
  fft_plan_free(P->fftB);
  fft_plan_free(P->fftW);
  select_scratch_free(P->selB);
  select_scratch_free(P->selW);
  select_scratch_free(P->selK);
  delete P;
}

// Clears the packed vote table the next run uses: table ((epoch + 1) & 1) of
// the two n/16-word tables, epoch being this run's (advanced by its first kernel).
__global__ void vote_clear_kernel(unsigned *vote, unsigned words, const unsigned *epoch) {
  uint4 *t = reinterpret_cast<uint4 *>(vote + (((*epoch + 1u) & 1u) ? words : 0u));
  const unsigned n4 = words / 4;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x)
    t[i] = make_uint4(0u, 0u, 0u, 0u);
}

int launch_vote_clear(unsigned *vote, int n, const unsigned *d_epoch, cudaStream_t st) {
  const unsigned words = (unsigned)n / 16;
  const unsigned blocks = std::min(608u, (words / 4 + 255) / 256);
  vote_clear_kernel<<<blocks, 256, 0, st>>>(vote, words, d_epoch);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_hinv(const double2 *d_ff, int n, int nb, double2 *hinv, cudaStream_t st) {
  hinv_kernel<<<(nb + 1 + 255) / 256, 256, 0, st>>>(d_ff, n, nb, hinv);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int launch_convert_taps(const double2 *d_ft, void *dst, int w, bool to_float, cudaStream_t st) {
  convert_taps_kernel<<<(w + 255) / 256, 256, 0, st>>>(d_ft, dst, w, to_float ? 1 : 0);
  GS_LAUNCHED();
  return GSFFT_OK;
}

int plan_set_filter(Plan *P, const void *d_ft, const void *d_ff, cudaStream_t st) {
  const gsfft_params &p = P->p;
  if (!d_ft || !d_ff) return GSFFT_ERR_PARAM;
  GS_CHECK(launch_convert_taps((const double2 *)d_ft, P->filt, p.w, P->precision == GSFFT_MIXED, st));
  if (P->use_stream) GS_CHECK(launch_stream_taps(P->precision, P->filt, p.w, p.B, P->filt_bm, st));
  GS_CHECK(launch_hinv((const double2 *)d_ff, p.n, p.n / p.B, P->hinv, st));
  GS_CUDA(cudaStreamSynchronize(st));
  P->filter_set = true;
  return GSFFT_OK;
}

int plan_epoch_advance(Plan *P, cudaStream_t st) {
  // epoch-tagged vote table: cleared only when the 24-bit epoch would wrap
  if (P->epoch + 1u >= (1u << 24)) {
    GS_CUDA(cudaMemsetAsync(P->vote, 0, sizeof(unsigned) * (size_t)P->p.n, st));
    GS_CUDA(cudaMemsetAsync(P->d_epoch, 0, sizeof(unsigned), st));
    P->epoch = 0;
  }
  P->epoch++;  // the run's first kernel makes the same step on the device
  return GSFFT_OK;
}

int plan_run(Plan *P, const void *d_x, const int *offs, const int *a, const int *ai,
             cudaStream_t st, bool capturing, int phases) {
  if (!P->filter_set) return GSFFT_ERR_STATE;
  if (phases < 1 || phases > PH_ALL) return GSFFT_ERR_PARAM;
  const gsfft_params &p = P->p;
  const int before = g_launch_counter;
  Draws d;
  memset(&d, 0, sizeof(d));
  if (!(phases & PH_FRONT)) {
    d = P->draws;  // the draws of the front phase queued last
  } else {
  for (int r = 0; r < p.RLFC_loops; r++) {
    if (offs[r] < 0 || offs[r] >= p.n / p.W_RLFC) return GSFFT_ERR_PARAM;
    d.offs[r] = offs[r];
  }
  for (int l = 0; l < p.loops; l++) {
    if ((a[l] & 1) == 0 || (ai[l] & 1) == 0 || a[l] <= 0 || ai[l] <= 0 || a[l] >= p.n || ai[l] >= p.n)
      return GSFFT_ERR_PARAM;
    if ((unsigned)a[l] * (unsigned)ai[l] % (unsigned)p.n != 1u) return GSFFT_ERR_PARAM;
    d.a[l] = a[l];
    d.ai[l] = ai[l];
  }
  P->draws = d;
  }
  if (!capturing && (phases & PH_FRONT)) GS_CHECK(plan_epoch_advance(P, st));
  const int kb = P->precision == GSFFT_FP64 ? 8 : 4;
  if (phases & PH_FRONT) {
    // about eight bitmap words per thread, at most 128 CTAs
    const long long bm_words = (long long)(p.W_RLFC / 32) * p.loops_loc;
    const int grid = (int)std::min<long long>(128, std::max<long long>(1, (bm_words + 2047) / 2048));
    run_begin_kernel<<<grid, 256, 0, st>>>(P->ctl, (unsigned long long *)P->rmax, p.RLFC_loops + p.loops,
                                           P->d_epoch, P->bm_sig, bm_words);
    GS_LAUNCHED();
    if (phases != PH_ALL) {
      // a phased run (batch tail): the tail reads this run's draws from the device
      store_draws_kernel<<<1, 32, 0, st>>>(d, P->d_draws);
      GS_LAUNCHED();
    }
  }
  void *rmax_w = P->rmax;  // RLFC rows, then bucket rows (u64 in FP64, u32 in FP32)
  void *rmax_b = (char *)P->rmax + (size_t)kb * p.RLFC_loops;
  cudaEvent_t *ev = nullptr;
  if (P->timing && !capturing && phases == PH_ALL && P->timed_runs < 512) {
    const size_t need = (size_t)(P->timed_runs + 1) * (2 * ST_COUNT);
    while (P->events.size() < need) {
      cudaEvent_t e;
      GS_CUDA(cudaEventCreate(&e));
      P->events.push_back(e);
    }
    ev = &P->events[(size_t)P->timed_runs * (2 * ST_COUNT)];
    P->timed_runs++;
  }
#define BEGIN(s) \
  if (ev) GS_CUDA(cudaEventRecord(ev[2 * (s)], st))
#define END(s) \
  if (ev) GS_CUDA(cudaEventRecord(ev[2 * (s) + 1], st))
#define BEGIN_ON(s, q) \
  if (ev) GS_CUDA(cudaEventRecord(ev[2 * (s)], q))
#define END_ON(s, q) \
  if (ev) GS_CUDA(cudaEventRecord(ev[2 * (s) + 1], q))
  const bool quirk = (P->flags & GSFFT_FLAG_QUIRK_RESIDUE) != 0;

  if (phases & PH_FRONT) {
  // A5 (+ RLFC sub-sampling when streaming): bins of every loop
  BEGIN(ST_PERM_FILTER);
  if (P->use_stream)
    GS_CHECK(launch_perm_filter_stream(P->precision, d_x, p.n, P->filt_bm, p.w, p.B, p.loops, d,
                                       P->bpart, p.RLFC_loops, P->ybuf, p.W_RLFC, &P->ctl->err, st,
                                       P->groups));
  else
    GS_CHECK(launch_perm_filter(P->precision, d_x, p.n, P->filt, p.w, p.B, p.loops, d, quirk,
                                P->bins, st));
  END(ST_PERM_FILTER);

  // A6: bucket FFT of every loop, cutoff of the location loops.  They need
  // only the perm+filter, so they run on the plan's side stream beside A4's
  // RLFC chain.  The location loops' rows go first: the cutoff needs only
  // them, and the main stream waits for the cutoff before the voting.  The
  // estimation loops' rows follow on the side stream, beside the voting; the
  // main stream waits for them before the estimation.
  GS_CUDA(cudaEventRecord(P->ev_fork, st));
  GS_CUDA(cudaStreamWaitEvent(P->side, P->ev_fork, 0));

  BEGIN_ON(ST_BUCKET_FFT, P->side);
  const void *bsrc = P->bins;
  {
    FftIo io;
    io.samples = P->bsamp;
    io.row_max = rmax_b;
    io.err = &P->ctl->err;
    const void *src = P->bins;
    if (P->use_stream) {
      // The row-group partials are added in group order: by a kernel over
      // every bin when there are several (a pass over few long rows would
      // read them on a handful of CTAs), else the single group is the input.
      if (P->groups > 1)
        GS_CHECK(launch_sum_partials(P->precision, P->bpart, P->groups, (long long)p.loops * p.B,
                                     P->bins, P->side));
      else
        src = P->bpart;
    }
    GS_CHECK(fft_exec(P->fftB, src, P->bins, p.loops_loc, -1, io, P->side));
    bsrc = src;
  }
  END_ON(ST_BUCKET_FFT, P->side);
  BEGIN_ON(ST_CUTOFF, P->side);
  GS_CHECK(select_top(P->bsamp, kb, p.B, nullptr, p.B_thresh, p.loops_loc, p.B, P->J, p.B_thresh,
                      nullptr, P->selB, P->side, rmax_b, P->floor_rel));
  END_ON(ST_CUTOFF, P->side);

  GS_CUDA(cudaEventRecord(P->ev_join, P->side));

  // A4: RLFC -- W-point FFT of the sub-sampled signal, |.|^2 epilogue, cutoff
  BEGIN(ST_RLFC_FFT);
  {
    FftIo io;
    const void *src = nullptr;
    if (P->use_stream) {
      src = P->ybuf;
    } else {
      io.gather_x = d_x;  // strided gather fused into the first FFT pass
      for (int r = 0; r < p.RLFC_loops; r++) io.gather_offsets[r] = d.offs[r];
      io.gather_stride = p.n / p.W_RLFC;
    }
    io.samples = P->rsamp;
    io.row_max = rmax_w;
    io.write_complex = false;
    GS_CHECK(fft_exec(P->fftW, src, P->rsamp, p.RLFC_loops, -1, io, st));
  }
  END(ST_RLFC_FFT);
  BEGIN(ST_RLFC_SELECT);
  GS_CHECK(select_top(P->rsamp, kb, p.W_RLFC, nullptr, p.B_thresh, p.RLFC_loops, p.W_RLFC, P->J2b,
                      p.B_thresh, nullptr, P->selW, st, rmax_w, P->floor_rel));
  END(ST_RLFC_SELECT);

  // the estimation loops' bucket FFT (side stream), queued behind the RLFC
  // cutoff: that cutoff is a cooperative launch whose whole grid must be
  // resident, so the FFT's blocks would hold back its start
  GS_CUDA(cudaEventRecord(P->ev_rsel, st));
  GS_CUDA(cudaStreamWaitEvent(P->side, P->ev_rsel, 0));
  if (p.loops > p.loops_loc) {
    FftIo io;  // complex bins only: the estimation reads no samples
    io.err = &P->ctl->err;
    const size_t off = (size_t)(P->precision == GSFFT_FP64 ? 16 : 8) * p.loops_loc * p.B;
    GS_CHECK(fft_exec(P->fftB, (const char *)bsrc + off, (char *)P->bins + off, p.loops - p.loops_loc, -1,
                      io, P->side));
  }
  GS_CUDA(cudaEventRecord(P->ev_bins, P->side));
  BEGIN(ST_J2);
  // F_l needs only the set of J2 ids, not the sorted list; the sorted J2
  // (num_RLFC ids) is compacted on demand by plan_debug
  GS_CHECK(launch_sigma_from_blocks(P->J2b, p.RLFC_loops * p.B_thresh, p.W_RLFC, p.loops_loc, d,
                                    P->bm_sig, P->ctl, st));
  END(ST_J2);

  // the side stream joins back before the voting, and the voting waits for
  // the clear of its packed table, queued by the previous eager run.  A clear
  // recorded in a captured graph is a graph node that every replay runs before
  // it completes (and an event recorded in a capture cannot be waited on
  // outside it); a capture needs no wait either, its replays following one
  // another on a stream.
  GS_CUDA(cudaStreamWaitEvent(st, P->ev_join, 0));
  if (P->packed_vote && !capturing && P->vclr_eager) GS_CUDA(cudaStreamWaitEvent(st, P->ev_vclr, 0));
  }  // front

  if (phases & PH_VOTE) {
  // A7: voting, one location loop after the other
  BEGIN(ST_VOTE);
  const size_t wW = (size_t)p.W_RLFC / 32;
  for (int l = 0; l < p.loops_loc; l++)
    GS_CHECK(launch_vote_loop(l, P->J + (size_t)l * p.B_thresh, p.B_thresh, p.n, p.B, p.W_RLFC,
                              P->bm_sig + wW * l, d, p.loops_thresh, P->d_epoch, P->vote, P->cand,
                              P->cap, P->cnt, P->blk, P->ctl, l + 1 >= p.loops_thresh, st,
                              P->packed_vote));
  END(ST_VOTE);
  }  // voting

  if (phases & PH_EST) {
  if (P->packed_vote) {
    // the voting is done: clear the other packed table for the next run,
    // beside this run's estimation and top-k
    GS_CUDA(cudaEventRecord(P->ev_voted, st));
    GS_CUDA(cudaStreamWaitEvent(P->aux, P->ev_voted, 0));
    GS_CHECK(launch_vote_clear(P->vote, p.n, P->d_epoch, P->aux));
    GS_CUDA(cudaEventRecord(P->ev_vclr, P->aux));
    P->vclr_eager = !capturing;
  }
  // A8: estimation (after the estimation loops' bucket FFT); A9: k largest
  GS_CUDA(cudaStreamWaitEvent(st, P->ev_bins, 0));
  BEGIN(ST_ESTIMATE);
  // the grid covers 8k candidates at one per thread (about 4.8k at the
  // 2^27 / 16000 workload); more are taken by the grid-stride loop
  GS_CHECK(launch_estimate(P->precision, P->cand, P->ctl, P->cap,
                           (int)std::min<long long>(P->cap, 8LL * p.k), P->bins, p.loops, p.n, p.B, d,
                           P->hinv, P->nodes, P->mag2, st));
  END(ST_ESTIMATE);
  }  // estimation

  if (phases & PH_TOPK) {
  BEGIN(ST_TOPK);
  // k largest |estimate|^2: 8-byte keys (FP64 path) or 4-byte keys (mixed path)
  GS_CHECK(select_top(P->mag2, P->precision == GSFFT_FP64 ? 8 : 4, P->cap, &P->ctl->cand_count, p.k, 1,
                      P->cap, P->topk_idx, p.k,
                      &P->ctl->n_topk, P->selK, st));
  GS_CHECK(launch_gather_nodes(P->nodes, P->topk_idx, &P->ctl->n_topk, p.k, P->topk, st));
  END(ST_TOPK);
  // the clear of the next run's vote table (queued after the voting) joins the
  // run here; it has long finished beside the estimation and top-k
  if (P->packed_vote && (phases & PH_EST)) GS_CUDA(cudaStreamWaitEvent(st, P->ev_vclr, 0));
  }  // top-k
#undef BEGIN
#undef END
#undef BEGIN_ON
#undef END_ON
  if (phases == PH_ALL) P->launches_per_run = g_launch_counter - before;
  if (phases & PH_TOPK) P->ran = true;
  return GSFFT_OK;
}

int plan_results(Plan *P, Node *h_nodes, int nodes_cap, int *I_F, Node *h_topk, int topk_cap,
                 int *n_topk, cudaStream_t st) {
  if (!P->ran) return GSFFT_ERR_STATE;
  RunCtl c;
  GS_CUDA(cudaMemcpyAsync(&c, P->ctl, sizeof(RunCtl), cudaMemcpyDeviceToHost, st));
  GS_CUDA(cudaStreamSynchronize(st));
  const int count = c.cand_count < P->cap ? c.cand_count : P->cap;
  if (I_F) *I_F = c.cand_count;
  if (h_nodes && nodes_cap > 0) {
    const int m = count < nodes_cap ? count : nodes_cap;
    if (m > 0)
      GS_CUDA(cudaMemcpyAsync(h_nodes, P->nodes, sizeof(Node) * m, cudaMemcpyDeviceToHost, st));
  }
  if (n_topk) *n_topk = c.n_topk;
  if (h_topk && topk_cap > 0) {
    const int m = c.n_topk < topk_cap ? c.n_topk : topk_cap;
    if (m > 0)
      GS_CUDA(cudaMemcpyAsync(h_topk, P->topk, sizeof(Node) * m, cudaMemcpyDeviceToHost, st));
  }
  GS_CUDA(cudaStreamSynchronize(st));
  if (c.err) {
    set_last_error(
        "a bounded device-side wait gave up (streaming perm+filter, tensor-core FFT or batch voting)");
    return GSFFT_ERR_TIMEOUT;
  }
  return c.overflow ? GSFFT_ERR_CAPACITY : GSFFT_OK;
}

const char *stage_name(int i) {
  static const char *names[ST_COUNT] = {"rlfc_fft", "rlfc_select", "j2_merge", "perm_filter",
                                        "bucket_fft", "cutoff", "vote", "estimate", "topk"};
  return (i >= 0 && i < ST_COUNT) ? names[i] : "";
}

int plan_enable_timing(Plan *P, bool on) {
  P->timing = on;
  P->timed_runs = 0;
  return GSFFT_OK;
}

int plan_stage_times(Plan *P, float *ms_avg, int max_stages, int *runs) {
  GS_CUDA(cudaDeviceSynchronize());
  const int R = P->timed_runs;
  if (runs) *runs = R;
  for (int sidx = 0; sidx < ST_COUNT && sidx < max_stages; sidx++) {
    double acc = 0.0;
    for (int r = 0; r < R; r++) {
      float ms = 0.f;
      cudaEvent_t *e = &P->events[(size_t)r * (2 * ST_COUNT)];
      GS_CUDA(cudaEventElapsedTime(&ms, e[2 * sidx], e[2 * sidx + 1]));
      acc += ms;
    }
    ms_avg[sidx] = R ? (float)(acc / R) : 0.f;
  }
  P->timed_runs = 0;
  return GSFFT_OK;
}

int plan_debug(Plan *P, int *h_J2, int *num_RLFC, int *h_J, void *h_bins, cudaStream_t st) {
  if (!P->ran) return GSFFT_ERR_STATE;
  const gsfft_params &p = P->p;
  if (h_J2 || num_RLFC)  // sorted, de-duplicated union of the last run's RLFC blocks
    GS_CHECK(launch_j2_merge(P->J2b, p.RLFC_loops * p.B_thresh, p.W_RLFC, P->bm_j2, P->J2, P->ctl,
                             P->tile_tmp, st));
  GS_CUDA(cudaStreamSynchronize(st));
  RunCtl c;
  GS_CUDA(cudaMemcpy(&c, P->ctl, sizeof(RunCtl), cudaMemcpyDeviceToHost));
  if (num_RLFC) *num_RLFC = c.num_rlfc;
  if (h_J2 && c.num_rlfc > 0)
    GS_CUDA(cudaMemcpy(h_J2, P->J2, sizeof(int) * c.num_rlfc, cudaMemcpyDeviceToHost));
  if (h_J)
    GS_CUDA(cudaMemcpy(h_J, P->J, sizeof(int) * (size_t)p.loops_loc * p.B_thresh,
                       cudaMemcpyDeviceToHost));
  if (h_bins)
    GS_CUDA(cudaMemcpy(h_bins, P->bins, P->es * (size_t)p.loops * p.B, cudaMemcpyDeviceToHost));
  return GSFFT_OK;
}

}  // namespace gsfft
