// Power-of-two complex FFT plans and execution (the pass kernel is in
// fft_pass.cuh).
#include "fft_pass.cuh"

#include <algorithm>

namespace gsfft {

namespace {

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

int dispatch_pass(bool dbl, int logr, const PassArgs &a, long long total_sub, cudaStream_t st) {
  if (dbl) return logr <= 9 ? fft_pass_f64_lo(logr, a, total_sub, st) : fft_pass_f64_hi(logr, a, total_sub, st);
  return logr <= 10 ? fft_pass_f32_lo(logr, a, total_sub, st) : fft_pass_f32_hi(logr, a, total_sub, st);
}

}  // namespace

int fft_plan_init(FftPlan &p, long long n, int precision, int max_batch, int first_logr) {
  fft_plan_free(p);
  if (n < 256 || (n & (n - 1)) != 0) return GSFFT_ERR_UNSUPPORTED;
  int L = 0;
  while ((1LL << L) < n) L++;
  const int one_pass_max = precision == GSFFT_FP64 ? 13 : 14;
  p.n = n;
  p.L = L;
  p.precision = precision;
  if (L <= one_pass_max) {
    if (first_logr > 0) return GSFFT_ERR_PARAM;  // one pass: no first radix to choose
    p.npass = 1;
    p.logR[0] = L;
  } else if (L <= 24) {
    p.npass = 2;
    p.logR[0] = (L + 1) / 2;
    if (first_logr > 0) {
      if (first_logr < 7 || first_logr > one_pass_max || L - first_logr < 7 ||
          L - first_logr > one_pass_max)
        return GSFFT_ERR_PARAM;
      p.logR[0] = first_logr;
    }
    p.logR[1] = L - p.logR[0];
  } else if (L <= 36) {
    if (first_logr > 0) return GSFFT_ERR_PARAM;
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

// FP32 plan whose first pass is a CUDA-core pass of radix 2^(L-6) and whose
// last pass is a tensor-core radix-64 pass (one DFT_64 product per 128
// sub-transforms, both sides read and written in 1 KiB runs): n = 2^L,
// 13 <= L <= 20.
int fft_plan_init_tc64(FftPlan &p, long long n, int max_batch) {
  fft_plan_free(p);
  if (n < 256 || (n & (n - 1)) != 0) return GSFFT_ERR_UNSUPPORTED;
  int L = 0;
  while ((1LL << L) < n) L++;
  if (L < 13 || L > 20) return GSFFT_ERR_UNSUPPORTED;
  p.n = n;
  p.L = L;
  p.precision = GSFFT_MIXED;
  p.npass = 2;
  p.logR[0] = L - 6;
  p.logR[1] = 6;
  p.tc[0] = false;
  p.tc[1] = true;
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
  GS_CHECK(tc_build_F_smem(&p.tc_F));
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
      if (dbl || a.gx || (p.logR[i] != 12 && p.logR[i] != 6)) return GSFFT_ERR_UNSUPPORTED;
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
      s = p.logR[i] == 6 ? launch_tc64_last_pass(t, st) : launch_tc4096_pass(t, st);
    } else {
      s = dispatch_pass(dbl, p.logR[i], a, total_sub, st);
    }
    if (s != GSFFT_OK) return s;
    src = dst;
    Ns <<= p.logR[i];
  }
  return GSFFT_OK;
}

}  // namespace gsfft
