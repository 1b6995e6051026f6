// A2: flat-window filter design on the GPU, FP64 throughout.
//
// Reference: make_multiple_t (cuExperiment.cu:277-448) with kernels K1-K4
// (:537-601) and cuShift (:507-522).  The reference runs two n-long loops on
// the host over managed memory (boxcar sum :389-396, phase ramp :410-420);
// both are sequential recurrences.  Here:
//   1. win[i] = T_{w-1}(t0 cos(pi i / w)) * tol, NaN -> 0      (K1, :538-552)
//   2. DFT_w(win) by Bluestein over power-of-two FFTs (w is odd)  (:305-308)
//   3. rotate by w/2, drop the imaginary part, place the halves around
//      index 0 of g[n] (one kernel instead of cuShift + K2 + two memcpys)
//   4. G = FFT_n(g)                                                (:362-365)
//   5. boxcar: ff[(i + b_f/2) mod n] = sum_{j=i}^{i+b_f-1} G[j mod n]; each
//      CTA computes the sum at the start of its 8192-output tile directly and
//      the rest as that sum plus a block prefix scan of G[j+b_f] - G[j]
//   6. ff /= max|ff| (K3), ff *= exp(-2 pi i ((w/2) i mod n) / n), the angle
//      reduced exactly in integers (no recurrence)
//   7. filter_time = IFFT_n(ff)[0:w] / n                           (:425-443, K4)
#include "engine.cuh"

namespace gsfft {

namespace {

constexpr int FT = 256;

__device__ double cheb(double m, double x) {  // cuExperiment.cu:593-601
  if (fabs(x) <= 1) return cos(m * acos(x));
  return cosh(m * acosh(x));
}

__global__ void cheb_window_kernel(double2 *win, int w, double t0, double tol) {
  const int i = blockIdx.x * FT + threadIdx.x;
  if (i >= w) return;
  const double v = cheb((double)(w - 1), t0 * cos(M_PI * i / (w))) * tol;
  win[i] = make_double2(isnan(v) ? 0.0 : v, 0.0);
}

// chirp c[m] = exp(-pi i (m^2 mod 2N) / N)
__device__ __forceinline__ double2 chirp(long long m, long long N) {
  const unsigned long long mm = ((unsigned long long)m * (unsigned long long)m) % (unsigned long long)(2 * N);
  double s, c;
  sincospi((double)mm / (double)N, &s, &c);
  return make_double2(c, -s);
}

__global__ void bluestein_prep_kernel(const double2 *__restrict__ x, long long N, long long M,
                                      double2 *a, double2 *b) {
  const long long m = (long long)blockIdx.x * FT + threadIdx.x;
  if (m >= M) return;
  double2 av = make_double2(0.0, 0.0), bv = make_double2(0.0, 0.0);
  if (m < N) {
    const double2 c = chirp(m, N);
    av = cmul(x[m], c);
    bv = make_double2(c.x, -c.y);
  } else if (M - m < N) {
    const double2 c = chirp(M - m, N);
    bv = make_double2(c.x, -c.y);
  }
  a[m] = av;
  b[m] = bv;
}

__global__ void pointwise_mul_kernel(double2 *a, const double2 *__restrict__ b, long long M) {
  const long long m = (long long)blockIdx.x * FT + threadIdx.x;
  if (m < M) a[m] = cmul(a[m], b[m]);
}

__global__ void bluestein_post_kernel(const double2 *__restrict__ conv, long long N, long long M,
                                      double2 *X) {
  const long long k = (long long)blockIdx.x * FT + threadIdx.x;
  if (k >= N) return;
  double2 v = conv[k];
  v.x /= (double)M;
  v.y /= (double)M;
  X[k] = cmul(v, chirp(k, N));
}

// g[j] = Re X[j] (j < h), g[n-h+j] = Re X[j+h+1] (j < h), else 0; h = w/2
__global__ void place_kernel(const double2 *__restrict__ X, int w, int n, double2 *g) {
  const long long i = (long long)blockIdx.x * FT + threadIdx.x;
  if (i >= n) return;
  const int h = w / 2;
  double v = 0.0;
  if (i < h) v = X[i].x;
  else if (i >= n - h) v = X[i - (n - h) + h + 1].x;
  g[i] = make_double2(v, 0.0);
}

constexpr int BOX_TILE = 8192;
constexpr int BOX_PER = BOX_TILE / FT;  // 32 outputs per thread

__global__ void __launch_bounds__(FT)
boxcar_kernel(const double2 *__restrict__ G, int n, int b_f, double2 *ff,
              unsigned long long *max_bits) {
  __shared__ double2 red[FT];
  __shared__ double2 scan[FT];
  const long long i0 = (long long)blockIdx.x * BOX_TILE;
  const unsigned long long nm = (unsigned long long)n - 1ull;
  // window sum at i0, by a block reduction in fixed order
  double2 s = make_double2(0.0, 0.0);
  for (int j = threadIdx.x; j < b_f; j += FT) {
    const double2 v = G[(i0 + j) & nm];
    s.x += v.x;
    s.y += v.y;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = FT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[threadIdx.x].x += red[threadIdx.x + o].x;
      red[threadIdx.x].y += red[threadIdx.x + o].y;
    }
    __syncthreads();
  }
  const double2 base = red[0];
  // per-thread sum of the differences over its 32 outputs
  const long long t0 = i0 + (long long)threadIdx.x * BOX_PER;
  double2 d = make_double2(0.0, 0.0);
  for (int q = 0; q < BOX_PER; q++) {
    const double2 in = G[(t0 + q + b_f) & nm], out = G[(t0 + q) & nm];
    d.x += in.x - out.x;
    d.y += in.y - out.y;
  }
  scan[threadIdx.x] = d;
  __syncthreads();
  // Hillis-Steele inclusive scan over the 256 thread totals
  for (int o = 1; o < FT; o <<= 1) {
    double2 v = scan[threadIdx.x];
    if (threadIdx.x >= o) {
      v.x += scan[threadIdx.x - o].x;
      v.y += scan[threadIdx.x - o].y;
    }
    __syncthreads();
    scan[threadIdx.x] = v;
    __syncthreads();
  }
  double2 cur = base;
  if (threadIdx.x > 0) {
    cur.x += scan[threadIdx.x - 1].x;
    cur.y += scan[threadIdx.x - 1].y;
  }
  const int off = b_f / 2;
  double mx = 0.0;
  for (int q = 0; q < BOX_PER; q++) {
    const long long i = t0 + q;
    if (i < n) {
      ff[(i + off) & nm] = cur;
      mx = fmax(mx, sqrt(cur.x * cur.x + cur.y * cur.y));
    }
    const double2 in = G[(i + b_f) & nm], out = G[i & nm];
    cur.x += in.x - out.x;
    cur.y += in.y - out.y;
  }
  atomicMax(max_bits, (unsigned long long)__double_as_longlong(mx));
}

__global__ void normalize_ramp_kernel(double2 *ff, int n, int h, const unsigned long long *max_bits) {
  const long long i = (long long)blockIdx.x * FT + threadIdx.x;
  if (i >= n) return;
  const double mx = __longlong_as_double((long long)*max_bits);
  double2 v = ff[i];
  v.x /= mx;
  v.y /= mx;
  const long long m = ((long long)h * i) % n;
  double s, c;
  sincospi(-2.0 * (double)m / (double)n, &s, &c);
  ff[i] = cmul(v, make_double2(c, s));
}

__global__ void extract_taps_kernel(const double2 *__restrict__ g, int w, int n, double2 *ft) {
  const int i = blockIdx.x * FT + threadIdx.x;
  if (i >= w) return;
  const double2 v = g[i];
  ft[i] = make_double2(v.x / n, v.y / n);
}

unsigned grid_of(long long count) { return (unsigned)((count + FT - 1) / FT); }

}  // namespace

int design_filter(const gsfft_params &p, double2 *d_ft, double2 *d_ff, cudaStream_t st) {
  const int n = p.n, w = p.w;
  if (w < 3 || w > n || (w & 1) == 0 || p.b_f < 1 || p.b_f > n) return GSFFT_ERR_PARAM;
  long long M = 256;
  while (M < 2LL * w - 1) M <<= 1;
  FftPlan fm, fn;
  double2 *win = nullptr, *a = nullptr, *b = nullptr, *g = nullptr, *ffb = nullptr;
  unsigned long long *mx = nullptr;
  int s = GSFFT_OK;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && s == GSFFT_OK) {
      set_last_error("design_filter: %s", cudaGetErrorString(e));
      s = GSFFT_ERR_CUDA;
    }
  };
  ck(cudaMalloc(&win, sizeof(double2) * w));
  ck(cudaMalloc(&a, sizeof(double2) * M));
  ck(cudaMalloc(&b, sizeof(double2) * M));
  ck(cudaMalloc(&g, sizeof(double2) * (size_t)n));
  ck(cudaMalloc(&mx, sizeof(unsigned long long)));
  if (!d_ff) ck(cudaMalloc(&ffb, sizeof(double2) * (size_t)n));
  double2 *ff = d_ff ? d_ff : ffb;
  if (s == GSFFT_OK) s = fft_plan_init(fm, M, GSFFT_FP64, 1);
  if (s == GSFFT_OK) s = fft_plan_init(fn, n, GSFFT_FP64, 1);
  FftIo io;
  if (s == GSFFT_OK) {
    cheb_window_kernel<<<grid_of(w), FT, 0, st>>>(win, w, p.t0, p.tolerance);
    ck(cudaGetLastError());
    bluestein_prep_kernel<<<grid_of(M), FT, 0, st>>>(win, w, M, a, b);
    ck(cudaGetLastError());
  }
  if (s == GSFFT_OK) s = fft_exec(fm, a, a, 1, -1, io, st);
  if (s == GSFFT_OK) s = fft_exec(fm, b, b, 1, -1, io, st);
  if (s == GSFFT_OK) {
    pointwise_mul_kernel<<<grid_of(M), FT, 0, st>>>(a, b, M);
    ck(cudaGetLastError());
  }
  if (s == GSFFT_OK) s = fft_exec(fm, a, a, 1, +1, io, st);
  if (s == GSFFT_OK) {
    bluestein_post_kernel<<<grid_of(w), FT, 0, st>>>(a, w, M, win);
    ck(cudaGetLastError());
    place_kernel<<<grid_of(n), FT, 0, st>>>(win, w, n, g);
    ck(cudaGetLastError());
  }
  if (s == GSFFT_OK) s = fft_exec(fn, g, g, 1, -1, io, st);
  if (s == GSFFT_OK) {
    ck(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st));
    boxcar_kernel<<<(unsigned)((n + BOX_TILE - 1) / BOX_TILE), FT, 0, st>>>(g, n, p.b_f, ff, mx);
    ck(cudaGetLastError());
    normalize_ramp_kernel<<<grid_of(n), FT, 0, st>>>(ff, n, w / 2, mx);
    ck(cudaGetLastError());
  }
  if (s == GSFFT_OK) s = fft_exec(fn, ff, g, 1, +1, io, st);
  if (s == GSFFT_OK) {
    extract_taps_kernel<<<grid_of(w), FT, 0, st>>>(g, w, n, d_ft);
    ck(cudaGetLastError());
    ck(cudaStreamSynchronize(st));
  }
  fft_plan_free(fm);
  fft_plan_free(fn);
  cudaFree(win);
  cudaFree(a);
  cudaFree(b);
  cudaFree(g);
  cudaFree(mx);
  if (ffb) cudaFree(ffb);
  return s;
}

}  // namespace gsfft
