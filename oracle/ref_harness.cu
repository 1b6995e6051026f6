// ref_harness.cu -- command-line driver around the reference implementation
// (pcdslab/gpu-sfft), built from the reference's own sources by
// oracle/build_ref.py into oracle/_ref/bin/ref_sfft.
//
// TEST INFRASTRUCTURE ONLY: the parity tests, the fixture script
// tests/golden/make_ref_fixtures.py and bench.py's reference-timing leg run
// it as a separate process; the product never links or calls it.
//
//   ref_sfft q k Bcst loops_loc loops_thresh loops_est RLFC_cst RLFC_loops
//            [--signal-seed S] [--snr-db D] [--outer-seed T] [--reps R]
//            [--dump DIR] [--candidate-bound N]
//   ref_sfft stage cutoff|rlfc|perm|vote|est DIR
//
// The stage form runs one of the reference's stage functions
// (innerLoop.h:32-50) on inputs read from DIR (see run_stage) and writes its
// outputs to DIR; it uses only inputs on which the reference's kernels are
// race-free, so that their outputs are fixed values to compare against.
//
// Runs the reference's experiment the way its main() does (experiment.c:48-95:
// parameters, then cudafft_experiment, cuExperiment.cu:64-137, which draws the
// signal, designs the filter with make_multiple_t and calls run_experiment).
// The harness sits at run_experiment's call of outer_loop
// (cuExperiment.cu:175-176):
//   * --dump DIR writes the signal, both filter arrays, the parameters and the
//     true locations that the reference hands to outer_loop;
//   * the reference's own outer_loop (outerLoop.cu:65-190, compiled under the
//     name ref_real_outer_loop) then runs R times; with --outer-seed T, glibc's
//     drand48 and random streams are seeded with T before each run (otherwise
//     the reference's unseeded streams simply continue); each run prints one
//     "REF_RUN r I_F ms" line and, with --dump, writes DIR/nodes_<r>.bin;
//   * the first run's result goes back to run_experiment, which prints the
//     reference's own report (MISSED counts, MSE*k).
//
// Safety limits, checked before any reference kernel runs:
//   * estimateValuesKernel (innerLoop.cu:825-870) takes 2 x loops doubles per
//     candidate from the device heap with malloc and writes through the
//     pointers without a check.  The default 8 MiB heap runs out near 60k
//     candidates (the n = 2^27 configurations have ~76k).  The harness raises
//     the heap to 1 GiB before the first launch: MAXSIZE_HITS (524288)
//     candidates x 2 allocations x 1 KiB, far above 32 loops x 8 bytes.
//   * run_experiment is called with repetitions = 1 only, as the reference's
//     main does: its I_F accumulates over repetitions while outer_loop
//     reallocates d_I, so a second repetition would estimate uninitialised
//     d_I entries and index d_bins_f with them.  Repeated runs go through the
//     harness instead, which starts each one with I_F = 0.
//   * reverseHashKernel (innerLoop.cu:783-817) appends to d_I (MAXSIZE_HITS
//     entries) without a bound.  Unless B_thresh * n/B (the most candidates a
//     location loop can produce) is below MAXSIZE_HITS, the caller must pass
//     --candidate-bound N, an upper estimate it has measured with another
//     implementation on the same configuration, and N must stay below
//     MAXSIZE_HITS / 4.
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sfft_oracle.h"

extern "C" {
#include "utils.h"
#include "timer.h"
#include "experiment.h"
#include "outerLoop.h"
#include "innerLoop.h"
Node *ref_real_outer_loop(complex_t *d_x, int n, complex_t *d_filter_time,
                          complex_t *d_filter_freq, int d_filter_size, int B, int B_thresh,
                          int W_RLFC, int RLFC_loops, int loop_threshold, int loops_loc,
                          int loops, int *I_F, float t_H_to_D);
}

namespace {

struct Options {
  long signal_seed = -1;
  double snr_db = NAN;
  long outer_seed = -1;
  int reps = 1;
  std::string dump;
  long candidate_bound = -1;
  int k = 0;
  std::vector<int> true_loc;
};
Options g_opt;

void die(const char *msg) {
  fprintf(stderr, "ref_sfft: %s\n", msg);
  exit(2);
}

void write_file(const std::string &path, const void *data, size_t bytes) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) die(("cannot write " + path).c_str());
  if (bytes && fwrite(data, 1, bytes, f) != bytes) die(("short write " + path).c_str());
  fclose(f);
}

void dump_inputs(const complex_t *d_x, int n, const complex_t *d_ft, int w,
                 const complex_t *d_ff, int B, int B_thresh, int W, int R, int thresh,
                 int loops_loc, int loops) {
  std::vector<complex_t> h((size_t)n);
  if (cudaMemcpy(h.data(), d_x, sizeof(complex_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    die("copy of the signal failed");
  write_file(g_opt.dump + "/x.bin", h.data(), sizeof(complex_t) * n);
  if (cudaMemcpy(h.data(), d_ft, sizeof(complex_t) * w, cudaMemcpyDeviceToHost) != cudaSuccess)
    die("copy of the filter taps failed");
  write_file(g_opt.dump + "/ft.bin", h.data(), sizeof(complex_t) * w);
  if (cudaMemcpy(h.data(), d_ff, sizeof(complex_t) * n, cudaMemcpyDefault) != cudaSuccess)
    die("copy of the filter response failed");
  write_file(g_opt.dump + "/ff.bin", h.data(), sizeof(complex_t) * n);
  write_file(g_opt.dump + "/true_loc.bin", g_opt.true_loc.data(),
             sizeof(int) * g_opt.true_loc.size());
  FILE *f = fopen((g_opt.dump + "/params.txt").c_str(), "w");
  if (!f) die("cannot write params.txt");
  fprintf(f, "%d %d %d %d %d %d %d %d %d %d\n", n, w, B, B_thresh, W, R, thresh, loops_loc, loops,
          g_opt.k);
  fclose(f);
}

// ---- stage mode -----------------------------------------------------------
// ref_sfft stage KIND DIR runs one of the reference's stage functions
// (innerLoop.h:32-50) on inputs read from DIR and writes its outputs there.
// DIR/meta.txt holds "name value" lines; arrays are raw little-endian files.

struct Meta {
  std::vector<std::pair<std::string, long>> kv;
  long get(const char *name) const {
    for (const auto &p : kv)
      if (p.first == name) return p.second;
    die((std::string("meta.txt lacks ") + name).c_str());
    return 0;
  }
};

Meta read_meta(const std::string &dir) {
  Meta m;
  FILE *f = fopen((dir + "/meta.txt").c_str(), "r");
  if (!f) die("cannot read meta.txt");
  char name[128];
  long v;
  while (fscanf(f, "%127s %ld", name, &v) == 2) m.kv.emplace_back(name, v);
  fclose(f);
  return m;
}

template <typename T>
std::vector<T> read_array(const std::string &path, size_t count) {
  std::vector<T> v(count);
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) die(("cannot read " + path).c_str());
  if (count && fread(v.data(), sizeof(T), count, f) != count) die(("short read " + path).c_str());
  fclose(f);
  return v;
}

template <typename T>
T *to_device(const std::vector<T> &h, bool managed = false) {
  T *d = nullptr;
  const size_t bytes = sizeof(T) * (h.size() ? h.size() : 1);
  if ((managed ? cudaMallocManaged((void **)&d, bytes) : cudaMalloc((void **)&d, bytes)) !=
      cudaSuccess)
    die("device allocation failed");
  if (h.size() && cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyDefault) != cudaSuccess)
    die("copy to the device failed");
  return d;
}

template <typename T>
std::vector<T> to_host(const T *d, size_t count) {
  std::vector<T> h(count);
  if (count && cudaMemcpy(h.data(), d, sizeof(T) * count, cudaMemcpyDefault) != cudaSuccess)
    die("copy to the host failed");
  return h;
}

bool pow2(long v) { return v > 0 && (v & (v - 1)) == 0; }

int run_stage(const std::string &kind, const std::string &dir) {
  const Meta m = read_meta(dir);
  double t = 0.0;
  if (kind == "cutoff") {
    // samples_indices (innerLoop.cu:484-539) + cutoff (:551-616): the num
    // largest |v|^2 of `size` samples, ascending.  samplesKernel covers
    // size / 256 blocks only, so size must be a multiple of 256.
    const long size = m.get("size"), num = m.get("num");
    if (size < 256 || size % 256 || num < 1 || num + 1 > size) die("cutoff: bad sizes");
    auto v = read_array<complex_t>(dir + "/v.bin", size);
    complex_t *d_v = to_device(v);
    // the tie pass of cutoff() writes the output from the host: managed memory
    int *d_out = to_device(std::vector<int>(num, -1), true);
    samples_indices(d_v, (int)num, (int)size, d_out, &t);
    if (cudaDeviceSynchronize() != cudaSuccess) die("cutoff: CUDA error");
    auto out = to_host(d_out, num);
    write_file(dir + "/J.bin", out.data(), sizeof(int) * num);
  } else if (kind == "rlfc") {
    // restr_loc_freq_coeff (innerLoop.cu:112-177): one RLFC block of
    // B_thresh ids; glibc's drand48 is seeded with `seed` first.
    const long n = m.get("n"), W = m.get("W_RLFC"), Bt = m.get("B_thresh"), seed = m.get("seed");
    if (!pow2(n) || !pow2(W) || W < 256 || W >= n || Bt < 1 || Bt >= W) die("rlfc: bad sizes");
    auto x = read_array<complex_t>(dir + "/x.bin", n);
    complex_t *d_x = to_device(x);
    int *d_J2 = to_device(std::vector<int>(Bt, -1), true);
    srand48(seed);
    const int offset = (int)(unsigned)floor(drand48() * (double)(n / W));
    srand48(seed);
    restr_loc_freq_coeff(d_x, (int)n, (int)Bt, (int)W, d_J2, &t);
    if (cudaDeviceSynchronize() != cudaSuccess) die("rlfc: CUDA error");
    auto out = to_host(d_J2, Bt);
    write_file(dir + "/J2.bin", out.data(), sizeof(int) * Bt);
    write_file(dir + "/offset.bin", &offset, sizeof(int));
  } else if (kind == "perm") {
    // perm_filter_cutoff (innerLoop.cu:194-286) with n < 2^27 and w a
    // multiple of B: permFilterTillKernel then has no residue taps, so no
    // two threads update the same bin and the sums are deterministic.
    const long n = m.get("n"), w = m.get("w"), B = m.get("B"), Bt = m.get("B_thresh");
    const long a = m.get("a"), ai = m.get("ai");
    if (!pow2(n) || n >= (1L << 27) || !pow2(B) || B < 256 || w % B || w / B < 2 || w > n ||
        Bt < 1 || Bt >= B || a <= 0 || a >= n || ai <= 0 || ai >= n)
      die("perm: bad sizes");
    auto x = read_array<complex_t>(dir + "/x.bin", n);
    auto ft = read_array<complex_t>(dir + "/ft.bin", w);
    complex_t *d_x = to_device(x);
    complex_t *d_ft = to_device(ft);
    complex_t *d_bins = to_device(std::vector<complex_t>(B));
    int *d_J = to_device(std::vector<int>(Bt, -1), true);
    double pf = 0.0, bc = 0.0;
    perm_filter_cutoff(d_x, (int)n, d_ft, (int)w, (int)Bt, (int)B, (int)a, (int)ai, d_bins, d_J, &pf,
                       &bc);
    if (cudaDeviceSynchronize() != cudaSuccess) die("perm: CUDA error");
    auto bins = to_host(d_bins, B);
    auto J = to_host(d_J, Bt);
    write_file(dir + "/bins_f.bin", bins.data(), sizeof(complex_t) * B);
    write_file(dir + "/J.bin", J.data(), sizeof(int) * Bt);
  } else if (kind == "vote") {
    // reverse_hash (innerLoop.cu:300-384) for loops_loc location loops on one
    // zeroed vote table, as outer_loop runs them (outerLoop.cu:141-146).
    const long n = m.get("n"), B = m.get("B"), Bt = m.get("B_thresh"), W = m.get("W_RLFC");
    const long R = m.get("RLFC_loops"), thresh = m.get("loops_thresh"), L = m.get("loops_loc");
    const long nr = m.get("num_RLFC");
    if (!pow2(n) || !pow2(B) || !pow2(W) || B >= n || W >= n || W <= n / B || Bt < 1 || Bt >= B ||
        nr < 1 || nr > W || L < 1 || L > 32)
      die("vote: bad sizes");
    if (Bt * (n / B) * L >= MAXSIZE_HITS) die("vote: candidate count could reach MAXSIZE_HITS");
    auto J = read_array<int>(dir + "/J.bin", (size_t)(L * Bt));
    auto J2 = read_array<int>(dir + "/J2.bin", nr);
    auto av = read_array<int>(dir + "/a.bin", L);
    auto aiv = read_array<int>(dir + "/ai.bin", L);
    for (long i = 0; i < L * Bt; i++)
      if (J[i] < 0 || J[i] >= B) die("vote: J out of range");
    for (long i = 0; i < nr; i++)
      if (J2[i] < 0 || J2[i] >= W) die("vote: J2 out of range");
    int *d_vote = to_device(std::vector<int>(n, 0));
    int *d_I = to_device(std::vector<int>(MAXSIZE_HITS, -1));
    int *d_J2 = to_device(J2, true);
    int I_F = 0;
    for (long l = 0; l < L; l++) {
      std::vector<int> Jl(J.begin() + l * Bt, J.begin() + (l + 1) * Bt);
      int *d_J = to_device(Jl);
      reverse_hash(d_J, (int)n, (int)Bt, (int)B, av[l], aiv[l], (int)thresh, d_vote, d_I, &I_F, &t,
                   d_J2, (int)nr, (int)W, (int)R);
      cudaFree(d_J);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) die("vote: CUDA error");
    auto I = to_host(d_I, I_F);
    auto vote = to_host(d_vote, n);
    write_file(dir + "/I.bin", I.data(), sizeof(int) * I.size());
    write_file(dir + "/vote.bin", vote.data(), sizeof(int) * n);
  } else if (kind == "est") {
    // estimate_values (innerLoop.cu:396-466) for I_F candidates.
    const long n = m.get("n"), B = m.get("B"), loops = m.get("loops"), I_F = m.get("I_F");
    const long ll = m.get("loops_loc");
    if (!pow2(n) || !pow2(B) || B >= n || loops < 1 || loops > 32 || I_F < 1 ||
        I_F > MAXSIZE_HITS)
      die("est: bad sizes");
    auto I = read_array<int>(dir + "/I.bin", I_F);
    for (long i = 0; i < I_F; i++)
      if (I[i] < 0 || I[i] >= n) die("est: candidate out of range");
    auto bins = read_array<complex_t>(dir + "/bins_f.bin", (size_t)(loops * B));
    auto perm = read_array<int>(dir + "/permute.bin", loops);
    auto ff = read_array<complex_t>(dir + "/ff.bin", n);
    int *d_I = to_device(I);
    complex_t *d_bins = to_device(bins);
    complex_t *d_ff = to_device(ff, true);
    int count = (int)I_F;
    Node *nodes = estimate_values(d_I, &count, d_bins, (int)loops, (int)n, perm.data(), (int)B,
                                  d_ff, (int)ll);
    if (cudaDeviceSynchronize() != cudaSuccess || !nodes) die("est: CUDA error");
    write_file(dir + "/nodes.bin", nodes, sizeof(Node) * (size_t)I_F);
    free(nodes);
  } else {
    die(("unknown stage " + kind).c_str());
  }
  printf("REF_STAGE %s ok\n", kind.c_str());
  return 0;
}

int raise_heap() {
  // estimateValuesKernel's per-thread malloc: 1 GiB, see the header comment
  const size_t heap = (size_t)1 << 30;
  size_t cur = 0;
  if (cudaDeviceGetLimit(&cur, cudaLimitMallocHeapSize) != cudaSuccess) die("no CUDA device");
  if (cur < heap) {
    if (cudaDeviceSetLimit(cudaLimitMallocHeapSize, heap) != cudaSuccess)
      die("cannot raise the device heap");
    if (cudaDeviceGetLimit(&cur, cudaLimitMallocHeapSize) != cudaSuccess || cur < heap)
      die("device heap below 1 GiB");
  }
  return 0;
}

}  // namespace

// Called by run_experiment (cuExperiment.cu:175-176) in place of the
// reference's outer_loop; runs the real one as the options ask.
extern "C" Node *outer_loop(complex_t *d_x, int n, complex_t *d_filter_time,
                            complex_t *d_filter_freq, int d_filter_size, int B, int B_thresh,
                            int W_RLFC, int RLFC_loops, int loop_threshold, int loops_loc,
                            int loops, int *I_F, float t_H_to_D) {
  if (!g_opt.dump.empty())
    dump_inputs(d_x, n, d_filter_time, d_filter_size, d_filter_freq, B, B_thresh, W_RLFC,
                RLFC_loops, loop_threshold, loops_loc, loops);
  Node *first = nullptr;
  int first_count = 0;
  for (int r = 0; r < g_opt.reps; r++) {
    if (g_opt.outer_seed >= 0) {
      srand48(g_opt.outer_seed);
      srandom((unsigned)g_opt.outer_seed);
    }
    int count = 0;
    reset_timer();
    const auto t0 = std::chrono::steady_clock::now();
    Node *res = ref_real_outer_loop(d_x, n, d_filter_time, d_filter_freq, d_filter_size, B,
                                    B_thresh, W_RLFC, RLFC_loops, loop_threshold, loops_loc,
                                    loops, &count, t_H_to_D);
    const double ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    printf("REF_RUN %d %d %.4f\n", r, count, ms);
    fflush(stdout);
    if (!g_opt.dump.empty()) {
      std::vector<char> buf(sizeof(int) + sizeof(Node) * (size_t)count);
      memcpy(buf.data(), &count, sizeof(int));
      if (count) memcpy(buf.data() + sizeof(int), res, sizeof(Node) * (size_t)count);
      write_file(g_opt.dump + "/nodes_" + std::to_string(r) + ".bin", buf.data(), buf.size());
    }
    if (r == 0) {
      first = res;
      first_count = count;
    } else {
      free(res);
    }
  }
  *I_F += first_count;
  return first;
}

int main(int argc, char **argv) {
  if (argc >= 2 && std::string(argv[1]) == "stage") {
    if (argc != 4) die("usage: ref_sfft stage cutoff|rlfc|perm|vote|est DIR");
    raise_heap();
    return run_stage(argv[2], argv[3]);
  }
  if (argc < 9) die("usage: ref_sfft q k Bcst loops_loc loops_thresh loops_est RLFC_cst "
                    "RLFC_loops [--signal-seed S] [--snr-db D] [--outer-seed T] [--reps R] "
                    "[--dump DIR] [--candidate-bound N]");
  const int q = atoi(argv[1]);
  const int k = atoi(argv[2]);
  const double Bcst = strtod(argv[3], nullptr);
  const int loops_loc = atoi(argv[4]);
  const int loops_thresh = atoi(argv[5]);
  const int loops_est = atoi(argv[6]);
  const double RLFC_cst = atoi(argv[7]);  // experiment.c:64 parses it with atoi
  const int RLFC_loops = atoi(argv[8]);
  for (int i = 9; i < argc; i++) {
    const std::string a = argv[i];
    if (i + 1 >= argc) die(("missing value for " + a).c_str());
    const char *v = argv[++i];
    if (a == "--signal-seed") g_opt.signal_seed = atol(v);
    else if (a == "--snr-db") g_opt.snr_db = strtod(v, nullptr);
    else if (a == "--outer-seed") g_opt.outer_seed = atol(v);
    else if (a == "--reps") g_opt.reps = atoi(v);
    else if (a == "--dump") g_opt.dump = v;
    else if (a == "--candidate-bound") g_opt.candidate_bound = atol(v);
    else die(("unknown option " + a).c_str());
  }
  if (g_opt.reps < 1 || g_opt.reps > 100) die("--reps must be in 1..100");
  if (!g_opt.dump.empty() && g_opt.signal_seed < 0) die("--dump needs --signal-seed");

  // experiment.c:54-84 (tolerance 1e-8, experiment.c:67), restated by the oracle
  oc_params p;
  if (oc_derive_params(q, k, Bcst, loops_loc, loops_thresh, loops_est, RLFC_cst, RLFC_loops,
                       1.0e-8, &p) != OC_OK)
    die("parameters fail one of the reference's asserts");
  if (p.loops > 32) die("more than 32 loops");
  const long long max_cand = (long long)p.B_thresh * (p.n / p.B);
  if (max_cand >= MAXSIZE_HITS) {
    if (g_opt.candidate_bound < 0 || g_opt.candidate_bound >= MAXSIZE_HITS / 4)
      die("B_thresh * n/B reaches MAXSIZE_HITS: pass --candidate-bound below MAXSIZE_HITS/4");
  }
  g_opt.k = k;

  // device heap for estimateValuesKernel's per-thread malloc, before any launch
  raise_heap();

  // experiment.c:66-70: snr 1e12 and a zero noise factor; --snr-db turns the
  // reference's AWGN (utils.c:187-219) on with std = sqrt(k / (2 snr)).
  double std_noise = 0.0;
  if (!std::isnan(g_opt.snr_db)) std_noise = sqrt(k / (2.0 * pow(10.0, g_opt.snr_db / 10.0)));

  if (g_opt.signal_seed >= 0) {
    // the locations cudafft_experiment will draw (cuExperiment.cu:84-88)
    srand48(g_opt.signal_seed);
    g_opt.true_loc.resize(k);
    for (int i = 0; i < k; i++) g_opt.true_loc[i] = (int)(unsigned)floor(drand48() * p.n);
    srand48(g_opt.signal_seed);
  }
  VERBOSE = false;
  printf("REF_PARAMS n=%d k=%d B=%d B_thresh=%d W_RLFC=%d w=%d b_f=%d loops=%d\n", p.n, k, p.B,
         p.B_thresh, p.W_RLFC, p.w, p.b_f, p.loops);
  fflush(stdout);
  cudafft_experiment(p.n, p.lobefrac, p.tolerance, p.b_f, p.B, p.B_thresh, loops_loc,
                     loops_thresh, loops_est, p.W_RLFC, RLFC_loops, /*repetitions=*/1, k,
                     std_noise);
  fflush(stdout);
  return 0;
}
