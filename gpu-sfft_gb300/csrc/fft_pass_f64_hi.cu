// Instantiations of the FFT pass kernel: double, radix 2^10 .. 2^13.
#include "fft_pass.cuh"

namespace gsfft {

int fft_pass_f64_hi(int logr, const PassArgs &a, long long total_sub, cudaStream_t st) {
  switch (logr) {
    case 10: return launch_pass<double, 10>(a, total_sub, st);
    case 11: return launch_pass<double, 11>(a, total_sub, st);
    case 12: return launch_pass<double, 12>(a, total_sub, st);
    case 13: return launch_pass<double, 13>(a, total_sub, st);
    default: return GSFFT_ERR_UNSUPPORTED;
  }
}

}  // namespace gsfft
