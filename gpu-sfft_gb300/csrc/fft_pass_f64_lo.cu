// Instantiations of the FFT pass kernel: double, radix 2^5 .. 2^9.
#include "fft_pass.cuh"

namespace gsfft {

int fft_pass_f64_lo(int logr, const PassArgs &a, long long total_sub, cudaStream_t st) {
  switch (logr) {
    case 5: return launch_pass<double, 5>(a, total_sub, st);
    case 6: return launch_pass<double, 6>(a, total_sub, st);
    case 7: return launch_pass<double, 7>(a, total_sub, st);
    case 8: return launch_pass<double, 8>(a, total_sub, st);
    case 9: return launch_pass<double, 9>(a, total_sub, st);
    default: return GSFFT_ERR_UNSUPPORTED;
  }
}

}  // namespace gsfft
