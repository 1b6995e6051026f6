// Instantiations of the FFT pass kernel: float, radix 2^11 .. 2^14.
#include "fft_pass.cuh"

namespace gsfft {

int fft_pass_f32_hi(int logr, const PassArgs &a, long long total_sub, cudaStream_t st) {
  switch (logr) {
    case 11: return launch_pass<float, 11>(a, total_sub, st);
    case 12: return launch_pass<float, 12>(a, total_sub, st);
    case 13: return launch_pass<float, 13>(a, total_sub, st);
    case 14: return launch_pass<float, 14>(a, total_sub, st);
    default: return GSFFT_ERR_UNSUPPORTED;
  }
}

}  // namespace gsfft
