// Instantiations of the FFT pass kernel: float, radix 2^5 .. 2^10.
#include "fft_pass.cuh"

namespace gsfft {

int fft_pass_f32_lo(int logr, const PassArgs &a, long long total_sub, cudaStream_t st) {
  switch (logr) {
    case 5: return launch_pass<float, 5>(a, total_sub, st);
    case 6: return launch_pass<float, 6>(a, total_sub, st);
    case 7: return launch_pass<float, 7>(a, total_sub, st);
    case 8: return launch_pass<float, 8>(a, total_sub, st);
    case 9: return launch_pass<float, 9>(a, total_sub, st);
    case 10: return launch_pass<float, 10>(a, total_sub, st);
    default: return GSFFT_ERR_UNSUPPORTED;
  }
}

}  // namespace gsfft
