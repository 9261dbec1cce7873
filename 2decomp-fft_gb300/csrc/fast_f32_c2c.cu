// Instantiations of the power-of-two axis passes (fft_fast.cuh) for
// float, complex-to-complex lines.
#include "fft_fast.cuh"

namespace gbfft {

cudaError_t launch_fast_f32_c2c(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  (void)kind;
  return contiguous ? fast::launch_pow2<float, K_C2C, true>(a, s) : fast::launch_pow2<float, K_C2C, false>(a, s);
}

}  // namespace gbfft
