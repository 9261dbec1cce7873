// Instantiations of the power-of-two axis passes (fft_fast.cuh) for
// double, r2c and c2r lines.
#include "fft_fast.cuh"

namespace gbfft {

cudaError_t launch_fast_f64_real(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  if (kind == K_R2C)
    return contiguous ? fast::launch_pow2<double, K_R2C, true>(a, s) : fast::launch_pow2<double, K_R2C, false>(a, s);
  return contiguous ? fast::launch_pow2<double, K_C2R, true>(a, s) : fast::launch_pow2<double, K_C2R, false>(a, s);
}

}  // namespace gbfft
