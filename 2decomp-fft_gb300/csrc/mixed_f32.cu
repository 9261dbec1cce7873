// Instantiations of the mixed-radix axis passes (fft_mixed.cuh) for float.
#include "fft_mixed.cuh"

namespace gbfft {

cudaError_t launch_mixed_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  if (kind == K_C2C)
    return contiguous ? mixed::launch<float, K_C2C, true>(a, s) : mixed::launch<float, K_C2C, false>(a, s);
  if (kind == K_R2C)
    return contiguous ? mixed::launch<float, K_R2C, true>(a, s) : mixed::launch<float, K_R2C, false>(a, s);
  return contiguous ? mixed::launch<float, K_C2R, true>(a, s) : mixed::launch<float, K_C2R, false>(a, s);
}

}  // namespace gbfft
