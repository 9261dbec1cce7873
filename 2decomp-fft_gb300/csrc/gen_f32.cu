// Balanced-plan non-power-of-two passes (fft_gen.cuh), FP32.
#include "fft_gen.cuh"

namespace gbfft {
cudaError_t launch_gen_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  return gen::launch<float>(kind, contiguous, a, s);
}
}  // namespace gbfft
