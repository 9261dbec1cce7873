// Instantiations of the fused x/y plane kernel (fft_fused.cuh) for float:
// square power-of-two planes 256^2, 512^2 and 1024^2, in the four orders the
// 3D transforms use (c2c x then y, c2c y then x, r2c x then y, c2r y then x).
#include "fft_fused.cuh"

namespace gbfft {

namespace {

template <int N, int TH>
cudaError_t launch_nt(int kindx, bool x_first, const FusedArgs& f, cudaStream_t s) {
  if (kindx == K_C2C)
    return x_first ? fused::launch<float, K_C2C, true, N, N, TH>(f, s)
                   : fused::launch<float, K_C2C, false, N, N, TH>(f, s);
  if (kindx == K_R2C && x_first) return fused::launch<float, K_R2C, true, N, N, TH>(f, s);
  if (kindx == K_C2R && !x_first) return fused::launch<float, K_C2R, false, N, N, TH>(f, s);
  return cudaErrorNotSupported;
}

template <int N>
cudaError_t launch_n(int kindx, bool x_first, const FusedArgs& f, cudaStream_t s) {
  if (f.threads == 256) return launch_nt<N, 256>(kindx, x_first, f, s);
  if (f.threads == 512) return launch_nt<N, 512>(kindx, x_first, f, s);
  return cudaErrorInvalidValue;
}

bool size_ok(int nx, int ny) { return nx == ny && (nx == 256 || nx == 512 || nx == 1024); }

}  // namespace

bool fused_supported(int prec_bytes, int kindx, bool x_first, int nx, int ny) {
  if (prec_bytes != 4 || !size_ok(nx, ny)) return false;
  if (kindx == K_C2C) return true;
  if (kindx == K_R2C) return x_first;
  if (kindx == K_C2R) return !x_first;
  return false;
}

cudaError_t launch_fused(int prec_bytes, int kindx, bool x_first, const FusedArgs& f, cudaStream_t stream) {
  if (!fused_supported(prec_bytes, kindx, x_first, f.ax.n, f.ay.n)) return cudaErrorNotSupported;
  switch (f.ax.n) {
    case 256: return launch_n<256>(kindx, x_first, f, stream);
    case 512: return launch_n<512>(kindx, x_first, f, stream);
    case 1024: return launch_n<1024>(kindx, x_first, f, stream);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace gbfft
