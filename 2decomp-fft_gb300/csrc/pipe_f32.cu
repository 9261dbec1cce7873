// Pipelined (persistent, cp.async multi-buffered) FP32 axis passes of
// 256, 512 and 1024 points: instantiations and launcher.
#include "fft_pipe.cuh"

namespace gbfft {

namespace {

int g_sms = 0;

cudaError_t sm_count(int* out) {
  if (g_sms == 0) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  *out = g_sms;
  return cudaSuccess;
}

template <int KIND, bool CONTIG, int N, int E, int D>
cudaError_t launch_pe(const PassArgs& a, cudaStream_t stream) {
  constexpr int TPL = N / E;
  const int L = a.L;
  const size_t smem = (size_t)D * fast_smem_entries(N, L) * sizeof(float2);
  if (smem > kPipeSmemLimit || L * TPL > pipe_max_threads(E) || (L & (L - 1)) != 0)
    return cudaErrorInvalidValue;
  auto kern = pipe::pipe_pass_kernel<float, KIND, CONTIG, N, E, D>;
  // resident CTAs per SM for each tile height (power of two up to 64)
  static int per_sm[7] = {0, 0, 0, 0, 0, 0, 0};
  const int lg = __builtin_ctz((unsigned)L);
  if (lg > 6) return cudaErrorInvalidValue;
  if (per_sm[lg] == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPipeSmemLimit);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, L * TPL, smem);
    if (e != cudaSuccess) return e;
    per_sm[lg] = n > 0 ? n : 1;
  }
  int sms = 0;
  cudaError_t e = sm_count(&sms);
  if (e != cudaSuccess) return e;
  const long long tiles_u = (a.nlines + L - 1) / L;
  const long long total = CONTIG ? tiles_u : tiles_u * a.nv;
  if (total <= 0) return cudaSuccess;
  long long grid = (long long)per_sm[lg] * sms;
  if (grid > total) grid = total;
  const dim3 block = CONTIG ? dim3(TPL, L) : dim3(L, TPL);
  kern<<<(unsigned)grid, block, smem, stream>>>(a, tiles_u, total);
  add_launches(1);
  return cudaGetLastError();
}

template <int KIND, bool CONTIG, int N, int E>
cudaError_t launch_e(const PassArgs& a, cudaStream_t s) {
  return a.pipe == 3 ? launch_pe<KIND, CONTIG, N, E, 3>(a, s) : launch_pe<KIND, CONTIG, N, E, 2>(a, s);
}

template <int KIND, bool CONTIG, int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t s) {
  if constexpr (N == 512 || N == 1024) {
    if (a.tpl == N / 16) return launch_e<KIND, CONTIG, N, 16>(a, s);
    return launch_e<KIND, CONTIG, N, 32>(a, s);
  } else {
    return launch_e<KIND, CONTIG, N, fast_points(N, CONTIG)>(a, s);
  }
}

template <int KIND, bool CONTIG>
cudaError_t launch_k(const PassArgs& a, cudaStream_t s) {
  switch (a.n) {
    case 256: return launch_n<KIND, CONTIG, 256>(a, s);
    case 512: return launch_n<KIND, CONTIG, 512>(a, s);
    case 1024: return launch_n<KIND, CONTIG, 1024>(a, s);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace

bool pipe_length(int n) { return n == 256 || n == 512 || n == 1024; }

cudaError_t launch_pipe_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  if (kind == K_C2C) return contiguous ? launch_k<K_C2C, true>(a, s) : launch_k<K_C2C, false>(a, s);
  if (kind == K_R2C) return contiguous ? launch_k<K_R2C, true>(a, s) : launch_k<K_R2C, false>(a, s);
  return contiguous ? launch_k<K_C2R, true>(a, s) : launch_k<K_C2R, false>(a, s);
}

}  // namespace gbfft
