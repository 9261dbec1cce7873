// Split-precision tensor-core axis passes (fft_split.cuh): the kernel and its
// instantiations for FP32 lines of 256, 512 and 1024 points.
#include "fft_split.cuh"

namespace gbfft {

namespace {

using namespace dev;
using split::kThreads;

template <int KIND, bool CONTIG, int N>
__global__ void __launch_bounds__(kThreads) split_pass_kernel(const __grid_constant__ PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int L = CONTIG ? 4 : 8;  // lines per CTA (split_lines_per_cta)
  constexpr int tpl = kThreads / L;
  float2* buf0 = reinterpret_cast<float2*>(smem_raw);
  float2* buf1 = buf0 + fast_smem_entries(N, L);
  const int tid = threadIdx.x;
  int t, line;
  if (CONTIG) {
    t = tid % tpl;
    line = tid / tpl;
  } else {
    line = tid % L;
    t = tid / L;
  }
  LineCtx<float, KIND, CONTIG> c;
  const long long cl = (long long)blockIdx.x * L + line;
  c.init_at(a, t, line, cl, CONTIG ? 0 : (long long)blockIdx.y, a.nlines);
  c.tpl = tpl;
  split::DftFrag F;
  split::dft16_frag(F, tid & 31);

  // load phase: line points in natural order into buf0
  if constexpr (KIND == K_C2R) {
    c.template stage_c2r<N, tpl>(buf1);
    __syncthreads();
    for (int n = t; n < N; n += tpl) buf0[c.sidx(n)] = c.sgather_c2r(buf1, n);
  } else {
    constexpr int B16 = 16;
    for (int i0 = t; i0 < N; i0 += B16 * tpl) {
      float2 r[B16];
#pragma unroll
      for (int j = 0; j < B16; ++j) {
        const int n = i0 + j * tpl;
        r[j] = n < N ? c.gload(n) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int j = 0; j < B16; ++j) {
        const int n = i0 + j * tpl;
        if (n < N) buf0[c.sidx(n)] = r[j];
      }
    }
  }
  __syncthreads();
  float2* A = buf0;
  float2* B = buf1;
  split::mma_stage16<N>(c, F, A, B, 1, L);
  __syncthreads();
  split::mma_stage16<N>(c, F, B, A, 16, L);
  __syncthreads();
  if constexpr (N == 512) {
    split::plain_stage<N, 2>(c, A, B, 256, L);
    __syncthreads();
    float2* tmp = A;
    A = B;
    B = tmp;
  } else if constexpr (N == 1024) {
    split::plain_stage<N, 4>(c, A, B, 256, L);
    __syncthreads();
    float2* tmp = A;
    A = B;
    B = tmp;
  }
  // store phase from A
  if constexpr (KIND == K_R2C) {
    c.store_r2c(A);
  } else {
    for (int n = t; n < N; n += tpl) c.gstore(n, A[c.sidx(n)]);
  }
}

template <int KIND, bool CONTIG, int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t stream) {
  const size_t smem = 2 * (size_t)fast_smem_entries(N, a.L) * sizeof(float2);
  auto kern = split_pass_kernel<KIND, CONTIG, N>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L), CONTIG ? 1u : (unsigned)a.nv);
  kern<<<grid, kThreads, smem, stream>>>(a);
  add_launches(1);
  return cudaGetLastError();
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

bool split_length(int n) { return n == 256 || n == 512 || n == 1024; }

int split_lines_per_cta(int n, bool contiguous) {
  (void)n;
  return contiguous ? 4 : 8;
}

cudaError_t launch_split_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  if (kind == K_C2C) return contiguous ? launch_k<K_C2C, true>(a, s) : launch_k<K_C2C, false>(a, s);
  if (kind == K_R2C) return contiguous ? launch_k<K_R2C, true>(a, s) : launch_k<K_R2C, false>(a, s);
  return contiguous ? launch_k<K_C2R, true>(a, s) : launch_k<K_C2R, false>(a, s);
}

}  // namespace gbfft
