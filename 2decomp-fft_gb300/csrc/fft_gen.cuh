// Compile-time-planned axis passes for the non-power-of-two lengths 243,
// 270, 360, 384 and 400 with balanced three-stage (two-stage for 400) plans
// (GenPlan, fft_fast.cuh): every thread of a line owns E points in every
// stage, where the two-stage mixed-radix kernel (fft_mixed.cuh) leaves all
// but R0 of its R1 threads idle in its second stage (243 = 9 x 27: 9 of 27).
// Same structure as the power-of-two kernel: stage 0 from global memory (or
// the staged c2r half spectra), exchanges in place through one padded
// shared-memory buffer, the last stage to global memory (r2c: to the pair
// slots of the half-spectrum split).
#pragma once

#include "fft_fast.cuh"

namespace gbfft {
namespace gen {

using namespace dev;

template <int N> struct PlanOf;
template <> struct PlanOf<243> { using type = fast::GenPlan<243, 9, 9, 9, 3>; };
template <> struct PlanOf<270> { using type = fast::GenPlan<270, 30, 15, 6, 3>; };
template <> struct PlanOf<360> { using type = fast::GenPlan<360, 30, 10, 6, 6>; };
template <> struct PlanOf<384> { using type = fast::GenPlan<384, 24, 8, 8, 6>; };
template <> struct PlanOf<400> { using type = fast::GenPlan<400, 20, 20, 20>; };

template <typename T, int KIND, bool CONTIG, int N>
__global__ void __launch_bounds__(gen_max_threads(PlanOf<N>::type::E, sizeof(T)), 1)
    gen_pass_kernel(const __grid_constant__ PassArgs a) {
  using P = typename PlanOf<N>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* Sm = reinterpret_cast<Cx<T>*>(smem_raw);
  chained_entry();
  LineCtx<T, KIND, CONTIG> c;
  c.init(a);
  Cx<T> v[P::E];
  fast::run_plan<P, 0>(c, Sm, v);
  if constexpr (KIND == K_R2C) c.store_r2c_pairs(Sm);
}

template <typename T, int KIND, bool CONTIG, int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t stream) {
  using P = typename PlanOf<N>::type;
  if (a.tpl != P::TPL || a.L < 1 || a.L * P::TPL > gen_max_threads(P::E, (int)sizeof(T)))
    return cudaErrorInvalidValue;
  const size_t smem = (size_t)fast_smem_entries(N, a.L) * sizeof(Cx<T>);
  auto kern = gen_pass_kernel<T, KIND, CONTIG, N>;
  if (smem > 48 * 1024) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  const dim3 block = CONTIG ? dim3(P::TPL, a.L) : dim3(a.L, P::TPL);
  const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L), CONTIG ? 1u : (unsigned)a.nv);
  const cudaError_t err = launch_chained(kern, grid, block, smem, stream, a);
  add_launches(1);
  return err != cudaSuccess ? err : cudaGetLastError();
}

template <typename T, int KIND, bool CONTIG>
cudaError_t launch_k(const PassArgs& a, cudaStream_t s) {
  switch (a.n) {
    case 243: return launch_n<T, KIND, CONTIG, 243>(a, s);
    case 270: return launch_n<T, KIND, CONTIG, 270>(a, s);
    case 360: return launch_n<T, KIND, CONTIG, 360>(a, s);
    case 384: return launch_n<T, KIND, CONTIG, 384>(a, s);
    case 400: return launch_n<T, KIND, CONTIG, 400>(a, s);
    default: return cudaErrorNotSupported;
  }
}

template <typename T>
cudaError_t launch(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  if (kind == K_C2C) return contiguous ? launch_k<T, K_C2C, true>(a, s) : launch_k<T, K_C2C, false>(a, s);
  if (kind == K_R2C) return contiguous ? launch_k<T, K_R2C, true>(a, s) : launch_k<T, K_R2C, false>(a, s);
  return contiguous ? launch_k<T, K_C2R, true>(a, s) : launch_k<T, K_C2R, false>(a, s);
}

}  // namespace gen
}  // namespace gbfft
