// Compile-time-planned axis passes for 7-smooth lengths that are not powers
// of two (the non-power-of-two grids: 384 x 400 x 243, 360 x 270 x 210, and
// the 48 / 96 / 192 lines of batched grids).
//
// Every such length splits as n = R0 * R1 with R0 <= R1 <= 32
// (mixed_r0 in gbfft_internal.h): two Stockham stages, one shared-memory
// exchange, TPL = R1 threads a line.
//   stage 0: radix R0, butterfly b = t (all TPL threads), points b + r R1,
//            read from global memory (or the staged c2r half spectra);
//   stage 1: radix R1 after NS = R0 points: threads t < R0 each own one
//            butterfly, twiddles W_n^{t r} from the stage-major table, and
//            write points t + r R0 to global memory.
// Radix butterflies other than 2, 3, 4, 5, 7, 8, 16, 32 are the composite
// ones of fft_common.cuh (dftg).
#pragma once

#include <type_traits>

#include "fft_fast.cuh"

namespace gbfft {
namespace mixed {

using namespace dev;

template <int N, class Ctx, class C>
__device__ __forceinline__ void run_mixed(const Ctx& c, C* Sm) {
  constexpr int R0 = mixed_r0(N), R1 = N / R0;
  constexpr int KIND = Ctx::kind;
  const int t = c.t;
  C v[R1];
  // stage 0: radix R0, butterfly b = t, points t + r R1
  if constexpr (KIND == K_C2R) {
    c.template stage_c2r<N, R1>(Sm);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R0; ++r) v[r] = c.sgather_c2r(Sm, t + r * R1);
    __syncthreads();
  } else {
#pragma unroll
    for (int r = 0; r < R0; ++r) v[r] = c.gload(t + r * R1);
  }
  dftg<R0>(v);
#pragma unroll
  for (int r = 0; r < R0; ++r) Sm[c.sidx(t * R0 + r)] = v[r];
  __syncthreads();
  // stage 1: radix R1 after NS = R0: butterflies b = t < R0, k = t
  const bool act = t < R0;
  if (act) {
#pragma unroll
    for (int r = 0; r < R1; ++r) v[r] = Sm[c.sidx(t + r * R0)];
#pragma unroll
    for (int r = 1; r < R1; ++r) v[r] = cmul(v[r], c.twiddle((R0 - 1) + (r - 1) * R0 + t));
    dftg<R1>(v);
  }
  if constexpr (KIND == K_R2C) {
    __syncthreads();
    if (act) {
#pragma unroll
      for (int r = 0; r < R1; ++r) c.put_r2c(Sm, t + r * R0, v[r]);
    }
    __syncthreads();
    c.store_r2c_pairs(Sm);
  } else {
    if (act) {
#pragma unroll
      for (int r = 0; r < R1; ++r) c.gstore(t + r * R0, v[r]);
    }
  }
}

template <typename T, int KIND, bool CONTIG, int N>
__global__ void __launch_bounds__(256) mixed_pass_kernel(const __grid_constant__ PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* Sm = reinterpret_cast<Cx<T>*>(smem_raw);
  chained_entry();
  LineCtx<T, KIND, CONTIG> c;
  c.init(a);
  run_mixed<N>(c, Sm);
}

template <typename T, int KIND, bool CONTIG, int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t stream) {
  constexpr int TPL = N / mixed_r0(N);
  const size_t smem = (size_t)fast_smem_entries(N, a.L) * sizeof(Cx<T>);
  auto kern = mixed_pass_kernel<T, KIND, CONTIG, N>;
  if (smem > 48 * 1024) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  const dim3 block = CONTIG ? dim3(TPL, a.L) : dim3(a.L, TPL);
  const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L), CONTIG ? 1u : (unsigned)a.nv);
  const cudaError_t err = launch_chained(kern, grid, block, smem, stream, a);
  add_launches(1);
  return err != cudaSuccess ? err : cudaGetLastError();
}

#define GBFFT_MIXED_CASES(T, KIND, CONTIG)                 \
  case 48: return launch_n<T, KIND, CONTIG, 48>(a, s);     \
  case 96: return launch_n<T, KIND, CONTIG, 96>(a, s);     \
  case 192: return launch_n<T, KIND, CONTIG, 192>(a, s);   \
  case 210: return launch_n<T, KIND, CONTIG, 210>(a, s);   \
  case 243: return launch_n<T, KIND, CONTIG, 243>(a, s);   \
  case 270: return launch_n<T, KIND, CONTIG, 270>(a, s);   \
  case 360: return launch_n<T, KIND, CONTIG, 360>(a, s);   \
  case 384: return launch_n<T, KIND, CONTIG, 384>(a, s);   \
  case 400: return launch_n<T, KIND, CONTIG, 400>(a, s);

template <typename T, int KIND, bool CONTIG>
cudaError_t launch(const PassArgs& a, cudaStream_t s) {
  switch (a.n) {
    GBFFT_MIXED_CASES(T, KIND, CONTIG)
    default: return cudaErrorNotSupported;
  }
}

}  // namespace mixed
}  // namespace gbfft
