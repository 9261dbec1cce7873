// Compile-time-planned axis passes for power-of-two lengths 16..4096.
//
// Same job and addressing as the runtime-planned kernel (fft_axis.cu), laid
// out for throughput:
//  * each thread owns E = 16 points of its line in registers (TPL = n/16
//    threads per line); every stage is radix 16 except the last, which takes
//    the remaining factor 2, 4 or 8;
//  * stage 0 loads its 16 points straight from global memory -- all 16 loads
//    in flight per thread, consecutive threads on consecutive points (or, on
//    strided axes, consecutive x positions) -- and the last stage stores
//    straight to global memory in the same coalesced order;
//  * between stages the line is exchanged in place through one padded
//    shared-memory buffer (one pad slot every 32 points);
//  * every index, stride and twiddle exponent is a compile-time function of
//    the thread index, so no integer division is left in the loop body.
#pragma once

#include "fft_common.cuh"

namespace gbfft {
namespace fast {

using namespace dev;

constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

template <int N>
struct P2Plan {
  static constexpr int LOG = ilog2(N);
  static constexpr int NFULL = LOG / 4;
  static constexpr int REM = LOG % 4;
  static constexpr int NST = NFULL + (REM ? 1 : 0);
  static constexpr int E = 16;
  static constexpr int TPL = N / E;
  __host__ __device__ static constexpr int radix(int s) { return s < NFULL ? 16 : (1 << REM); }
  __host__ __device__ static constexpr int ns(int s) {
    int v = 1;
    for (int i = 0; i < s; ++i) v *= radix(i);
    return v;
  }
};

template <typename T, int KIND, bool CONTIG, int N, int S>
__device__ __forceinline__ void run_stages(const LineCtx<T, KIND, CONTIG>& c, Cx<T>* Sm,
                                           Cx<T> (&v)[16]) {
  using P = P2Plan<N>;
  if constexpr (S < P::NST) {
    constexpr int R = P::radix(S), NS = P::ns(S), MB = P::E / R, NB = N / R, TPL = P::TPL;
    constexpr bool FIRST = (S == 0), LAST = (S == P::NST - 1);
    constexpr int TSTRIDE = N / (NS * R);
    const int t = c.t;
    if constexpr (FIRST) {
#pragma unroll
      for (int m = 0; m < MB; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) v[m * R + r] = c.gload(t + m * TPL + r * NB);
    } else {
#pragma unroll
      for (int m = 0; m < MB; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) v[m * R + r] = Sm[c.sidx(t + m * TPL + r * NB)];
    }
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int b = t + m * TPL;
      const int k = b & (NS - 1);
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[m * R + r] = cmul(v[m * R + r], c.twiddle(k * r * TSTRIDE));
      }
      dftp<R>(&v[m * R]);
    }
    if constexpr (LAST && KIND != K_R2C) {
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        const int b = t + m * TPL;
        const int k = b & (NS - 1);
        const int base = (b - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) c.gstore(base + r * NS, v[m * R + r]);
      }
    } else {
      if constexpr (!FIRST) __syncthreads();
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        const int b = t + m * TPL;
        const int k = b & (NS - 1);
        const int base = (b - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) Sm[c.sidx(base + r * NS)] = v[m * R + r];
      }
      __syncthreads();
    }
    run_stages<T, KIND, CONTIG, N, S + 1>(c, Sm, v);
  }
}

template <typename T, int KIND, bool CONTIG, int N>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256)
    fast_pass_kernel(const __grid_constant__ PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* Sm = reinterpret_cast<Cx<T>*>(smem_raw);
  LineCtx<T, KIND, CONTIG> c;
  c.init(a);
  Cx<T> v[16];
  run_stages<T, KIND, CONTIG, N, 0>(c, Sm, v);
  if constexpr (KIND == K_R2C) c.store_r2c(Sm);
}

template <typename T, int KIND, bool CONTIG, int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t stream) {
  const size_t e = (size_t)N * a.L;
  const size_t smem = (e + (e >> 5) + 1) * sizeof(Cx<T>);
  auto kern = fast_pass_kernel<T, KIND, CONTIG, N>;
  if (smem > 48 * 1024) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  const dim3 block = CONTIG ? dim3(P2Plan<N>::TPL, a.L) : dim3(a.L, P2Plan<N>::TPL);
  const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L), CONTIG ? 1u : (unsigned)a.nv);
  kern<<<grid, block, smem, stream>>>(a);
  add_launches(1);
  return cudaGetLastError();
}

template <typename T, int KIND, bool CONTIG>
cudaError_t launch_pow2(const PassArgs& a, cudaStream_t stream) {
  switch (a.n) {
    case 16: return launch_n<T, KIND, CONTIG, 16>(a, stream);
    case 32: return launch_n<T, KIND, CONTIG, 32>(a, stream);
    case 64: return launch_n<T, KIND, CONTIG, 64>(a, stream);
    case 128: return launch_n<T, KIND, CONTIG, 128>(a, stream);
    case 256: return launch_n<T, KIND, CONTIG, 256>(a, stream);
    case 512: return launch_n<T, KIND, CONTIG, 512>(a, stream);
    case 1024: return launch_n<T, KIND, CONTIG, 1024>(a, stream);
    case 2048: return launch_n<T, KIND, CONTIG, 2048>(a, stream);
    case 4096: return launch_n<T, KIND, CONTIG, 4096>(a, stream);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace fast
}  // namespace gbfft
