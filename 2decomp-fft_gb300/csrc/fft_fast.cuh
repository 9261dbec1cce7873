// Compile-time-planned axis passes for power-of-two lengths 16..4096.
//
// Same job and addressing as the runtime-planned kernel (fft_axis.cu), laid
// out for throughput:
//  * each thread owns E points of its line in registers (TPL = n/E threads
//    per line): 512 and 1024 run as two stages (32 x 16, 32 x 32) with
//    E = 32; the other lengths run radix 16 stages and a last stage of the
//    remaining factor 2, 4 or 8 with E = 16;
//  * stage 0 loads its 16 points straight from global memory -- all 16 loads
//    in flight per thread, consecutive threads on consecutive points (or, on
//    strided axes, consecutive x positions) -- and the last stage stores
//    straight to global memory in the same coalesced order;
//  * between stages the line is exchanged in place through one padded
//    shared-memory buffer (one pad slot every 16 points);
//  * twiddles come from a stage-major table (a.tw): stage s of radix R that
//    follows NS = R_0...R_{s-1} points finds W_{NS R}^{k r} at
//    (NS - 1) + (r - 1) NS + k, so the lanes of a warp read consecutive
//    entries; the stage offsets telescope and the table has n - 1 entries;
//  * every index, stride and twiddle exponent is a compile-time function of
//    the thread index, so no integer division is left in the loop body.
#pragma once

#include <cooperative_groups.h>

#include "fft_common.cuh"

namespace gbfft {
namespace fast {

using namespace dev;

template <int N_, int E_>
struct P2Plan {
  static constexpr int N = N_, E = E_;
  static constexpr int NST = fast_nst(N_, E_);
  static constexpr int TPL = N_ / E_;
  __host__ __device__ static constexpr int radix(int s) { return fast_radix(N_, E_, s); }
  __host__ __device__ static constexpr int ns(int s) {
    int v = 1;
    for (int i = 0; i < s; ++i) v *= radix(i);
    return v;
  }
};

// Barrier between stages: a line whose threads all sit in one warp
// (contiguous lines, at most 32 threads per line) only needs the warp.
template <bool WARP_LOCAL> __device__ __forceinline__ void stage_barrier() {
  if constexpr (WARP_LOCAL) __syncwarp();
  else __syncthreads();
}

// SMEM0: stage 0 reads its points from Sm (already filled by the caller:
// natural order for c2c / r2c, the staged half spectra for c2r) instead of
// global memory.
// A compile-time plan P (P2Plan, GenPlan): line length P::N, P::E points a
// thread, P::TPL threads a line, P::NST stages of radix P::radix(s) after
// P::ns(s) points; every radix divides E.  TO_SMEM: the last stage writes
// its outputs to Sm in natural order (slot sidx) and synchronises instead of
// storing them to global memory.
template <class P, int S, class Ctx, class C, bool SMEM0 = false, bool TO_SMEM = false>
__device__ __forceinline__ void run_plan(const Ctx& c, C* Sm, C (&v)[P::E]) {
  constexpr int N = P::N, E = P::E;
  constexpr int KIND = Ctx::kind;
  // warp-local barriers need every line inside one warp: TPL must divide 32
  constexpr bool WL = Ctx::contiguous && P::TPL <= 32 && 32 % P::TPL == 0;
  if constexpr (S < P::NST) {
    constexpr int R = P::radix(S), NS = P::ns(S), MB = E / R, NB = N / R, TPL = P::TPL;
    constexpr bool FIRST = (S == 0), LAST = (S == P::NST - 1);
    const int t = c.t;
    if constexpr (FIRST && KIND == K_C2R) {
      // half spectra staged in shared memory (each value read from global
      // memory once, coalesced), then the Hermitian gather
      if constexpr (!SMEM0) {
        c.template stage_c2r<N, TPL>(Sm);
        __syncthreads();
      }
#pragma unroll
      for (int m = 0; m < MB; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) v[m * R + r] = c.sgather_c2r(Sm, t + m * TPL + r * NB);
      __syncthreads();
    } else if constexpr (FIRST && SMEM0) {
#pragma unroll
      for (int m = 0; m < MB; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) v[m * R + r] = c.sload(Sm, t + m * TPL + r * NB);
      // all points of the tile are in registers before stage 0's outputs
      // overwrite the buffer
      __syncthreads();
    } else if constexpr (FIRST) {
#pragma unroll
      for (int m = 0; m < MB; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) v[m * R + r] = c.gload(t + m * TPL + r * NB);
    } else if constexpr (TPL % 16 == 0 && NB % 16 == 0) {
      // every point is t + 16 c: one slot computation, then constant steps
      const int s0 = c.sidx(t), st = c.sstep16();
#pragma unroll
      for (int m = 0; m < MB; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) v[m * R + r] = Sm[s0 + ((m * TPL + r * NB) / 16) * st];
    } else {
#pragma unroll
      for (int m = 0; m < MB; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) v[m * R + r] = Sm[c.sidx(t + m * TPL + r * NB)];
    }
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int b = t + m * TPL;
      const int k = b % NS;
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[m * R + r] = cmul(v[m * R + r], c.twiddle((NS - 1) + (r - 1) * NS + k));
      }
      dftg<R>(&v[m * R]);
    }
    if constexpr (LAST && KIND != K_R2C && !TO_SMEM) {
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        const int b = t + m * TPL;
        const int k = b % NS;
        const int base = (b - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) c.gstore(base + r * NS, v[m * R + r]);
      }
    } else {
      // r2c's last stage writes pair slots, which straddle the regions of
      // neighbouring lines: the whole CTA must be done reading
      if constexpr (!FIRST) {
        if constexpr (LAST && KIND == K_R2C) __syncthreads();
        else stage_barrier<WL>();
      }
      // (SMEM0: the first stage synchronised after its shared-memory reads)
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        const int b = t + m * TPL;
        const int k = b % NS;
        const int base = (b - k) * R + k;
        if constexpr (LAST && KIND == K_R2C) {
#pragma unroll
          for (int r = 0; r < R; ++r) c.put_r2c(Sm, base + r * NS, v[m * R + r]);
        } else if constexpr (NS % 16 == 0) {
          // points base + 16 (r NS / 16)
          const int s0 = c.sidx(base), st = c.sstep16();
#pragma unroll
          for (int r = 0; r < R; ++r) Sm[s0 + r * (NS / 16) * st] = v[m * R + r];
        } else if constexpr (NS == 1 && R % 16 == 0 && Ctx::contiguous) {
          // base = b R is a multiple of 16, and so is the line's first entry
          const int s0 = c.sidx(base);
#pragma unroll
          for (int r = 0; r < R; ++r) Sm[s0 + r + (r >> 4)] = v[m * R + r];
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) Sm[c.sidx(base + r * NS)] = v[m * R + r];
        }
      }
      // the r2c split after the last stage reads other lines' points
      if constexpr (LAST) __syncthreads();
      else stage_barrier<WL>();
    }
    run_plan<P, S + 1, Ctx, C, SMEM0, TO_SMEM>(c, Sm, v);
  }
}

template <int N, int E, int S, class Ctx, class C, bool SMEM0 = false>
__device__ __forceinline__ void run_stages(const Ctx& c, C* Sm, C (&v)[E]) {
  run_plan<P2Plan<N, E>, S, Ctx, C, SMEM0>(c, Sm, v);
}

// Plans for 7-smooth lengths that are not powers of two, chosen so that
// every radix divides E and all TPL threads of a line work in every stage:
// 243 = 9 9 3 (E 9), 270 = 15 6 3 (E 30), 360 = 10 6 6 (E 30),
// 384 = 8 8 6 (E 24), 400 = 20 20 (E 20).
template <int N_, int E_, int R0, int R1, int R2 = 1>
struct GenPlan {
  static constexpr int N = N_, E = E_, TPL = N_ / E_;
  static constexpr int NST = R2 > 1 ? 3 : 2;
  __host__ __device__ static constexpr int radix(int s) { return s == 0 ? R0 : (s == 1 ? R1 : R2); }
  __host__ __device__ static constexpr int ns(int s) { return s == 0 ? 1 : (s == 1 ? R0 : R0 * R1); }
  static_assert(R0 * R1 * R2 == N_ && E_ % R0 == 0 && E_ % R1 == 0 && E_ % R2 == 0, "bad plan");
};

// 16 points a thread, FP32: up to 1024 threads, i.e. at most 64 registers a
// thread, so a 512-thread strided tile still runs two CTAs per SM and a
// 1024-thread one (16 lines of 1024 points, 32 of 512: 128- and 256-byte
// row segments on strided axes) one.  32 points a thread: up to 512
// threads, at most 128 registers.
template <typename T, int KIND, bool CONTIG, int N, int E>
__global__ void __launch_bounds__(fast_max_threads(E, sizeof(T)), 1)
    fast_pass_kernel(const __grid_constant__ PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* Sm = reinterpret_cast<Cx<T>*>(smem_raw);
  chained_entry();
  // launched in clusters: start together, so that neighbouring CTAs' loads
  // of the same rows are in the DRAM queues at the same time
  if (a.csync) cooperative_groups::this_cluster().sync();
  // unpredicated padding-line loads
  LineCtx<T, KIND, CONTIG, false, false> c;
  c.init(a);
  // the block is (TPL, L) or (L, TPL): the compiler may fold the per-point
  // conditions of the c2r gather and the r2c split that depend on t.
  // Measured per kernel: faster on contiguous lines and strided 1024-point
  // lines, slower on strided 512-point lines (128 registers instead of 112,
  // z pass 0.76 -> 0.86 ms on 1024 x 1024 x 512) and 256-point ones.
  if constexpr (CONTIG || N == 1024) __builtin_assume(c.t >= 0 && c.t < N / E);
  Cx<T> v[E];
  run_stages<N, E, 0>(c, Sm, v);
  if constexpr (KIND == K_R2C) c.template store_r2c_pairs_ct<N, N / E>(Sm);
}

template <typename T, int KIND, bool CONTIG, int N, int E>
cudaError_t launch_ne(const PassArgs& a, cudaStream_t stream) {
  const size_t smem = (size_t)fast_smem_entries(N, a.L) * sizeof(Cx<T>);
  auto kern = fast_pass_kernel<T, KIND, CONTIG, N, E>;
  if (smem > 48 * 1024) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  constexpr int TPL = N / E;
  const dim3 block = CONTIG ? dim3(TPL, a.L) : dim3(a.L, TPL);
  const long long tiles = (a.nlines + a.L - 1) / a.L;
  if (a.csize > 1) {
    // grid.x padded to whole clusters; the padding CTAs own no line
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((tiles + a.csize - 1) / a.csize * a.csize), CONTIG ? 1u : (unsigned)a.nv, 1);
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)a.csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t err = cudaLaunchKernelEx(&cfg, kern, a);
    add_launches(1);
    return err != cudaSuccess ? err : cudaGetLastError();
  }
  if (a.csync) return cudaErrorInvalidValue;  // a cluster barrier needs a cluster launch
  const dim3 grid((unsigned)tiles, CONTIG ? 1u : (unsigned)a.nv);
  const cudaError_t err = launch_chained(kern, grid, block, smem, stream, a);
  add_launches(1);
  return err != cudaSuccess ? err : cudaGetLastError();
}

// Lines of 512 and 1024 points have two plans: 32 points a thread (two
// stages; the strided default; a contiguous line is then one warp) or 16
// (three stages; the contiguous default); a.tpl says which.
template <typename T, int KIND, bool CONTIG, int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t stream) {
  if constexpr (N == 512 || N == 1024) {
    if (a.tpl == N / 16) return launch_ne<T, KIND, CONTIG, N, 16>(a, stream);
    return launch_ne<T, KIND, CONTIG, N, 32>(a, stream);
  } else {
    // short lines: 4 or 8 points a thread when the engine chose them
    if constexpr (N <= 128)
      if (a.tpl == N / 4) return launch_ne<T, KIND, CONTIG, N, 4>(a, stream);
    if constexpr (N <= 256)
      if (a.tpl == N / 8) return launch_ne<T, KIND, CONTIG, N, 8>(a, stream);
    return launch_ne<T, KIND, CONTIG, N, fast_points(N, CONTIG)>(a, stream);
  }
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
