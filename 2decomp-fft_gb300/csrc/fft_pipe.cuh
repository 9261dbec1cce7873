// Pipelined axis passes: a persistent CTA streams tiles of lines through D
// shared-memory buffers with asynchronous copies (cp.async), so that the
// loads of the next D - 1 tiles are in flight while it transforms the
// current one.
//
// The one-shot kernels (fft_fast.cuh) keep a CTA's loads in flight only
// during its own load phase; with two or three CTAs per SM, an SM's memory
// pipe sits idle whenever its CTAs are all exchanging or computing.  Here
// every SM always has a tile or two of loads outstanding:
//
//   prologue:  issue tiles 0 .. D-2 of this CTA
//   tile i:    issue tile i + D - 1 into buffer (i - 1) mod D
//              wait for tile i's copies, barrier
//              stages from shared memory (in place in buffer i mod D), the
//              last stage storing straight to global memory
//              barrier (the buffer may be refilled)
//
// A CTA takes tiles blockIdx.x, blockIdx.x + gridDim.x, ... so that the
// tiles in flight across the GPU form one contiguous window of the array.
// Copies are 8-byte (FP32 complex) or 16-byte (FP64 complex) cp.async into
// the padded layout of the stages (slot sidx); padding lines are not loaded
// and their results are not stored.
#pragma once

#include "fft_fast.cuh"

namespace gbfft {
namespace pipe {

using namespace dev;

template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

__device__ __forceinline__ int pad_slot(int a) { return a + (a >> 4); }

// Issue the copies of one tile: lines u0 .. u0 + L - 1 (complex lines, x
// positions on strided axes) at second index v.  lg = log2(L).
template <typename T, int KIND, bool CONTIG, int N>
__device__ __forceinline__ void issue_tile(const PassArgs& a, Cx<T>* S, long long u0, long long v, int L, int lg,
                                           int tid, int nthreads) {
  using C = Cx<T>;
  const long long nl = a.nlines;
  if constexpr (KIND == K_C2C) {
    const C* src = reinterpret_cast<const C*>(a.src);
    for (int e = tid; e < N * L; e += nthreads) {
      const int line = CONTIG ? e / N : (e & (L - 1));
      const int n = CONTIG ? (e & (N - 1)) : (e >> lg);
      const long long cl = u0 + line;
      if (cl >= nl) continue;
      const long long off = CONTIG ? cl * a.s_src_l + n : cl + v * a.s_src_l + (long long)n * a.s_src_n;
      cp_async<sizeof(C)>(S + pad_slot(CONTIG ? line * N + n : n * L + line), src + off);
    }
  } else if constexpr (KIND == K_R2C) {
    const T* src = reinterpret_cast<const T*>(a.src);
    const bool pv = !CONTIG && (a.pair_vec & 1);
    for (int e = tid; e < N * L; e += nthreads) {
      const int line = CONTIG ? e / N : (e & (L - 1));
      const int n = CONTIG ? (e & (N - 1)) : (e >> lg);
      const long long cl = u0 + line;
      if (cl >= nl) continue;
      const long long r0 = 2 * cl, r1 = r0 + 1;
      const bool has1 = r1 < a.real_lines;
      const long long o0 = CONTIG ? r0 * a.s_src_l + n : r0 + v * a.s_src_l + (long long)n * a.s_src_n;
      const long long o1 = CONTIG ? r1 * a.s_src_l + n : r1 + v * a.s_src_l + (long long)n * a.s_src_n;
      C* d = S + pad_slot(CONTIG ? line * N + n : n * L + line);
      if (pv && has1) {
        cp_async<sizeof(C)>(d, src + o0);
      } else {
        cp_async<sizeof(T)>(&d->x, src + o0);
        if (has1) cp_async<sizeof(T)>(&d->y, src + o1);
        else d->y = T(0);
      }
    }
  } else {
    // c2r: the two half spectra of each line pair, interleaved: X_hh[j] is
    // half hh of pair slot j (CONTIG: line (N/2+1) + j, strided: j L + line,
    // as LineCtx::sstage); on strided axes neighbouring lanes take the two
    // lines of a pair and then neighbouring pairs, i.e. consecutive x
    // positions
    const C* src = reinterpret_cast<const C*>(a.src);
    constexpr int H = N / 2 + 1;
    for (int e = tid; e < 2 * H * L; e += nthreads) {
      int line, hh, j;
      if (CONTIG) {
        line = e / (2 * H);
        const int r = e - line * (2 * H);
        hh = r >= H;
        j = r - hh * H;
      } else {
        const int p = e & (2 * L - 1);
        line = p >> 1;
        hh = p & 1;
        j = e >> (lg + 1);
      }
      const long long cl = u0 + line;
      if (cl >= nl) continue;
      const long long r = 2 * cl + hh;
      C* d = S + 2 * (CONTIG ? line * H + j : j * L + line) + hh;
      if (r < a.real_lines) {
        const long long off = CONTIG ? r * a.s_src_l + j : r + v * a.s_src_l + (long long)j * a.s_src_n;
        cp_async<sizeof(C)>(d, src + off);
      } else {
        d->x = T(0);
        d->y = T(0);
      }
    }
  }
}

template <typename T, int KIND, bool CONTIG, int N, int E, int D>
__global__ void __launch_bounds__(pipe_max_threads(E), 1)
    pipe_pass_kernel(const __grid_constant__ PassArgs a, long long tiles_u, long long total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using C = Cx<T>;
  const int L = a.L;
  const int lg = __ffs(L) - 1;
  const int entries = fast_smem_entries(N, L);
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int nthreads = blockDim.x * blockDim.y;
  const int t = CONTIG ? threadIdx.x : threadIdx.y;
  const int line = CONTIG ? threadIdx.y : threadIdx.x;
  const long long G = gridDim.x;
  const long long k0 = blockIdx.x;

  auto issue = [&](long long tile, int b) {
    const long long ub = CONTIG ? tile : tile % tiles_u;
    const long long v = CONTIG ? 0 : tile / tiles_u;
    issue_tile<T, KIND, CONTIG, N>(a, buf0 + (long long)b * entries, ub * L, v, L, lg, tid, nthreads);
  };

#pragma unroll
  for (int d = 0; d < D - 1; ++d) {
    const long long tile = k0 + d * G;
    if (tile < total) issue(tile, d);
    cp_commit();
  }
  int cur = 0;
  for (long long tile = k0; tile < total; tile += G) {
    const long long nt = tile + (D - 1) * G;
    if (nt < total) issue(nt, (cur + D - 1) % D);
    cp_commit();
    cp_wait<D - 1>();
    __syncthreads();
    C* Sm = buf0 + (long long)cur * entries;
    const long long ub = CONTIG ? tile : tile % tiles_u;
    const long long v = CONTIG ? 0 : tile / tiles_u;
    LineCtx<T, KIND, CONTIG> c;
    c.init_at(a, t, line, ub * L + line, v, a.nlines);
    C x[E];
    fast::run_stages<N, E, 0, LineCtx<T, KIND, CONTIG>, C, true>(c, Sm, x);
    if constexpr (KIND == K_R2C) c.store_r2c_pairs(Sm);
    __syncthreads();
    cur = (cur + 1) % D;
  }
  cp_wait<0>();
}

}  // namespace pipe
}  // namespace gbfft
