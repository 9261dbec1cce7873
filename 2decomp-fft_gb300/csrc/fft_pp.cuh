// Shared-memory ping-pong Stockham stages with a runtime radix, used by the
// runtime-planned axis kernel (fft_axis.cu) and the real-to-real kernel
// (dtt.cu).  The line sits in a padded shared buffer (LineCtx::sidx); the
// twiddles come from a full-length table exp(-2 pi i m / N) (LineCtx::tw).
#pragma once

#include "fft_common.cuh"

namespace gbfft {
namespace dev {

// One Stockham stage of radix R, shared buffer A -> B.  Butterfly b
// (0 <= b < n/R) reads points b + r n/R, multiplies by
// W_{Ns R}^{(b mod Ns) r}, transforms, and writes points
// (b - b mod Ns) R + b mod Ns + r Ns.  One butterfly in flight per thread.
// Ctx: a LineCtx (or a type derived from it that supplies its own twiddle()).
template <typename T, int KIND, bool CONTIG, int R, class Ctx = LineCtx<T, KIND, CONTIG>>
__device__ __forceinline__ void stage_pp(const Ctx& c, const Cx<T>* A, Cx<T>* B, int Ns) {
  using C = Cx<T>;
  const int nb = c.N / R;
  const int tstride = c.N / (Ns * R);
#pragma unroll 1
  for (int b = c.t; b < nb; b += c.tpl) {
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = A[c.sidx(b + r * nb)];
    const int k = b % Ns;
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], c.twiddle(k * r * tstride));
    }
    dftg<R>(v);
    const int base = (b - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) B[c.sidx(base + r * Ns)] = v[r];
  }
}

// A stage of any radix (primes above 7): each output point is a direct sum
// over its R inputs, O(n R) per line.
template <typename T, int KIND, bool CONTIG, class Ctx = LineCtx<T, KIND, CONTIG>>
__device__ void stage_pp_generic(const Ctx& c, const Cx<T>* A, Cx<T>* B, int R, int Ns) {
  using C = Cx<T>;
  const int N = c.N, nb = N / R, tstride = N / (Ns * R);
#pragma unroll 1
  for (int o = c.t; o < N; o += c.tpl) {
    const int k = o % Ns;
    const int r = (o / Ns) % R;
    const int q = o / (Ns * R);
    const int b = q * Ns + k;
    const int step = (k * tstride + r * nb) % N;
    C acc = cmk<C>(T(0), T(0));
    int e = 0;
#pragma unroll 1
    for (int j = 0; j < R; ++j) {
      const C x = A[c.sidx(b + j * nb)], w = c.twiddle(e);
      acc.x += x.x * w.x - x.y * w.y;
      acc.y += x.x * w.y + x.y * w.x;
      e += step;
      if (e >= N) e -= N;
    }
    B[c.sidx(o)] = acc;
  }
}

}  // namespace dev
}  // namespace gbfft
