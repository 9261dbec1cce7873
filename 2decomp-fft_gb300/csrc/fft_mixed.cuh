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
// Radix butterflies other than 2, 3, 4, 5, 7, 8, 16, 32 are built at compile
// time as a two-level Cooley-Tukey split R = P * Q in registers, with the
// internal twiddles W_R^{n2 k1} evaluated by a constexpr sine/cosine (argument
// reduced exactly on the rational angle, Taylor series in double).
#pragma once

#include <type_traits>

#include "fft_fast.cuh"

namespace gbfft {
namespace mixed {

using namespace dev;

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double taylor_sin(double x) {
  double t = x, s = x;
  for (int k = 1; k < 14; ++k) {
    t *= -x * x / ((2.0 * k) * (2.0 * k + 1));
    s += t;
  }
  return s;
}
constexpr double taylor_cos(double x) {
  double t = 1, s = 1;
  for (int k = 1; k < 14; ++k) {
    t *= -x * x / ((2.0 * k - 1) * (2.0 * k));
    s += t;
  }
  return s;
}
struct SinCos {
  double s, c;
};
// sin and cos of 2 pi m / d: reduced to [0, pi/4] by exact rational steps
// (f -> 1 - f, 1/2 - f, 1/4 - f), then Taylor series.
constexpr SinCos sincos_2pi(long long m, long long d) {
  m %= d;
  if (m < 0) m += d;
  double ss = 1, sc = 1;
  bool swap = false;
  if (2 * m > d) {
    m = d - m;
    ss = -1;
  }
  if (4 * m > d) {
    m = d - 2 * m;
    d = 2 * d;
    sc = -sc;
  }
  if (8 * m > d) {
    m = d - 4 * m;
    d = 4 * d;
    swap = true;
  }
  const double x = kTwoPi * (double)m / (double)d;
  double s = taylor_sin(x), c = taylor_cos(x);
  if (swap) {
    const double t = s;
    s = c;
    c = t;
  }
  return {ss * s, sc * c};
}

template <int R, int M>
__device__ __forceinline__ constexpr double root_c() {
  constexpr SinCos v = sincos_2pi(M, R);
  return v.c;
}
template <int R, int M>
__device__ __forceinline__ constexpr double root_s() {
  constexpr SinCos v = sincos_2pi(M, R);
  return v.s;
}

template <int B, int E, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

constexpr bool special_radix(int r) {
  return r == 2 || r == 3 || r == 4 || r == 5 || r == 7 || r == 8 || r == 16 || r == 32;
}
constexpr int pick_p(int r) {
  for (int p : {16, 8, 4, 5, 3, 7, 2})
    if (r % p == 0 && r != p) return p;
  return r;
}

// Forward DFT of size R in registers, natural order in and out.
template <int R, typename C>
__device__ __forceinline__ void dftg(C* v) {
  if constexpr (R == 1) {
  } else if constexpr (special_radix(R)) {
    dftp<R>(v);
  } else {
    using T = decltype(C::x);
    constexpr int P = pick_p(R), Q = R / P;
    C a[R];
    // n = Q n1 + n2, k = k1 + P k2: DFT_P over n1, twiddle W_R^{n2 k1}
    static_for<0, Q>([&](auto I2) {
      constexpr int n2 = decltype(I2)::value;
      C t[P];
      static_for<0, P>([&](auto I1) {
        constexpr int n1 = decltype(I1)::value;
        t[n1] = v[Q * n1 + n2];
      });
      dftg<P>(t);
      static_for<0, P>([&](auto K1) {
        constexpr int k1 = decltype(K1)::value;
        constexpr int e = (n2 * k1) % R;
        if constexpr (e == 0)
          a[n2 * P + k1] = t[k1];
        else
          a[n2 * P + k1] = cmul(t[k1], cmk<C>(T(root_c<R, e>()), T(-root_s<R, e>())));
      });
    });
    // DFT_Q over n2 for each k1
    static_for<0, P>([&](auto K1) {
      constexpr int k1 = decltype(K1)::value;
      C u[Q];
      static_for<0, Q>([&](auto I2) {
        constexpr int n2 = decltype(I2)::value;
        u[n2] = a[n2 * P + k1];
      });
      dftg<Q>(u);
      static_for<0, Q>([&](auto K2) {
        constexpr int k2 = decltype(K2)::value;
        v[k1 + P * k2] = u[k2];
      });
    });
  }
}

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
  kern<<<grid, block, smem, stream>>>(a);
  add_launches(1);
  return cudaGetLastError();
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
