// Real-to-real transforms (DCT-I..IV, DST-I..IV) along one axis, the 1D
// passes of decomp_2d_dtt_3d_r2r (src/fft_fftw3_f03.f90:1555-1656, where
// they are FFTW r2r plans).
//
// Every kind is a complex FFT of length M of an extension of the window:
//   DCT-I   M = 2(n-1): even extension x_0..x_{n-1}, x_{n-2}..x_1;  Y_k = Re F_k
//   DST-I   M = 2(n+1): odd extension 0, x_0..x_{n-1}, 0, -x_{n-1}..-x_0;
//                       Y_k = -Im F_{k+1}
//   DCT-II  M = 2n: x_0..x_{n-1}, x_{n-1}..x_0;  Y_k = Re(W^k F_k)
//   DCT-III M = 2n: c_j x_j W^j (c_0 = 1, else 2), zero padded;  Y_k = Re F_k
//   DCT-IV  M = 2n: x_j W^j, zero padded;  Y_k = 2 Re(e^{-i pi/(4n)} W^k F_k)
// with W = exp(-2 pi i / (4n)), and the sine kinds from the cosine ones:
//   DST-II(x)_k  = DCT-II((-1)^j x_j)_{n-1-k}
//   DST-III(x)_k = (-1)^k DCT-III(x_{n-1-j})_k
//   DST-IV(x)_k  = (-1)^k DCT-IV(x_{n-1-j})_k
// A CTA owns L lines.  Each line's extension is built in shared memory
// straight from the real window, transformed by the runtime-planned Stockham
// stages (fft_pp.cuh) and reduced to the n real outputs, which go back to the
// window's positions; with src != dst the points outside the window are
// copied through.
#include "fft_common.cuh"
#include "fft_fast.cuh"
#include "fft_pp.cuh"
#include "gbfft_internal.h"

namespace gbfft {

namespace {

using namespace dev;

// Point m of the length-M extension of the window (x(j): window point j).
template <typename C, class XF>
__device__ __forceinline__ C extension(int kind, int m, int n, int M, const XF& X, const C* w4) {
  using T = decltype(C::x);
  C z = cmk<C>(T(0), T(0));
  switch (kind) {
    case 1:
      z.x = X(m < n ? m : M - m);
      break;
    case 5:
      if (m != 0 && m != n + 1) z.x = m <= n ? X(m - 1) : -X(M - m - 1);
      break;
    case 2:
    case 6: {
      const int j = m < n ? m : 2 * n - 1 - m;
      z.x = (kind == 6 && (j & 1)) ? -X(j) : X(j);
      break;
    }
    case 3:
    case 7:
    case 4:
    case 8:
      if (m < n) {
        const T x = (kind == 3 || kind == 4) ? X(m) : X(n - 1 - m);
        const T s = ((kind == 3 || kind == 7) && m > 0) ? T(2) : T(1);
        const C w = w4[m];
        z = cmk<C>(s * x * w.x, s * x * w.y);
      }
      break;
    default:
      break;
  }
  return z;
}

// Output k of the transform from the FFT F of the extension (F(i): point i).
template <typename C, class FF>
__device__ __forceinline__ decltype(C::x) output(int kind, int k, int n, const FF& F, const C* w4, C c0) {
  using T = decltype(C::x);
  T y;
  switch (kind) {
    case 1:
      y = F(k).x;
      break;
    case 5:
      y = -F(k + 1).y;
      break;
    case 2:
    case 6: {
      const int kk = kind == 2 ? k : n - 1 - k;
      const C f = F(kk), w = w4[kk];
      y = w.x * f.x - w.y * f.y;
      break;
    }
    case 3:
    case 7:
      y = F(k).x;
      if (kind == 7 && (k & 1)) y = -y;
      break;
    default: {  // 4, 8
      const C f = F(k), w = cmul(c0, w4[k]);
      y = T(2) * (w.x * f.x - w.y * f.y);
      if (kind == 8 && (k & 1)) y = -y;
      break;
    }
  }
  return y;
}

// The length-M line's context: shared-memory layout of LineCtx, twiddles
// from a copy of the table in shared memory.
template <typename T, bool CONTIG>
struct DttCtx : LineCtx<T, K_C2C, CONTIG> {
  const Cx<T>* stw;
  __device__ __forceinline__ Cx<T> twiddle(int e) const { return stw[e]; }
};

template <typename T, bool CONTIG>
__global__ void __launch_bounds__(kMaxThreads) dtt_pass_kernel(const __grid_constant__ DttArgs a) {
  using C = Cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int t, line;
  long long u, v;
  if (CONTIG) {
    t = threadIdx.x;
    line = threadIdx.y;
    u = (long long)blockIdx.x * a.L + line;
    v = 0;
  } else {
    line = threadIdx.x;
    t = threadIdx.y;
    u = (long long)blockIdx.x * a.L + line;
    v = blockIdx.y;
  }
  const bool valid = u < a.nlines;
  const long long base = CONTIG ? u * a.sl : u + v * a.sl;
  const T* src = reinterpret_cast<const T*>(a.src);
  T* dst = reinterpret_cast<T*>(a.dst);
  const int n = a.n, M = a.M, kind = a.kind, tpl = a.tpl;
  const C* w4 = reinterpret_cast<const C*>(a.w4);

  DttCtx<T, CONTIG> c;  // shared-memory layout and twiddles of the length-M line
  c.tw = reinterpret_cast<const C*>(a.tw);
  c.N = M;
  c.L = a.L;
  c.t = t;
  c.tpl = tpl;
  c.line = line;
  const size_t e = (size_t)M * a.L;
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + (e + (e >> 4) + 1);
  C* stw = buf1 + (e + (e >> 4) + 1);  // the M twiddles
  c.stw = stw;
  {
    const int nthreads = blockDim.x * blockDim.y, tid = threadIdx.x + threadIdx.y * blockDim.x;
    for (int m = tid; m < M; m += nthreads) stw[m] = c.tw[m];
  }

  auto X = [&](int j) -> T { return valid ? src[base + (long long)(a.off + j) * a.sn] : T(0); };

  // the extension of the window, natural order
#pragma unroll 1
  for (int m = t; m < M; m += tpl) buf0[c.sidx(m)] = extension<C>(kind, m, n, M, X, w4);
  __syncthreads();

  C* A = buf0;
  C* B = buf1;
  int Ns = 1;
#pragma unroll 1
  for (int s = 0; s < a.nst; ++s) {
    const int R = a.radix[s];
    using Ctx = DttCtx<T, CONTIG>;
    if (R == 16) stage_pp<T, K_C2C, CONTIG, 16, Ctx>(c, A, B, Ns);
    else if (R == 8) stage_pp<T, K_C2C, CONTIG, 8, Ctx>(c, A, B, Ns);
    else if (R == 4) stage_pp<T, K_C2C, CONTIG, 4, Ctx>(c, A, B, Ns);
    else if (R == 2) stage_pp<T, K_C2C, CONTIG, 2, Ctx>(c, A, B, Ns);
    else if (R == 3) stage_pp<T, K_C2C, CONTIG, 3, Ctx>(c, A, B, Ns);
    else if (R == 5) stage_pp<T, K_C2C, CONTIG, 5, Ctx>(c, A, B, Ns);
    else if (R == 7) stage_pp<T, K_C2C, CONTIG, 7, Ctx>(c, A, B, Ns);
    else if (R == 11) stage_pp<T, K_C2C, CONTIG, 11, Ctx>(c, A, B, Ns);
    else if (R == 13) stage_pp<T, K_C2C, CONTIG, 13, Ctx>(c, A, B, Ns);
    else if (R == 17) stage_pp<T, K_C2C, CONTIG, 17, Ctx>(c, A, B, Ns);
    else if (R == 19) stage_pp<T, K_C2C, CONTIG, 19, Ctx>(c, A, B, Ns);
    else if (R == 23) stage_pp<T, K_C2C, CONTIG, 23, Ctx>(c, A, B, Ns);
    else if (sizeof(T) == 4 && (R == 29 || R == 31)) {
      // in FP64 a butterfly of 29 or 31 points does not fit the registers
      if constexpr (sizeof(T) == 4) {
        if (R == 29) stage_pp<T, K_C2C, CONTIG, 29, Ctx>(c, A, B, Ns);
        else stage_pp<T, K_C2C, CONTIG, 31, Ctx>(c, A, B, Ns);
      }
    } else {
      stage_pp_generic<T, K_C2C, CONTIG, Ctx>(c, A, B, R, Ns);
    }
    __syncthreads();
    C* tmp = A;
    A = B;
    B = tmp;
    Ns *= R;
  }

  if (!valid) return;
  const C c0 = cmk<C>(T(a.c0x), T(a.c0y));
#pragma unroll 1
  for (int k = t; k < n; k += tpl)
    dst[base + (long long)(a.off + k) * a.sn] = output<C>(kind, k, n, [&](int i) { return A[c.sidx(i)]; }, w4, c0);
  if (a.src != a.dst) {
#pragma unroll 1
    for (int j = t; j < a.naxis; j += tpl)
      if (j < a.off || j >= a.off + n) dst[base + (long long)j * a.sn] = src[base + (long long)j * a.sn];
  }
}

// Power-of-two extension length: the extension is transformed by the
// compile-time 16-point plan (fft_fast.cuh), reading it from and leaving its
// transform in one padded shared buffer.
template <typename T, bool CONTIG, int M>
__global__ void __launch_bounds__(fast_max_threads(16, sizeof(T)), 1)
    dtt_fast_kernel(const __grid_constant__ DttArgs a) {
  using C = Cx<T>;
  using P = fast::P2Plan<M, 16>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* Sm = reinterpret_cast<C*>(smem_raw);
  int t, line;
  long long u, v;
  if (CONTIG) {
    t = threadIdx.x;
    line = threadIdx.y;
    u = (long long)blockIdx.x * a.L + line;
    v = 0;
  } else {
    line = threadIdx.x;
    t = threadIdx.y;
    u = (long long)blockIdx.x * a.L + line;
    v = blockIdx.y;
  }
  const bool valid = u < a.nlines;
  const long long base = CONTIG ? u * a.sl : u + v * a.sl;
  const T* src = reinterpret_cast<const T*>(a.src);
  T* dst = reinterpret_cast<T*>(a.dst);
  const int n = a.n, kind = a.kind;
  const C* w4 = reinterpret_cast<const C*>(a.w4);
  LineCtx<T, K_C2C, CONTIG> c;
  c.tw = reinterpret_cast<const C*>(a.twf);
  c.N = M;
  c.L = a.L;
  c.t = t;
  c.tpl = P::TPL;
  c.line = line;
  c.inverse = false;
  auto X = [&](int j) -> T { return valid ? src[base + (long long)(a.off + j) * a.sn] : T(0); };
#pragma unroll 1
  for (int m = t; m < M; m += P::TPL) Sm[c.sidx(m)] = extension<C>(kind, m, n, M, X, w4);
  __syncthreads();
  C x[16];
  fast::run_plan<P, 0, LineCtx<T, K_C2C, CONTIG>, C, true, true>(c, Sm, x);
  if (!valid) return;
  const C c0 = cmk<C>(T(a.c0x), T(a.c0y));
#pragma unroll 1
  for (int k = t; k < n; k += P::TPL)
    dst[base + (long long)(a.off + k) * a.sn] = output<C>(kind, k, n, [&](int i) { return Sm[c.sidx(i)]; }, w4, c0);
  if (a.src != a.dst) {
#pragma unroll 1
    for (int j = t; j < a.naxis; j += P::TPL)
      if (j < a.off || j >= a.off + n) dst[base + (long long)j * a.sn] = src[base + (long long)j * a.sn];
  }
}

// Extension length M = R0 * R1 (dtt_mixed_length): the two-stage plan of the
// mixed-radix passes (fft_mixed.cuh) on the extension in one padded shared
// buffer.  R1 threads a line: stage 0 radix R0 (butterfly t, points t + r R1),
// stage 1 radix R1 (threads t < R0, points t + r R0, twiddles from the
// stage-major table a.twf), in place.
template <typename T, bool CONTIG, int M>
__global__ void __launch_bounds__(256) dtt_mixed_kernel(const __grid_constant__ DttArgs a) {
  using C = Cx<T>;
  constexpr int R0 = mixed_r0(M), R1 = M / R0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* Sm = reinterpret_cast<C*>(smem_raw);
  int t, line;
  long long u, v;
  if (CONTIG) {
    t = threadIdx.x;
    line = threadIdx.y;
    u = (long long)blockIdx.x * a.L + line;
    v = 0;
  } else {
    line = threadIdx.x;
    t = threadIdx.y;
    u = (long long)blockIdx.x * a.L + line;
    v = blockIdx.y;
  }
  const bool valid = u < a.nlines;
  const long long base = CONTIG ? u * a.sl : u + v * a.sl;
  const T* src = reinterpret_cast<const T*>(a.src);
  T* dst = reinterpret_cast<T*>(a.dst);
  const int n = a.n, kind = a.kind;
  const C* w4 = reinterpret_cast<const C*>(a.w4);
  const C* tw = reinterpret_cast<const C*>(a.twf);
  LineCtx<T, K_C2C, CONTIG> c;
  c.N = M;
  c.L = a.L;
  c.t = t;
  c.tpl = R1;
  c.line = line;
  auto X = [&](int j) -> T { return valid ? src[base + (long long)(a.off + j) * a.sn] : T(0); };
#pragma unroll 1
  for (int m = t; m < M; m += R1) Sm[c.sidx(m)] = extension<C>(kind, m, n, M, X, w4);
  __syncthreads();
  C x[R1];
  // stage 0: radix R0, butterfly t, points t + r R1
#pragma unroll
  for (int r = 0; r < R0; ++r) x[r] = Sm[c.sidx(t + r * R1)];
  dftg<R0>(x);
  __syncthreads();  // every point read before the stage's outputs overwrite them
#pragma unroll
  for (int r = 0; r < R0; ++r) Sm[c.sidx(t * R0 + r)] = x[r];
  __syncthreads();
  // stage 1: radix R1 after R0 points, butterflies t < R0, in place
  if (t < R0) {
#pragma unroll
    for (int r = 0; r < R1; ++r) x[r] = Sm[c.sidx(t + r * R0)];
#pragma unroll
    for (int r = 1; r < R1; ++r) x[r] = cmul(x[r], tw[(R0 - 1) + (r - 1) * R0 + t]);
    dftg<R1>(x);
#pragma unroll
    for (int r = 0; r < R1; ++r) Sm[c.sidx(t + r * R0)] = x[r];
  }
  __syncthreads();
  if (!valid) return;
  const C c0 = cmk<C>(T(a.c0x), T(a.c0y));
#pragma unroll 1
  for (int k = t; k < n; k += R1)
    dst[base + (long long)(a.off + k) * a.sn] = output<C>(kind, k, n, [&](int i) { return Sm[c.sidx(i)]; }, w4, c0);
  if (a.src != a.dst) {
#pragma unroll 1
    for (int j = t; j < a.naxis; j += R1)
      if (j < a.off || j >= a.off + n) dst[base + (long long)j * a.sn] = src[base + (long long)j * a.sn];
  }
}

template <typename T, bool CONTIG, int M>
cudaError_t launch_mixed_m(const DttArgs& a, cudaStream_t stream) {
  constexpr int TPL = M / mixed_r0(M);
  if (a.tpl != TPL || a.L * TPL > 256) return cudaErrorInvalidValue;
  const size_t smem = (size_t)fast_smem_entries(M, a.L) * sizeof(Cx<T>);
  auto kern = dtt_mixed_kernel<T, CONTIG, M>;
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

template <typename T, bool CONTIG>
cudaError_t launch_mixed(const DttArgs& a, cudaStream_t s) {
  switch (a.M) {
    case 126: return launch_mixed_m<T, CONTIG, 126>(a, s);
    case 510: return launch_mixed_m<T, CONTIG, 510>(a, s);
    default: return cudaErrorNotSupported;
  }
}

template <typename T, bool CONTIG, int M>
cudaError_t launch_fast_m(const DttArgs& a, cudaStream_t stream) {
  constexpr int TPL = M / 16;
  if (a.tpl != TPL || a.L * TPL > fast_max_threads(16, (int)sizeof(T))) return cudaErrorInvalidValue;
  const size_t smem = (size_t)fast_smem_entries(M, a.L) * sizeof(Cx<T>);
  auto kern = dtt_fast_kernel<T, CONTIG, M>;
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

template <typename T, bool CONTIG>
cudaError_t launch_fast(const DttArgs& a, cudaStream_t s) {
  switch (a.M) {
    case 32: return launch_fast_m<T, CONTIG, 32>(a, s);
    case 64: return launch_fast_m<T, CONTIG, 64>(a, s);
    case 128: return launch_fast_m<T, CONTIG, 128>(a, s);
    case 256: return launch_fast_m<T, CONTIG, 256>(a, s);
    case 512: return launch_fast_m<T, CONTIG, 512>(a, s);
    case 1024: return launch_fast_m<T, CONTIG, 1024>(a, s);
    case 2048: return launch_fast_m<T, CONTIG, 2048>(a, s);
    default: return cudaErrorNotSupported;
  }
}

template <typename T, bool CONTIG>
cudaError_t launch_t(const DttArgs& a, cudaStream_t stream) {
  const size_t smem = dtt_smem_bytes((int)sizeof(T), a.M, a.L);
  auto kern = dtt_pass_kernel<T, CONTIG>;
  if (smem > 48 * 1024) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  const dim3 block = CONTIG ? dim3(a.tpl, a.L) : dim3(a.L, a.tpl);
  const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L), CONTIG ? 1u : (unsigned)a.nv);
  kern<<<grid, block, smem, stream>>>(a);
  add_launches(1);
  return cudaGetLastError();
}

}  // namespace

size_t dtt_smem_bytes(int prec_bytes, int M, int L) {
  const size_t e = (size_t)M * (size_t)L;
  return (2 * (e + (e >> 4) + 1) + (size_t)M) * (size_t)(2 * prec_bytes);  // two line buffers, twiddles
}

namespace {
cudaError_t launch_dtt_one(int prec_bytes, bool contiguous, const DttArgs& a, cudaStream_t stream) {
  if (a.n < 1 || a.M < 2 || a.L < 1 || a.tpl < 1) return cudaErrorInvalidValue;
  if (a.twf && dtt_mixed_length(a.M)) {
    // FP32 only: the engine keeps FP64 on the runtime plan
    if (prec_bytes != 4) return cudaErrorInvalidValue;
    return contiguous ? launch_mixed<float, true>(a, stream) : launch_mixed<float, false>(a, stream);
  }
  if (a.twf) {
    if (!dtt_fast_length(a.M)) return cudaErrorInvalidValue;
    if (prec_bytes == 4) return contiguous ? launch_fast<float, true>(a, stream) : launch_fast<float, false>(a, stream);
    return contiguous ? launch_fast<double, true>(a, stream) : launch_fast<double, false>(a, stream);
  }
  if (a.L * a.tpl > kMaxThreads) return cudaErrorInvalidValue;
  if (prec_bytes == 4) return contiguous ? launch_t<float, true>(a, stream) : launch_t<float, false>(a, stream);
  return contiguous ? launch_t<double, true>(a, stream) : launch_t<double, false>(a, stream);
}
}  // namespace

// Strided passes with more planes than a grid's y extent allows run as
// several launches of at most kMaxGridY planes, the arrays offset by the
// planes already done (a line (u, v) starts at u + v * sl).
cudaError_t launch_dtt_pass(int prec_bytes, bool contiguous, const DttArgs& a, cudaStream_t stream) {
  if (contiguous || a.nv <= kMaxGridY) return launch_dtt_one(prec_bytes, contiguous, a, stream);
  for (long long v0 = 0; v0 < a.nv; v0 += kMaxGridY) {
    DttArgs b = a;
    b.nv = (int)(a.nv - v0 < kMaxGridY ? a.nv - v0 : kMaxGridY);
    b.src = static_cast<const char*>(a.src) + v0 * a.sl * prec_bytes;
    b.dst = static_cast<char*>(a.dst) + v0 * a.sl * prec_bytes;
    cudaError_t err = launch_dtt_one(prec_bytes, contiguous, b, stream);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

}  // namespace gbfft
