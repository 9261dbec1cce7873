// Batched 1D FFT passes along one axis of an x-fastest 3D array, for sm_103a.
//
// This file replaces the 1D transforms of the reference backends -- the
// Glassman loops c2c_1m_{x,y,z} / r2c_1m_{x,z} / c2r_1m_{x,z} of
// src/fft_generic.f90:112-384 and the cuFFT plans of
// src/fft_cufft.f90:73-258 -- with one kernel family:
//
//  * A CTA owns L whole lines.  Each line is transformed by `tpl` threads
//    with a mixed-radix Stockham (self-sorting) FFT: every stage reads the
//    line at stride n/R, applies twiddles and a radix-R butterfly in
//    registers and writes it back in sorted order.  Between stages the line
//    sits in shared memory, padded by one slot every 32 to keep strided
//    accesses bank-conflict free.
//  * This file holds the runtime-planned kernel, which handles any length up
//    to kMaxN: lines are loaded into shared memory, each stage ping-pongs
//    between two shared buffers, and the result is stored from the last one.
//    Power-of-two lengths run the compile-time-planned kernels of
//    fft_fast.cu instead.
//  * Along y and z the lanes of a warp walk neighbouring x positions, so the
//    strided transforms still read and write contiguous x segments.
//  * r2c/c2r carry two real lines in one complex line (z = a + i b) and
//    separate / combine the two half spectra in the last / first stage, which
//    halves the FFT work and keeps the reference's c2r rule that the
//    imaginary parts of the DC and Nyquist bins are ignored
//    (src/fft_generic.f90:318-330: buf(i) = conjg(buf(d1+2-i)), real part).
//  * Backward transforms run as conj(F(conj(x))), so only forward butterflies
//    and one table of forward twiddles exp(-2 pi i m/n) exist.
#include <atomic>

#include "fft_common.cuh"
#include "fft_pp.cuh"
#include "gbfft_internal.h"

namespace gbfft {

namespace {

using namespace dev;

std::atomic<long long> g_launches{0};

// Runtime-planned pass: any length up to kMaxN, any factorisation.  The
// lines are loaded into shared buffer 0, each stage ping-pongs between the
// two buffers, and the result is stored from the last buffer written.
template <typename T, int KIND, bool CONTIG>
__global__ void __launch_bounds__(kMaxThreads)
    axis_pass_kernel(const __grid_constant__ PassArgs a) {
  using C = Cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  chained_entry();
  LineCtx<T, KIND, CONTIG> c;
  c.init(a);
  const size_t e = (size_t)a.n * a.L;
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + (e + (e >> 4) + 1);

#pragma unroll 1
  for (int n = c.t; n < c.N; n += c.tpl) buf0[c.sidx(n)] = c.gload(n);
  __syncthreads();

  C* A = buf0;
  C* B = buf1;
  int Ns = 1;
#pragma unroll 1
  for (int s = 0; s < a.nst; ++s) {
    const int R = a.radix[s];
    if (R == 16) stage_pp<T, KIND, CONTIG, 16>(c, A, B, Ns);
    else if (R == 8) stage_pp<T, KIND, CONTIG, 8>(c, A, B, Ns);
    else if (R == 4) stage_pp<T, KIND, CONTIG, 4>(c, A, B, Ns);
    else if (R == 2) stage_pp<T, KIND, CONTIG, 2>(c, A, B, Ns);
    else if (R == 3) stage_pp<T, KIND, CONTIG, 3>(c, A, B, Ns);
    else if (R == 5) stage_pp<T, KIND, CONTIG, 5>(c, A, B, Ns);
    else if (R == 7) stage_pp<T, KIND, CONTIG, 7>(c, A, B, Ns);
    else if (R == 11) stage_pp<T, KIND, CONTIG, 11>(c, A, B, Ns);
    else if (R == 13) stage_pp<T, KIND, CONTIG, 13>(c, A, B, Ns);
    else if (R == 17) stage_pp<T, KIND, CONTIG, 17>(c, A, B, Ns);
    else if (R == 19) stage_pp<T, KIND, CONTIG, 19>(c, A, B, Ns);
    else if (R == 23) stage_pp<T, KIND, CONTIG, 23>(c, A, B, Ns);
    else if (sizeof(T) == 4 && (R == 29 || R == 31)) {
      // in FP64 a butterfly of 29 or 31 points does not fit the registers
      if constexpr (sizeof(T) == 4) {
        if (R == 29) stage_pp<T, KIND, CONTIG, 29>(c, A, B, Ns);
        else stage_pp<T, KIND, CONTIG, 31>(c, A, B, Ns);
      }
    } else {
      stage_pp_generic<T, KIND, CONTIG>(c, A, B, R, Ns);
    }
    __syncthreads();
    C* tmp = A;
    A = B;
    B = tmp;
    Ns *= R;
  }

  if (KIND == K_R2C) {
    c.store_r2c(A);
  } else {
#pragma unroll 1
    for (int n = c.t; n < c.N; n += c.tpl) c.gstore(n, A[c.sidx(n)]);
  }
}

template <typename T, int KIND, bool CONTIG>
cudaError_t launch_typed(const PassArgs& a, cudaStream_t stream) {
  const size_t smem = pass_smem_bytes(sizeof(T), a.n, a.L);
  auto kern = axis_pass_kernel<T, KIND, CONTIG>;
  // the limit is a per-device attribute of the kernel: set it on every
  // launch that needs it (cheap), so a second device is covered too
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const dim3 block = CONTIG ? dim3(a.tpl, a.L) : dim3(a.L, a.tpl);
  const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L), CONTIG ? 1u : (unsigned)a.nv);
  const cudaError_t err = launch_chained(kern, grid, block, smem, stream, a);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return err != cudaSuccess ? err : cudaGetLastError();
}

// Identity copy, 16 bytes per access, 4 accesses in flight per thread.
__global__ void __launch_bounds__(256) copy16_kernel(const uint4* __restrict__ s, uint4* __restrict__ d,
                                                      size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    uint4 a0 = s[i], a1 = s[i + stride], a2 = s[i + 2 * stride], a3 = s[i + 3 * stride];
    d[i] = a0;
    d[i + stride] = a1;
    d[i + 2 * stride] = a2;
    d[i + 3 * stride] = a3;
  }
  for (; i < n; i += stride) d[i] = s[i];
}

__global__ void copy1_kernel(const unsigned char* __restrict__ s, unsigned char* __restrict__ d,
                             size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) d[i] = s[i];
}

int sm_count() {
  static std::atomic<int> cached{0};
  int v = cached.load();
  if (v) return v;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
  cached.store(v);
  return v;
}

}  // namespace

size_t pass_smem_bytes(int prec_bytes, int n, int L) {
  const size_t e = (size_t)n * (size_t)L;
  return 2 * (e + (e >> 4) + 1) * (size_t)(2 * prec_bytes);
}

namespace {
cudaError_t launch_axis_one(int prec_bytes, int kind, bool contiguous, const PassArgs& a, cudaStream_t stream) {
  if (a.tma) {
    if (!tma_pass_supported(prec_bytes, kind, contiguous, a)) return cudaErrorInvalidValue;
    return launch_tma_pass(a, stream);
  }
  if (a.fast == 5) {
    if (!tc_pass_supported(prec_bytes, kind, contiguous, a)) return cudaErrorInvalidValue;
    return launch_tc_pass(a, stream);
  }
  if (a.fast == 4) return prec_bytes == 4 ? launch_gen_f32(kind, contiguous, a, stream)
                                          : launch_gen_f64(kind, contiguous, a, stream);
  if (a.fast == 3) {
    if (prec_bytes != 4) return cudaErrorInvalidValue;
    return launch_split_f32(kind, contiguous, a, stream);
  }
  if (a.fast == 2) return prec_bytes == 4 ? launch_mixed_f32(kind, contiguous, a, stream)
                                          : launch_mixed_f64(kind, contiguous, a, stream);
  if (a.fast) {
    if (prec_bytes == 4)
      return kind == K_C2C ? launch_fast_f32_c2c(kind, contiguous, a, stream)
                           : launch_fast_f32_real(kind, contiguous, a, stream);
    return kind == K_C2C ? launch_fast_f64_c2c(kind, contiguous, a, stream)
                         : launch_fast_f64_real(kind, contiguous, a, stream);
  }
#define GB_DISPATCH(T)                                                              \
  switch (kind) {                                                                   \
    case K_C2C: return contiguous ? launch_typed<T, K_C2C, true>(a, stream)         \
                                  : launch_typed<T, K_C2C, false>(a, stream);       \
    case K_R2C: return contiguous ? launch_typed<T, K_R2C, true>(a, stream)         \
                                  : launch_typed<T, K_R2C, false>(a, stream);       \
    case K_C2R: return contiguous ? launch_typed<T, K_C2R, true>(a, stream)         \
                                  : launch_typed<T, K_C2R, false>(a, stream);       \
    default: return cudaErrorInvalidValue;                                          \
  }
  if (prec_bytes == 4) {
    GB_DISPATCH(float)
  } else if (prec_bytes == 8) {
    GB_DISPATCH(double)
  }
#undef GB_DISPATCH
  return cudaErrorInvalidValue;
}
}  // namespace

// Strided one-shot passes with more planes than a grid's y extent allows
// run as several launches of at most kMaxGridY planes, each side's array
// offset by the planes already done (a line (u, v) starts at u + v * s_l, in
// elements of that side's type).  The persistent bulk-copy pass walks any
// number of planes itself.
cudaError_t launch_axis_pass(int prec_bytes, int kind, bool contiguous, const PassArgs& a,
                             cudaStream_t stream) {
  if (contiguous || a.tma || a.fast == 5 || a.nv <= kMaxGridY)  // persistent kernels take any plane count
    return launch_axis_one(prec_bytes, kind, contiguous, a, stream);
  const size_t cs = 2 * (size_t)prec_bytes, rs = (size_t)prec_bytes;
  const size_t src_e = kind == K_R2C ? rs : cs, dst_e = kind == K_C2R ? rs : cs;
  for (long long v0 = 0; v0 < a.nv; v0 += kMaxGridY) {
    PassArgs b = a;
    b.nv = (int)(a.nv - v0 < kMaxGridY ? a.nv - v0 : kMaxGridY);
    b.src = static_cast<const char*>(a.src) + v0 * a.s_src_l * src_e;
    b.dst = static_cast<char*>(a.dst) + v0 * a.s_dst_l * dst_e;
    cudaError_t err = launch_axis_one(prec_bytes, kind, contiguous, b, stream);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

cudaError_t launch_copy(const void* src, void* dst, size_t bytes, cudaStream_t stream) {
  if (bytes == 0 || src == dst) return cudaSuccess;
  const int blocks_max = sm_count() * 8;
  const uintptr_t ps = (uintptr_t)src, pd = (uintptr_t)dst;
  size_t head = 0;
  if (((ps | pd) & 15) == 0) {
    const size_t n16 = bytes / 16;
    if (n16) {
      const size_t want = (n16 + 4 * 256 - 1) / (4 * 256);
      const int blocks = (int)(want < (size_t)blocks_max ? (want ? want : 1) : blocks_max);
      copy16_kernel<<<blocks, 256, 0, stream>>>(reinterpret_cast<const uint4*>(src),
                                                 reinterpret_cast<uint4*>(dst), n16);
      g_launches.fetch_add(1, std::memory_order_relaxed);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    head = n16 * 16;
  }
  if (head < bytes) {
    const size_t rest = bytes - head;
    const size_t want = (rest + 255) / 256;
    const int blocks = (int)(want < (size_t)blocks_max ? want : blocks_max);
    copy1_kernel<<<blocks, 256, 0, stream>>>(reinterpret_cast<const unsigned char*>(src) + head,
                                              reinterpret_cast<unsigned char*>(dst) + head, rest);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  }
  return cudaSuccess;
}

long long launch_counter() { return g_launches.load(); }
void add_launches(long long n) { g_launches.fetch_add(n); }

}  // namespace gbfft
