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
//  * Stage 0 reads global memory directly and the last stage writes global
//    memory directly (the Stockham read/write patterns j + r*n/R are
//    coalesced), so a pass costs one HBM read and one HBM write of the array.
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

#include "gbfft_internal.h"

namespace gbfft {

namespace {

std::atomic<long long> g_launches{0};

template <typename T> struct CxOf;
template <> struct CxOf<float> { using type = float2; };
template <> struct CxOf<double> { using type = double2; };
template <typename T> using Cx = typename CxOf<T>::type;

template <typename C> __device__ __forceinline__ C cmk(decltype(C::x) a, decltype(C::x) b) {
  C r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * (-i)
template <typename C> __device__ __forceinline__ C cmul_mi(C a) { return cmk<C>(a.y, -a.x); }
// a * s for a real s
template <typename C> __device__ __forceinline__ C cscale(C a, decltype(C::x) s) { return cmk<C>(a.x * s, a.y * s); }

// ---------------------------------------------------------------------------
// Forward butterflies (sign -1), natural order in and out.
// ---------------------------------------------------------------------------
template <typename C> __device__ __forceinline__ void dft(C (&v)[2]) {
  C a = v[0];
  v[0] = cadd(a, v[1]);
  v[1] = csub(a, v[1]);
}

template <typename C> __device__ __forceinline__ void dft4v(C& a0, C& a1, C& a2, C& a3) {
  C t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = cmul_mi(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

template <typename C> __device__ __forceinline__ void dft(C (&v)[4]) { dft4v(v[0], v[1], v[2], v[3]); }

template <typename C> __device__ __forceinline__ void dft(C (&v)[3]) {
  using T = decltype(C::x);
  const T h = T(-0.5), s = T(0.86602540378443864676);
  C t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  C m = cmk<C>(v[0].x + h * t.x, v[0].y + h * t.y);
  v[0] = cadd(v[0], t);
  v[1] = cmk<C>(m.x + s * d.y, m.y - s * d.x);
  v[2] = cmk<C>(m.x - s * d.y, m.y + s * d.x);
}

template <typename C> __device__ __forceinline__ void dft(C (&v)[5]) {
  using T = decltype(C::x);
  const T c1 = T(0.3090169943749474241), c2 = T(-0.8090169943749474241);
  const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);
  C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  C a0 = v[0];
  C m1 = cmk<C>(a0.x + c1 * t1.x + c2 * t2.x, a0.y + c1 * t1.y + c2 * t2.y);
  C m2 = cmk<C>(a0.x + c2 * t1.x + c1 * t2.x, a0.y + c2 * t1.y + c1 * t2.y);
  C n1 = cmk<C>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
  C n2 = cmk<C>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
  v[0] = cadd(a0, cadd(t1, t2));
  // y = m -/+ i n
  v[1] = cmk<C>(m1.x + n1.y, m1.y - n1.x);
  v[4] = cmk<C>(m1.x - n1.y, m1.y + n1.x);
  v[2] = cmk<C>(m2.x + n2.y, m2.y - n2.x);
  v[3] = cmk<C>(m2.x - n2.y, m2.y + n2.x);
}

template <typename C> __device__ __forceinline__ void dft(C (&v)[7]) {
  using T = decltype(C::x);
  // cos(2 pi j / 7), sin(2 pi j / 7), j = 0..6
  const T cs[7] = {T(1.0), T(0.62348980185873353053), T(-0.22252093395631440429),
                   T(-0.90096886790241912624), T(-0.90096886790241912624),
                   T(-0.22252093395631440429), T(0.62348980185873353053)};
  const T sn[7] = {T(0.0), T(0.78183148246802980871), T(0.97492791218182360702),
                   T(0.43388373911755812048), T(-0.43388373911755812048),
                   T(-0.97492791218182360702), T(-0.78183148246802980871)};
  C t[3], u[3];
#pragma unroll
  for (int k = 1; k <= 3; ++k) {
    t[k - 1] = cadd(v[k], v[7 - k]);
    u[k - 1] = csub(v[k], v[7 - k]);
  }
  C a0 = v[0];
  v[0] = cadd(a0, cadd(t[0], cadd(t[1], t[2])));
#pragma unroll
  for (int m = 1; m <= 3; ++m) {
    C re = a0, im = cmk<C>(T(0), T(0));
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
      const T c = cs[(k * m) % 7], s = sn[(k * m) % 7];
      re = cmk<C>(re.x + c * t[k - 1].x, re.y + c * t[k - 1].y);
      im = cmk<C>(im.x + s * u[k - 1].x, im.y + s * u[k - 1].y);
    }
    v[m] = cmk<C>(re.x + im.y, re.y - im.x);
    v[7 - m] = cmk<C>(re.x - im.y, re.y + im.x);
  }
}

template <typename C> __device__ __forceinline__ void dft(C (&v)[8]) {
  using T = decltype(C::x);
  const T r2 = T(0.70710678118654752440);
  // even / odd radix-4 halves
  dft4v(v[0], v[2], v[4], v[6]);
  dft4v(v[1], v[3], v[5], v[7]);
  // odd half times W8^k1, k1 = 0..3; odd k1 values sit at v[1 + 2 k1]
  C o1 = cmk<C>((v[3].x + v[3].y) * r2, (v[3].y - v[3].x) * r2);    // * (1 - i)/sqrt2
  C o2 = cmul_mi(v[5]);                                                // * -i
  C o3 = cmk<C>((v[7].y - v[7].x) * r2, -(v[7].x + v[7].y) * r2);   // * (-1 - i)/sqrt2
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}

template <typename C> __device__ __forceinline__ void dft(C (&v)[16]) {
  using T = decltype(C::x);
  const T r2 = T(0.70710678118654752440);
  const T c8 = T(0.92387953251128675613), s8 = T(0.38268343236508977173);
  // n = j + 4 m, k = k1 + 4 k2: first DFT4 over m for each j
#pragma unroll
  for (int j = 0; j < 4; ++j) dft4v(v[j], v[j + 4], v[j + 8], v[j + 12]);
  // v[j + 4 k1] = b_j[k1]; multiply by W16^(j k1)
  v[5] = cmul(v[5], cmk<C>(c8, -s8));    // W^1
  v[9] = cmk<C>((v[9].x + v[9].y) * r2, (v[9].y - v[9].x) * r2);   // W^2
  v[13] = cmul(v[13], cmk<C>(s8, -c8));  // W^3
  v[6] = cmk<C>((v[6].x + v[6].y) * r2, (v[6].y - v[6].x) * r2);   // W^2
  v[10] = cmul_mi(v[10]);                // W^4
  v[14] = cmk<C>((v[14].y - v[14].x) * r2, -(v[14].x + v[14].y) * r2);  // W^6
  v[7] = cmul(v[7], cmk<C>(s8, -c8));    // W^3
  v[11] = cmk<C>((v[11].y - v[11].x) * r2, -(v[11].x + v[11].y) * r2);  // W^6
  v[15] = cmul(v[15], cmk<C>(-c8, s8));  // W^9
  // second DFT4 over j for each k1; result y[k1 + 4 k2] lands at v[4 k1 + k2]
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4v(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
  C w[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) w[i] = v[i];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = w[4 * k1 + k2];
}

// ---------------------------------------------------------------------------
// Per-thread view of one line: shared-memory slots and global addressing.
// ---------------------------------------------------------------------------
template <typename T, int KIND, bool CONTIG>
struct LineCtx {
  using C = Cx<T>;
  const C* tw;
  const void* src;
  void* dst;
  long long sb0, sb1, db0, db1, ssn, dsn;
  int N, L, tpl, t, line;
  bool valid, has1, inverse;

  __device__ __forceinline__ int sidx(int n) const {
    const int a = CONTIG ? line * N + n : n * L + line;
    return a + (a >> 5);
  }
  __device__ __forceinline__ C twiddle(int e) const { return __ldg(tw + e); }

  // Point n of the complex line this thread works on, as the forward
  // transform must see it.
  __device__ __forceinline__ C gload(int n) const {
    if (!valid) return cmk<C>(T(0), T(0));
    if (KIND == K_C2C) {
      C x = reinterpret_cast<const C*>(src)[sb0 + n * ssn];
      if (inverse) x.y = -x.y;
      return x;
    } else if (KIND == K_R2C) {
      const T* s = reinterpret_cast<const T*>(src);
      const T re = s[sb0 + n * ssn];
      const T im = has1 ? s[sb1 + n * ssn] : T(0);
      return cmk<C>(re, im);
    } else {
      // Hermitian extension of both half spectra (src/fft_generic.f90:318-330)
      const C* s = reinterpret_cast<const C*>(src);
      const bool low = 2 * n <= N;
      const int m = low ? n : N - n;
      C x1 = s[sb0 + m * ssn];
      C x2 = has1 ? s[sb1 + m * ssn] : cmk<C>(T(0), T(0));
      if (!low) {
        x1.y = -x1.y;
        x2.y = -x2.y;
      }
      if (n == 0 || 2 * n == N) {  // c2r ignores Im of the DC and Nyquist bins
        x1.y = T(0);
        x2.y = T(0);
      }
      // z = x1 + i x2, conjugated for the inverse-by-conjugation
      return cmk<C>(x1.x - x2.y, -(x1.y + x2.x));
    }
  }

  __device__ __forceinline__ void gstore(int n, C v) const {
    if (!valid) return;
    if (KIND == K_C2C) {
      if (inverse) v.y = -v.y;
      reinterpret_cast<C*>(dst)[db0 + n * dsn] = v;
    } else if (KIND == K_C2R) {
      T* d = reinterpret_cast<T*>(dst);
      d[db0 + n * dsn] = v.x;
      if (has1) d[db1 + n * dsn] = -v.y;
    }
  }
};

// One Stockham stage of radix R, shared buffer A -> B.  Butterfly b
// (0 <= b < n/R) reads points b + r n/R, multiplies by
// W_{Ns R}^{(b mod Ns) r}, transforms, and writes points
// (b - b mod Ns) R + b mod Ns + r Ns.  One butterfly in flight per thread.
template <typename T, int KIND, bool CONTIG, int R>
__device__ __forceinline__ void stage_pp(const LineCtx<T, KIND, CONTIG>& c, const Cx<T>* A, Cx<T>* B,
                                         int Ns) {
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
    dft(v);
    const int base = (b - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) B[c.sidx(base + r * Ns)] = v[r];
  }
}

// A stage of any radix (primes above 7): each output point is a direct sum
// over its R inputs, O(n R) per line.
template <typename T, int KIND, bool CONTIG>
__device__ void stage_pp_generic(const LineCtx<T, KIND, CONTIG>& c, const Cx<T>* A, Cx<T>* B, int R,
                                 int Ns) {
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

// Runtime-planned pass: any length up to kMaxN, any factorisation.  The
// lines are loaded into shared buffer 0, each stage ping-pongs between the
// two buffers, and the result is stored from the last buffer written.
template <typename T, int KIND, bool CONTIG>
__global__ void __launch_bounds__(kMaxThreads)
    axis_pass_kernel(const __grid_constant__ PassArgs a) {
  using C = Cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LineCtx<T, KIND, CONTIG> c;
  c.tw = reinterpret_cast<const C*>(a.tw);
  c.src = a.src;
  c.dst = a.dst;
  c.N = a.n;
  c.L = a.L;
  c.tpl = a.tpl;
  c.inverse = a.inverse != 0;
  c.ssn = a.s_src_n;
  c.dsn = a.s_dst_n;
  if (CONTIG) {
    c.t = threadIdx.x;
    c.line = threadIdx.y;
  } else {
    c.line = threadIdx.x;
    c.t = threadIdx.y;
  }
  const long long cl = (long long)blockIdx.x * a.L + c.line;
  const long long v = CONTIG ? 0 : (long long)blockIdx.y;
  c.valid = cl < a.nlines;
  if (KIND == K_C2C) {
    c.has1 = false;
    c.sb0 = CONTIG ? cl * a.s_src_l : cl + v * a.s_src_l;
    c.db0 = CONTIG ? cl * a.s_dst_l : cl + v * a.s_dst_l;
    c.sb1 = c.sb0;
    c.db1 = c.db0;
  } else {
    const long long r0 = 2 * cl, r1 = 2 * cl + 1;
    c.has1 = r1 < a.real_lines;
    c.sb0 = CONTIG ? r0 * a.s_src_l : r0 + v * a.s_src_l;
    c.sb1 = CONTIG ? r1 * a.s_src_l : r1 + v * a.s_src_l;
    c.db0 = CONTIG ? r0 * a.s_dst_l : r0 + v * a.s_dst_l;
    c.db1 = CONTIG ? r1 * a.s_dst_l : r1 + v * a.s_dst_l;
  }
  const size_t e = (size_t)a.n * a.L;
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + (e + (e >> 5) + 1);

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
    else stage_pp_generic<T, KIND, CONTIG>(c, A, B, R, Ns);
    __syncthreads();
    C* tmp = A;
    A = B;
    B = tmp;
    Ns *= R;
  }

  if (KIND == K_R2C) {
    // Separate the two half spectra: X1 = (Z_k + conj Z_{n-k}) / 2,
    // X2 = (Z_k - conj Z_{n-k}) / (2i), k = 0..n/2.
    if (c.valid) {
      C* d = reinterpret_cast<C*>(c.dst);
      const T h = T(0.5);
#pragma unroll 1
      for (int k = c.t; 2 * k <= c.N; k += c.tpl) {
        const C zk = A[c.sidx(k)], zm = A[c.sidx(k == 0 ? 0 : c.N - k)];
        d[c.db0 + k * c.dsn] = cmk<C>((zk.x + zm.x) * h, (zk.y - zm.y) * h);
        if (c.has1) d[c.db1 + k * c.dsn] = cmk<C>((zk.y + zm.y) * h, (zm.x - zk.x) * h);
      }
    }
  } else {
#pragma unroll 1
    for (int n = c.t; n < c.N; n += c.tpl) c.gstore(n, A[c.sidx(n)]);
  }
}

template <typename T, int KIND, bool CONTIG>
cudaError_t launch_typed(const PassArgs& a, cudaStream_t stream) {
  const size_t smem = pass_smem_bytes(sizeof(T), a.n, a.L);
  auto kern = axis_pass_kernel<T, KIND, CONTIG>;
  static std::atomic<size_t> smem_set{48 * 1024};
  if (smem > smem_set.load()) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    smem_set.store(smem);
  }
  const dim3 block = CONTIG ? dim3(a.tpl, a.L) : dim3(a.L, a.tpl);
  const dim3 grid((unsigned)((a.nlines + a.L - 1) / a.L), CONTIG ? 1u : (unsigned)a.nv);
  kern<<<grid, block, smem, stream>>>(a);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
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
  return 2 * (e + (e >> 5) + 1) * (size_t)(2 * prec_bytes);
}

cudaError_t launch_axis_pass(int prec_bytes, int kind, bool contiguous, const PassArgs& a,
                             cudaStream_t stream) {
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
