// Axis passes longer than one shared-memory tile: any length, any
// factorisation (src/glassman.f90:29-67 takes any N, and so must the
// backend).
//
// A line that does not fit a CTA's shared memory (more than kMaxN points,
// or FP64 lines whose two buffers exceed the tile limit) is transformed one
// radix stage per kernel, in global memory:
//  * every stage is the Stockham step of the single-tile kernels -- read the
//    line at stride n / R, twiddle by W_(NS R)^(r k) (taken from the n-root
//    table: index r k n / (NS R)), butterfly, write it back sorted -- with
//    one thread per butterfly; radices 2..16 keep the butterfly in
//    registers (dftg), any other prime runs as a direct sum, one thread per
//    output, accumulated in double;
//  * the first stage reads the pass's source and the last one writes its
//    destination; the stages between ping-pong through two engine-owned
//    scratch buffers (a single stage whose source is its destination goes
//    through one of them);
//  * r2c / c2r along a long real axis carry two real lines in one complex
//    line, as the single-tile kernels do: a pack (r2c) or Hermitian-merge
//    (c2r, Im of DC and Nyquist ignored: src/fft_generic.f90:318-330) kernel
//    fills a scratch buffer first, and a split (r2c) or unpack (c2r) kernel
//    writes the pass's destination last;
//  * backward transforms run as conj(F(conj x)), as everywhere else;
//  * strided passes map consecutive threads to neighbouring lines (unit
//    stride along x) and keep the scratch lines interleaved the same way,
//    contiguous passes map them to neighbouring points; both stay
//    coalesced.
// Each stage reads and writes the whole array, so a long axis costs about
// (stages + 2) sweeps instead of one.
//
// Lengths with a prime factor above kBluePrime (in or beyond one tile) run
// the chirp-z transform instead of a direct sum (Bluestein's algorithm):
// with w_j = exp(-i pi j^2 / n), jk = (j^2 + k^2 - (k - j)^2) / 2 gives
//   X_k = w_k sum_j (x_j w_j) conj(w_(k-j)),
// a circular convolution of length m (a power of two >= 2n - 1) of the
// zero-padded a_j = x_j w_j with b (conj w_j at j and m - j).  It runs as
// chirp-in (a, n -> m points), an m-point FFT, a pointwise product with
// FFT_m(b) / m conjugated, a second m-point FFT, and chirp-out
// (X_k = w_k conj F_k, m -> n points): O(n log n) instead of O(n p).
#include <algorithm>
#include <atomic>

#include "fft_common.cuh"
#include "gbfft_internal.h"

namespace gbfft {
namespace lng {

using namespace dev;

// Point j of line l (u = l % nu, v = l / nu) sits at u*s_u + v*s_v + j*s_n,
// in elements of the side's type.
struct Side {
  void* p;
  long long s_u, s_v, s_n;
};

struct StageArgs {
  Side in, out;
  const void* tw;        // exp(-2 pi i m / n), m < n
  long long lines, nu;   // lines of the pass, lines along u
  long long m;           // n / R: butterflies a line
  int n, R, NS;
  int conj_in, conj_out;
};

__device__ __forceinline__ long long line_off(const Side& s, long long l, long long nu) {
  return (l % nu) * s.s_u + (l / nu) * s.s_v;
}

constexpr int kThreads = 256;

// One radix-R stage, the butterfly in registers.  UFAST: consecutive
// threads take neighbouring lines (strided passes), else neighbouring
// butterflies of one line.
template <typename T, int R, bool UFAST>
__global__ void __launch_bounds__(kThreads) stage_kernel(const __grid_constant__ StageArgs a) {
  using C = Cx<T>;
  const C* in = static_cast<const C*>(a.in.p);
  C* out = static_cast<C*>(a.out.p);
  const C* tw = static_cast<const C*>(a.tw);
  const long long total = a.lines * a.m;
  const long long step_tw = (long long)a.n / ((long long)a.NS * R);
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    long long l, b;
    if (UFAST) {
      l = idx % a.lines;
      b = idx / a.lines;
    } else {
      b = idx % a.m;
      l = idx / a.m;
    }
    const long long k = b % a.NS;
    const long long ib = line_off(a.in, l, a.nu), ob = line_off(a.out, l, a.nu);
    C x[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      x[r] = in[ib + (b + r * a.m) * a.in.s_n];
      if (a.conj_in) x[r].y = -x[r].y;
    }
    if (a.NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) x[r] = cmul(x[r], tw[r * k * step_tw]);  // r k < NS R: index < n
    }
    dftg<R>(x);
    const long long jb = (b - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      C y = x[r];
      if (a.conj_out) y.y = -y.y;
      out[ob + (jb + (long long)r * a.NS) * a.out.s_n] = y;
    }
  }
}

// One stage of any radix R, as a direct sum: one thread per output q of a
// butterfly, y_q = sum_r x_r W_n^(r (k n/(NS R) + q n/R)), in double.
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) stage_generic_kernel(const __grid_constant__ StageArgs a) {
  using C = Cx<T>;
  const C* in = static_cast<const C*>(a.in.p);
  C* out = static_cast<C*>(a.out.p);
  const C* tw = static_cast<const C*>(a.tw);
  const long long R = a.R, n = a.n;
  const long long total = a.lines * n;
  const long long step_tw = n / ((long long)a.NS * R), step_q = n / R;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    long long l, b, q;
    if (UFAST) {
      l = idx % a.lines;
      const long long rest = idx / a.lines;
      q = rest % R;
      b = rest / R;
    } else {
      b = idx % a.m;
      const long long rest = idx / a.m;
      q = rest % R;
      l = rest / R;
    }
    const long long k = b % a.NS;
    const long long ib = line_off(a.in, l, a.nu), ob = line_off(a.out, l, a.nu);
    const long long e1 = (k * step_tw + q * step_q) % n;  // exponent step per input r
    double sx = 0.0, sy = 0.0;
    long long e = 0;
    for (long long r = 0; r < R; ++r) {
      C x = in[ib + (b + r * a.m) * a.in.s_n];
      const double xx = (double)x.x, xy = a.conj_in ? -(double)x.y : (double)x.y;
      const C w = tw[e];
      sx += xx * (double)w.x - xy * (double)w.y;
      sy += xx * (double)w.y + xy * (double)w.x;
      e += e1;
      if (e >= n) e -= n;
    }
    C y;
    y.x = (T)sx;
    y.y = (T)(a.conj_out ? -sy : sy);
    out[ob + ((b - k) * R + k + q * a.NS) * a.out.s_n] = y;
  }
}

// Real-line pairs of an r2c / c2r pass: complex line l (u = l % nu pairs,
// v = l / nu) carries real lines 2u and 2u + 1 (the latter when
// 2u + 1 < real_u).  `cx` is the complex side (the half spectra), `re` the
// real side, `s` the scratch lines (interleaved like a Side).
struct RealArgs {
  Side re, cx, s;
  long long lines, nu, real_u;
  int n;
};

__device__ __forceinline__ long long pair_off(const Side& s, long long l, long long nu, int half) {
  return (2 * (l % nu) + half) * s.s_u + (l / nu) * s.s_v;
}

// r2c input: z_j = a_j + i b_j.
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) pack_kernel(const __grid_constant__ RealArgs a) {
  using C = Cx<T>;
  const T* re = static_cast<const T*>(a.re.p);
  C* s = static_cast<C*>(a.s.p);
  const long long total = a.lines * a.n;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    const long long l = UFAST ? idx % a.lines : idx / a.n, j = UFAST ? idx / a.lines : idx % a.n;
    const bool has1 = 2 * (l % a.nu) + 1 < a.real_u;
    C z;
    z.x = re[pair_off(a.re, l, a.nu, 0) + j * a.re.s_n];
    z.y = has1 ? re[pair_off(a.re, l, a.nu, 1) + j * a.re.s_n] : T(0);
    s[line_off(a.s, l, a.nu) + j * a.s.s_n] = z;
  }
}

// r2c output: X1_k = (Z_k + conj Z_(n-k)) / 2, X2_k = (Z_k - conj Z_(n-k)) / (2 i).
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) split_kernel(const __grid_constant__ RealArgs a) {
  using C = Cx<T>;
  const C* s = static_cast<const C*>(a.s.p);
  C* cx = static_cast<C*>(a.cx.p);
  const long long h = a.n / 2 + 1, total = a.lines * h;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    const long long l = UFAST ? idx % a.lines : idx / h, k = UFAST ? idx / a.lines : idx % h;
    const long long so = line_off(a.s, l, a.nu);
    const C zk = s[so + k * a.s.s_n], zm = s[so + ((a.n - k) % a.n) * a.s.s_n];
    const T half = T(0.5);
    C x1, x2;
    x1.x = (zk.x + zm.x) * half;
    x1.y = (zk.y - zm.y) * half;
    x2.x = (zk.y + zm.y) * half;
    x2.y = (zm.x - zk.x) * half;
    cx[pair_off(a.cx, l, a.nu, 0) + k * a.cx.s_n] = x1;
    if (2 * (l % a.nu) + 1 < a.real_u) cx[pair_off(a.cx, l, a.nu, 1) + k * a.cx.s_n] = x2;
  }
}

// c2r input: the Hermitian extension of both half spectra (Im of the DC and
// Nyquist bins ignored), z = x1 + i x2, conjugated for the inverse.
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) merge_kernel(const __grid_constant__ RealArgs a) {
  using C = Cx<T>;
  const C* cx = static_cast<const C*>(a.cx.p);
  C* s = static_cast<C*>(a.s.p);
  const long long total = a.lines * a.n;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    const long long l = UFAST ? idx % a.lines : idx / a.n, j = UFAST ? idx / a.lines : idx % a.n;
    const bool low = 2 * j <= a.n, has1 = 2 * (l % a.nu) + 1 < a.real_u;
    const long long m = low ? j : a.n - j;
    C x1 = cx[pair_off(a.cx, l, a.nu, 0) + m * a.cx.s_n];
    C x2 = has1 ? cx[pair_off(a.cx, l, a.nu, 1) + m * a.cx.s_n] : C{T(0), T(0)};
    if (!low) {
      x1.y = -x1.y;
      x2.y = -x2.y;
    }
    if (j == 0 || 2 * j == a.n) {
      x1.y = T(0);
      x2.y = T(0);
    }
    C z;
    z.x = x1.x - x2.y;
    z.y = -(x1.y + x2.x);
    s[line_off(a.s, l, a.nu) + j * a.s.s_n] = z;
  }
}

// c2r output: the forward transform Y of conj(z) gives z's inverse as
// conj(Y): real line 2u = Re Y, real line 2u + 1 = -Im Y.
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) unpack_kernel(const __grid_constant__ RealArgs a) {
  using C = Cx<T>;
  const C* s = static_cast<const C*>(a.s.p);
  T* re = static_cast<T*>(a.re.p);
  const long long total = a.lines * a.n;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    const long long l = UFAST ? idx % a.lines : idx / a.n, j = UFAST ? idx / a.lines : idx % a.n;
    const C y = s[line_off(a.s, l, a.nu) + j * a.s.s_n];
    re[pair_off(a.re, l, a.nu, 0) + j * a.re.s_n] = y.x;
    if (2 * (l % a.nu) + 1 < a.real_u) re[pair_off(a.re, l, a.nu, 1) + j * a.re.s_n] = -y.y;
  }
}


// ---- chirp-z path
struct ChirpArgs {
  Side in, out;
  const void* chirp;  // w_j, j < n
  const void* filt;   // FFT_m(b) / m
  long long lines, nu;
  int n, m;
  int conj_in, conj_out;
};

// a_j = x_j w_j (j < n), 0 (n <= j < m): the pass's (or a packed) line in,
// an m-point scratch line out
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) chirp_in_kernel(const __grid_constant__ ChirpArgs a) {
  using C = Cx<T>;
  const C* in = static_cast<const C*>(a.in.p);
  C* out = static_cast<C*>(a.out.p);
  const C* w = static_cast<const C*>(a.chirp);
  const long long total = a.lines * a.m;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    const long long l = UFAST ? idx % a.lines : idx / a.m, j = UFAST ? idx / a.lines : idx % a.m;
    C y{T(0), T(0)};
    if (j < a.n) {
      C x = in[line_off(a.in, l, a.nu) + j * a.in.s_n];
      if (a.conj_in) x.y = -x.y;
      y = cmul(x, w[j]);
    }
    out[line_off(a.out, l, a.nu) + j * a.out.s_n] = y;
  }
}

// in place: A_k <- conj(A_k FFT_m(b)_k / m), so that the next forward FFT
// gives the conjugate of the convolution
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) chirp_filter_kernel(const __grid_constant__ ChirpArgs a) {
  using C = Cx<T>;
  C* buf = static_cast<C*>(a.out.p);
  const C* f = static_cast<const C*>(a.filt);
  const long long total = a.lines * a.m;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    const long long l = UFAST ? idx % a.lines : idx / a.m, k = UFAST ? idx / a.lines : idx % a.m;
    const long long o = line_off(a.out, l, a.nu) + k * a.out.s_n;
    C p = cmul(buf[o], f[k]);
    p.y = -p.y;
    buf[o] = p;
  }
}

// X_k = w_k conj(F_k), k < n: an m-point scratch line in, the pass's (or a
// scratch) line out
template <typename T, bool UFAST>
__global__ void __launch_bounds__(kThreads) chirp_out_kernel(const __grid_constant__ ChirpArgs a) {
  using C = Cx<T>;
  const C* in = static_cast<const C*>(a.in.p);
  C* out = static_cast<C*>(a.out.p);
  const C* w = static_cast<const C*>(a.chirp);
  const long long total = a.lines * a.n;
  for (long long idx = (long long)blockIdx.x * kThreads + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * kThreads) {
    const long long l = UFAST ? idx % a.lines : idx / a.n, k = UFAST ? idx / a.lines : idx % a.n;
    C f = in[line_off(a.in, l, a.nu) + k * a.in.s_n];
    f.y = -f.y;
    C x = cmul(w[k], f);
    if (a.conj_out) x.y = -x.y;
    out[line_off(a.out, l, a.nu) + k * a.out.s_n] = x;
  }
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

unsigned grid_for(long long work) {
  const long long want = (work + kThreads - 1) / kThreads;
  const long long cap = (long long)sm_count() * 16;
  return (unsigned)std::max(1ll, std::min(want, cap));
}

template <typename T, bool UFAST>
cudaError_t launch_stage(const StageArgs& s, cudaStream_t st) {
  const unsigned g = grid_for(s.lines * (s.R <= 16 ? s.m : (long long)s.n));
  switch (s.R) {
    case 1: stage_kernel<T, 1, UFAST><<<g, kThreads, 0, st>>>(s); break;
    case 2: stage_kernel<T, 2, UFAST><<<g, kThreads, 0, st>>>(s); break;
    case 3: stage_kernel<T, 3, UFAST><<<g, kThreads, 0, st>>>(s); break;
    case 4: stage_kernel<T, 4, UFAST><<<g, kThreads, 0, st>>>(s); break;
    case 5: stage_kernel<T, 5, UFAST><<<g, kThreads, 0, st>>>(s); break;
    case 7: stage_kernel<T, 7, UFAST><<<g, kThreads, 0, st>>>(s); break;
    case 8: stage_kernel<T, 8, UFAST><<<g, kThreads, 0, st>>>(s); break;
    case 16: stage_kernel<T, 16, UFAST><<<g, kThreads, 0, st>>>(s); break;
    default: stage_generic_kernel<T, UFAST><<<g, kThreads, 0, st>>>(s); break;
  }
  add_launches(1);
  return cudaGetLastError();
}

template <typename T, bool UFAST>
cudaError_t run(int kind, const PassArgs& a, void* scratch, size_t scratch_bytes, cudaStream_t st) {
  using C = Cx<T>;
  const int n = a.n;
  const bool contig = !UFAST;
  // lines of the pass: complex lines (pairs for r2c / c2r), over u and v
  const long long nu = a.nlines, lines = a.nlines * (contig ? 1 : (long long)a.nv);
  const size_t need = (size_t)lines * n * sizeof(C);
  if (2 * need > scratch_bytes) return cudaErrorInvalidValue;
  C* sb[2] = {static_cast<C*>(scratch), reinterpret_cast<C*>(static_cast<char*>(scratch) + need)};
  // scratch lines interleaved like the pass's lines
  auto scratch_side = [&](int i) {
    Side s;
    s.p = sb[i];
    if (UFAST) {
      s.s_u = 1;
      s.s_v = nu;
      s.s_n = lines;
    } else {
      s.s_u = n;
      s.s_v = (long long)n * nu;
      s.s_n = 1;
    }
    return s;
  };
  // the pass's own sides (complex or real elements)
  auto side = [&](const void* p, long long s_n, long long s_l) {
    Side s;
    s.p = const_cast<void*>(p);
    s.s_n = s_n;
    s.s_u = contig ? s_l : 1;
    s.s_v = contig ? 0 : s_l;
    return s;
  };
  const Side src = side(a.src, a.s_src_n, a.s_src_l), dst = side(a.dst, a.s_dst_n, a.s_dst_l);
  RealArgs ra;
  ra.lines = lines;
  ra.nu = nu;
  ra.real_u = a.real_lines;
  ra.n = n;
  const unsigned g = grid_for(lines * (long long)n);
  cudaError_t err;
  // stage inputs: the pass's source (c2c) or scratch 0 after pack / merge
  Side first_in = src;
  int first_conj = a.inverse;
  if (kind == K_R2C) {
    ra.re = src;
    ra.s = scratch_side(0);
    pack_kernel<T, UFAST><<<g, kThreads, 0, st>>>(ra);
    add_launches(1);
    first_in = scratch_side(0);
    first_conj = 0;
  } else if (kind == K_C2R) {
    ra.cx = src;
    ra.s = scratch_side(0);
    merge_kernel<T, UFAST><<<g, kThreads, 0, st>>>(ra);
    add_launches(1);
    first_in = scratch_side(0);
    first_conj = 0;
  }
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  // stage outputs: scratch, except the last stage of a c2c pass (the
  // destination, unless a single stage would read and write it in place)
  const int nst = a.nst;
  const bool direct_out = kind == K_C2C && !(nst == 1 && a.src == a.dst);
  int cur = kind == K_C2C ? -1 : 0;  // scratch buffer holding the stage input (-1: source)
  int ns = 1;
  for (int s = 0; s < nst; ++s) {
    const int R = a.radix[s];
    StageArgs sa;
    sa.in = cur < 0 ? first_in : (s == 0 ? first_in : scratch_side(cur));
    const bool last = s == nst - 1;
    int next = cur < 0 ? 0 : 1 - cur;
    sa.out = (last && direct_out) ? dst : scratch_side(next);
    sa.tw = a.tw;
    sa.lines = lines;
    sa.nu = nu;
    sa.m = n / R;
    sa.n = n;
    sa.R = R;
    sa.NS = ns;
    sa.conj_in = s == 0 ? first_conj : 0;
    sa.conj_out = (last && direct_out) ? a.inverse : 0;
    if ((err = launch_stage<T, UFAST>(sa, st)) != cudaSuccess) return err;
    cur = next;
    ns *= R;
  }
  if (kind == K_C2C && !direct_out) {
    // one stage went to scratch: copy it out (radix 1), conjugated back
    StageArgs sa;
    sa.in = scratch_side(cur);
    sa.out = dst;
    sa.tw = a.tw;
    sa.lines = lines;
    sa.nu = nu;
    sa.m = n;
    sa.n = n;
    sa.R = 1;
    sa.NS = 1;
    sa.conj_in = 0;
    sa.conj_out = a.inverse;
    if ((err = launch_stage<T, UFAST>(sa, st)) != cudaSuccess) return err;
  } else if (kind == K_R2C) {
    ra.s = scratch_side(cur);
    ra.cx = dst;
    split_kernel<T, UFAST><<<grid_for(lines * (long long)(n / 2 + 1)), kThreads, 0, st>>>(ra);
    add_launches(1);
  } else if (kind == K_C2R) {
    ra.s = scratch_side(cur);
    ra.re = dst;
    unpack_kernel<T, UFAST><<<g, kThreads, 0, st>>>(ra);
    add_launches(1);
  }
  return cudaGetLastError();
}


// The chirp-z pass: pack / merge (real passes), chirp-in, m-point FFT,
// filter, m-point FFT, chirp-out, split / unpack (real passes).  Scratch:
// two buffers of `lines` m-point lines; the packed n-point lines sit in
// buffer 1 until chirp-in has read them.
template <typename T, bool UFAST>
cudaError_t run_blue(int kind, const PassArgs& a, void* scratch, size_t scratch_bytes, cudaStream_t st) {
  using C = Cx<T>;
  const BlueTables& b = *a.blue;
  const int n = a.n, m = b.m;
  const bool contig = !UFAST;
  const long long nu = a.nlines, lines = a.nlines * (contig ? 1 : (long long)a.nv);
  const size_t need = (size_t)lines * m * sizeof(C);
  if (2 * need > scratch_bytes) return cudaErrorInvalidValue;
  C* sb[2] = {static_cast<C*>(scratch), reinterpret_cast<C*>(static_cast<char*>(scratch) + need)};
  auto scratch_side = [&](int i, int len) {
    Side s;
    s.p = sb[i];
    if (UFAST) {
      s.s_u = 1;
      s.s_v = nu;
      s.s_n = lines;
    } else {
      s.s_u = len;
      s.s_v = (long long)len * nu;
      s.s_n = 1;
    }
    return s;
  };
  auto side = [&](const void* p, long long s_n, long long s_l) {
    Side s;
    s.p = const_cast<void*>(p);
    s.s_n = s_n;
    s.s_u = contig ? s_l : 1;
    s.s_v = contig ? 0 : s_l;
    return s;
  };
  const Side src = side(a.src, a.s_src_n, a.s_src_l), dst = side(a.dst, a.s_dst_n, a.s_dst_l);
  RealArgs ra;
  ra.lines = lines;
  ra.nu = nu;
  ra.real_u = a.real_lines;
  ra.n = n;
  cudaError_t err;
  ChirpArgs ca;
  ca.chirp = b.chirp;
  ca.filt = b.filt;
  ca.lines = lines;
  ca.nu = nu;
  ca.n = n;
  ca.m = m;
  ca.in = src;
  ca.conj_in = a.inverse;
  ca.conj_out = 0;
  if (kind == K_R2C || kind == K_C2R) {
    ra.s = scratch_side(1, n);
    if (kind == K_R2C) {
      ra.re = src;
      pack_kernel<T, UFAST><<<grid_for(lines * (long long)n), kThreads, 0, st>>>(ra);
    } else {
      ra.cx = src;
      merge_kernel<T, UFAST><<<grid_for(lines * (long long)n), kThreads, 0, st>>>(ra);
    }
    add_launches(1);
    ca.in = scratch_side(1, n);
    ca.conj_in = 0;
  }
  ca.out = scratch_side(0, m);
  chirp_in_kernel<T, UFAST><<<grid_for(lines * (long long)m), kThreads, 0, st>>>(ca);
  add_launches(1);
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  int cur = 0;
  for (int round = 0; round < 2; ++round) {
    int ns = 1;
    for (int s = 0; s < b.nst; ++s) {
      const int R = b.radix[s];
      StageArgs sa;
      sa.in = scratch_side(cur, m);
      sa.out = scratch_side(1 - cur, m);
      sa.tw = b.twm;
      sa.lines = lines;
      sa.nu = nu;
      sa.m = m / R;
      sa.n = m;
      sa.R = R;
      sa.NS = ns;
      sa.conj_in = 0;
      sa.conj_out = 0;
      if ((err = launch_stage<T, UFAST>(sa, st)) != cudaSuccess) return err;
      cur = 1 - cur;
      ns *= R;
    }
    if (round == 0) {
      ca.out = scratch_side(cur, m);
      chirp_filter_kernel<T, UFAST><<<grid_for(lines * (long long)m), kThreads, 0, st>>>(ca);
      add_launches(1);
      if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
  }
  ca.in = scratch_side(cur, m);
  if (kind == K_C2C) {
    ca.out = dst;
    ca.conj_out = a.inverse;
  } else {
    ca.out = scratch_side(1 - cur, n);
    ca.conj_out = 0;
  }
  chirp_out_kernel<T, UFAST><<<grid_for(lines * (long long)n), kThreads, 0, st>>>(ca);
  add_launches(1);
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  if (kind == K_R2C) {
    ra.s = scratch_side(1 - cur, n);
    ra.cx = dst;
    split_kernel<T, UFAST><<<grid_for(lines * (long long)(n / 2 + 1)), kThreads, 0, st>>>(ra);
    add_launches(1);
  } else if (kind == K_C2R) {
    ra.s = scratch_side(1 - cur, n);
    ra.re = dst;
    unpack_kernel<T, UFAST><<<grid_for(lines * (long long)n), kThreads, 0, st>>>(ra);
    add_launches(1);
  }
  return cudaGetLastError();
}

}  // namespace lng

size_t long_pass_scratch_bytes(int prec_bytes, bool contiguous, const PassArgs& a) {
  const long long lines = a.nlines * (contiguous ? 1 : (long long)a.nv);
  const long long len = a.blue ? a.blue->m : a.n;
  return 2 * (size_t)lines * (size_t)len * 2 * (size_t)prec_bytes;
}

cudaError_t launch_long_pass(int prec_bytes, int kind, bool contiguous, const PassArgs& a, void* scratch,
                             size_t scratch_bytes, cudaStream_t stream) {
  if (a.row_w != 0 || !scratch) return cudaErrorInvalidValue;
  if (a.blue) {
    const BlueTables& b = *a.blue;
    if (b.m < 2 * a.n - 1 || b.nst < 1 || !b.chirp || !b.filt || !b.twm) return cudaErrorInvalidValue;
    if (prec_bytes == 4)
      return contiguous ? lng::run_blue<float, false>(kind, a, scratch, scratch_bytes, stream)
                        : lng::run_blue<float, true>(kind, a, scratch, scratch_bytes, stream);
    if (prec_bytes == 8)
      return contiguous ? lng::run_blue<double, false>(kind, a, scratch, scratch_bytes, stream)
                        : lng::run_blue<double, true>(kind, a, scratch, scratch_bytes, stream);
    return cudaErrorInvalidValue;
  }
  if (a.nst < 1 || !a.tw) return cudaErrorInvalidValue;
  if (kind == K_C2C && a.n < 1) return cudaErrorInvalidValue;
  if (prec_bytes == 4)
    return contiguous ? lng::run<float, false>(kind, a, scratch, scratch_bytes, stream)
                      : lng::run<float, true>(kind, a, scratch, scratch_bytes, stream);
  if (prec_bytes == 8)
    return contiguous ? lng::run<double, false>(kind, a, scratch, scratch_bytes, stream)
                      : lng::run<double, true>(kind, a, scratch, scratch_bytes, stream);
  return cudaErrorInvalidValue;
}

}  // namespace gbfft
