// Complex helpers, radix butterflies and the per-line addressing shared by
// the axis-pass kernels (fft_axis.cu: runtime plans; fft_fast.cu:
// compile-time power-of-two plans).
#pragma once

#include <type_traits>

#include "gbfft_internal.h"

namespace gbfft {
namespace dev {

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
// FP32: one packed two-lane add (FADD2) per complex add or subtract, rounded
// exactly as the two scalar adds.  A swapped or negated pair (a * -i) as an
// operand would cost register moves, so the butterflies below write
// t +/- (-i) d component-wise.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }

// ---------------------------------------------------------------------------
// Forward butterflies (sign -1), natural order in and out.
// ---------------------------------------------------------------------------
template <typename C> __device__ __forceinline__ void dft4v(C& a0, C& a1, C& a2, C& a3) {
  C t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), d = csub(a1, a3);
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cmk<C>(t1.x + d.y, t1.y - d.x);  // t1 + (-i) d
  a3 = cmk<C>(t1.x - d.y, t1.y + d.x);  // t1 - (-i) d
}

template <typename C> __device__ __forceinline__ void dft2p(C* v) {
  C a = v[0];
  v[0] = cadd(a, v[1]);
  v[1] = csub(a, v[1]);
}

template <typename C> __device__ __forceinline__ void dft4p(C* v) { dft4v(v[0], v[1], v[2], v[3]); }

template <typename C> __device__ __forceinline__ void dft3p(C* v) {
  using T = decltype(C::x);
  const T h = T(-0.5), s = T(0.86602540378443864676);
  C t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  C m = cmk<C>(v[0].x + h * t.x, v[0].y + h * t.y);
  v[0] = cadd(v[0], t);
  v[1] = cmk<C>(m.x + s * d.y, m.y - s * d.x);
  v[2] = cmk<C>(m.x - s * d.y, m.y + s * d.x);
}

template <typename C> __device__ __forceinline__ void dft5p(C* v) {
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

template <typename C> __device__ __forceinline__ void dft7p(C* v) {
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

template <typename C> __device__ __forceinline__ void dft8p(C* v) {
  using T = decltype(C::x);
  const T r2 = T(0.70710678118654752440);
  dft4v(v[0], v[2], v[4], v[6]);
  dft4v(v[1], v[3], v[5], v[7]);
  // odd half times W8^k1 (k1 = 1..3); its values sit at v[1 + 2 k1]
  C o1 = cmk<C>((v[3].x + v[3].y) * r2, (v[3].y - v[3].x) * r2);   // * (1 - i)/sqrt2
  C o2 = cmul_mi(v[5]);                                               // * -i
  C o3 = cmk<C>((v[7].y - v[7].x) * r2, -(v[7].x + v[7].y) * r2);  // * (-1 - i)/sqrt2
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cmk<C>(e2.x + o2.x, e2.y + o2.y);  // o2 = -i v[5]: component-wise
  v[6] = cmk<C>(e2.x - o2.x, e2.y - o2.y);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}

template <typename C> __device__ __forceinline__ void dft16p(C* v) {
  using T = decltype(C::x);
  const T r2 = T(0.70710678118654752440);
  const T c8 = T(0.92387953251128675613), s8 = T(0.38268343236508977173);
  // n = j + 4 m, k = k1 + 4 k2: DFT4 over m for each j
#pragma unroll
  for (int j = 0; j < 4; ++j) dft4v(v[j], v[j + 4], v[j + 8], v[j + 12]);
  // v[j + 4 k1] = b_j[k1]; multiply by W16^(j k1)
  v[5] = cmul(v[5], cmk<C>(c8, -s8));                                    // W^1
  v[9] = cmk<C>((v[9].x + v[9].y) * r2, (v[9].y - v[9].x) * r2);        // W^2
  v[13] = cmul(v[13], cmk<C>(s8, -c8));                                  // W^3
  v[6] = cmk<C>((v[6].x + v[6].y) * r2, (v[6].y - v[6].x) * r2);        // W^2
  v[10] = cmul_mi(v[10]);                                                // W^4
  v[14] = cmk<C>((v[14].y - v[14].x) * r2, -(v[14].x + v[14].y) * r2);  // W^6
  v[7] = cmul(v[7], cmk<C>(s8, -c8));                                    // W^3
  v[11] = cmk<C>((v[11].y - v[11].x) * r2, -(v[11].x + v[11].y) * r2);  // W^6
  v[15] = cmul(v[15], cmk<C>(-c8, s8));                                  // W^9
  // DFT4 over j for each k1; y[k1 + 4 k2] lands at v[4 k1 + k2]
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

// Radix 32 as two radix-16 halves (even / odd points) joined by W32^k.
template <typename C> __device__ __forceinline__ void dft32p(C* v) {
  using T = decltype(C::x);
  // cos(pi k / 16), k = 0..8
  const T c[9] = {T(1.0), T(0.98078528040323044913), T(0.92387953251128675613),
                  T(0.83146961230254523708), T(0.70710678118654752440), T(0.55557023301960222474),
                  T(0.38268343236508977173), T(0.19509032201612826785), T(0.0)};
  C e[16], o[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    e[i] = v[2 * i];
    o[i] = v[2 * i + 1];
  }
  dft16p(e);
  dft16p(o);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    // W32^k = cos(pi k/16) - i sin(pi k/16); sin(pi k/16) = cos(pi (8-k)/16)
    C w;
    if (k <= 8) w = cmk<C>(c[k], -c[8 - k]);
    else w = cmk<C>(-c[16 - k], -c[k - 8]);
    if (k == 8) {  // t = -i o
      v[k] = cmk<C>(e[k].x + o[k].y, e[k].y - o[k].x);
      v[k + 16] = cmk<C>(e[k].x - o[k].y, e[k].y + o[k].x);
      continue;
    }
    C t = (k == 0) ? o[k] : cmul(o[k], w);
    v[k] = cadd(e[k], t);
    v[k + 16] = csub(e[k], t);
  }
}

template <int R, typename C> __device__ __forceinline__ void dftp(C* v) {
  if constexpr (R == 2) dft2p(v);
  else if constexpr (R == 3) dft3p(v);
  else if constexpr (R == 4) dft4p(v);
  else if constexpr (R == 5) dft5p(v);
  else if constexpr (R == 7) dft7p(v);
  else if constexpr (R == 8) dft8p(v);
  else if constexpr (R == 16) dft16p(v);
  else if constexpr (R == 32) dft32p(v);
}

// ---------------------------------------------------------------------------
// Butterflies of any 7-smooth radix up to 32 (and products of those), built
// at compile time as a two-level Cooley-Tukey split R = P * Q in registers,
// with the internal twiddles W_R^{n2 k1} evaluated by a constexpr
// sine/cosine (argument reduced exactly on the rational angle, Taylor series
// in double).
// ---------------------------------------------------------------------------
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

// Forward DFT of an odd prime size R in registers from the symmetric pairs
// t_j = x_j + x_{R-j}, u_j = x_j - x_{R-j} (j = 1..(R-1)/2):
//   Y_m     = x_0 + sum_j cos(2 pi j m / R) t_j - i sum_j sin(2 pi j m / R) u_j
//   Y_{R-m} = the same with + i,
// (R-1)^2 real multiply-adds per component instead of 2 R^2.
template <int R, typename C>
__device__ __forceinline__ void dft_odd(C* v) {
  using T = decltype(C::x);
  constexpr int H = (R - 1) / 2;
  C t[H], u[H];
  static_for<1, H + 1>([&](auto J) {
    constexpr int j = decltype(J)::value;
    t[j - 1] = cadd(v[j], v[R - j]);
    u[j - 1] = csub(v[j], v[R - j]);
  });
  const C a0 = v[0];
  C s0 = a0;
  static_for<0, H>([&](auto J) { s0 = cadd(s0, t[decltype(J)::value]); });
  v[0] = s0;
  static_for<1, H + 1>([&](auto Mi) {
    constexpr int m = decltype(Mi)::value;
    C re = a0, im = cmk<C>(T(0), T(0));
    static_for<1, H + 1>([&](auto J) {
      constexpr int j = decltype(J)::value;
      constexpr int e = (j * m) % R;
      const T c = T(root_c<R, e>()), sn = T(root_s<R, e>());
      re = cmk<C>(re.x + c * t[j - 1].x, re.y + c * t[j - 1].y);
      im = cmk<C>(im.x + sn * u[j - 1].x, im.y + sn * u[j - 1].y);
    });
    v[m] = cmk<C>(re.x + im.y, re.y - im.x);
    v[R - m] = cmk<C>(re.x - im.y, re.y + im.x);
  });
}

// Forward DFT of size R in registers, natural order in and out.
template <int R, typename C>
__device__ __forceinline__ void dftg(C* v) {
  if constexpr (R == 1) {
  } else if constexpr (special_radix(R)) {
    dftp<R>(v);
  } else if constexpr (pick_p(R) == R) {
    static_assert(R % 2 == 1, "composite radix without a small factor");
    dft_odd<R>(v);
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


// ---------------------------------------------------------------------------
// Per-thread view of one line: shared-memory slots and global addressing.
// ---------------------------------------------------------------------------
// CG: read sources through L2 only (ld.global.cg), for data other CTAs of
// the same kernel wrote moments earlier.  PRED: loads of padding lines are
// predicated off (and read as zero); without it a padding line loads the
// line it is clamped to (see init_at) and only its stores are skipped --
// faster in the power-of-two kernel, slower in the balanced and
// mixed-radix ones (measured).
template <typename T, int KIND, bool CONTIG, bool CG = false, bool PRED = true>
struct LineCtx {
  using C = Cx<T>;
  using real_t = T;
  static constexpr int kind = KIND;
  static constexpr bool contiguous = CONTIG;
  const C* tw;
  const void* src;
  void* dst;
  long long sb0, sb1, db0, db1, ssn, dsn;
  int N, L, tpl, t, line;
  bool valid, has1, inverse, pvec, cvec;
#ifdef GB_DEBUG_BOUNDS
  // bounds-checked build: every global access is checked against the
  // array's extent; one outside it records 2 in the status word and is
  // skipped (a load reads zero)
  long long se, de;
  int* st;
  __device__ __forceinline__ bool ok(long long off, int w, long long n) const {
    if (off >= 0 && off + w <= n) return true;
    if (st) atomicExch(st, 2);
    return false;
  }
#define GB_SRC(off, w) ok((off), (w), se)
#define GB_DST(off, w) ok((off), (w), de)
#else
#define GB_SRC(off, w) true
#define GB_DST(off, w) true
#endif

  __device__ __forceinline__ void init(const PassArgs& a) {
    if (CONTIG)
      init_at(a, threadIdx.x, threadIdx.y, (long long)blockIdx.x * a.L + threadIdx.y, 0, a.nlines);
    else
      init_at(a, threadIdx.y, threadIdx.x, (long long)blockIdx.x * a.L + threadIdx.x,
              (long long)blockIdx.y, a.nlines);
  }

  // Thread `t_` of line `line_` of a tile; cl is the complex line (its u
  // index on strided axes), v the strided axes' second index, and lines at
  // or past `limit` are padding.
  __device__ __forceinline__ void init_at(const PassArgs& a, int t_, int line_, long long cl, long long v,
                                          long long limit) {
    tw = reinterpret_cast<const C*>(a.tw);
    src = a.src;
    dst = a.dst;
    N = a.n;
    L = a.L;
    tpl = a.tpl;
    inverse = a.inverse != 0;
    ssn = a.s_src_n;
    dsn = a.s_dst_n;
#ifdef GB_DEBUG_BOUNDS
    se = a.src_elems;
    de = a.dst_elems;
    st = a.status;
#endif
    pvec = !CONTIG && (a.pair_vec & 1);
    cvec = !CONTIG && std::is_same<T, float>::value && (a.pair_vec & 2);
    t = t_;
    line = line_;
    valid = cl < limit;
    // a padding line is clamped to the last line before `limit` (line 0 of
    // the first plane when there is none): its addresses stay in bounds, so
    // that without PRED its loads need no predicate
    if (!valid) {
      if (limit > 0) {
        cl = limit - 1;
      } else {
        cl = 0;
        v = 0;
      }
    }
    if (KIND == K_C2C) {
      has1 = false;
      sb0 = CONTIG ? cl * a.s_src_l : cl + v * a.s_src_l;
      db0 = CONTIG ? cl * a.s_dst_l : cl + v * a.s_dst_l;
      if (!CONTIG && a.row_w > 0) {
        sb0 = flat_off(cl, a.row_w, a.s_src_r);
        db0 = flat_off(cl, a.row_w, a.s_dst_r);
      }
      sb1 = sb0;
      db1 = db0;
    } else {
      const long long r0 = 2 * cl, r1 = 2 * cl + 1;
      has1 = r1 < a.real_lines;
      sb0 = CONTIG ? r0 * a.s_src_l : r0 + v * a.s_src_l;
      sb1 = CONTIG ? r1 * a.s_src_l : r1 + v * a.s_src_l;
      db0 = CONTIG ? r0 * a.s_dst_l : r0 + v * a.s_dst_l;
      db1 = CONTIG ? r1 * a.s_dst_l : r1 + v * a.s_dst_l;
      if (!CONTIG && a.row_w > 0) {
        sb0 = flat_off(r0, a.row_w, a.s_src_r);
        sb1 = flat_off(r1, a.row_w, a.s_src_r);
        db0 = flat_off(r0, a.row_w, a.s_dst_r);
        db1 = flat_off(r1, a.row_w, a.s_dst_r);
      }
    }
  }
  // Start of flat line u of a plane whose rows of w lines lie `pitch`
  // elements apart (u < 2^31: the engine bounds the lines of a plane).
  __device__ __forceinline__ static long long flat_off(long long u, int w, long long pitch) {
    const unsigned q = (unsigned)u / (unsigned)w;
    return (long long)q * pitch + ((unsigned)u - q * (unsigned)w);
  }

  // One pad slot every 16 entries: 8-byte values are served per half-warp
  // and 16-byte values per quarter-warp, and this spacing keeps radix-16
  // strided writes on distinct banks within each of them.
  __device__ __forceinline__ int sidx(int n) const {
    const int a = CONTIG ? line * N + n : n * L + line;
    return a + (a >> 4);
  }
  // Slot of point n + 16 c is sidx(n) + c * sstep16() (n >= 0): 16 c points
  // span 16 c entries (contiguous) or 16 c L (strided), plus one pad slot per
  // 16 entries.
  __device__ __forceinline__ int sstep16() const { return CONTIG ? 17 : 17 * L; }
  // slot of point n of any line of the tile (same layout as sidx)
  __device__ __forceinline__ int sidx_at(int line_, int n) const {
    const int a = CONTIG ? line_ * N + n : n * L + line_;
    return a + (a >> 4);
  }
  __device__ __forceinline__ C twiddle(int e) const { return __ldg(tw + e); }

  // Point n of the complex line this thread works on, as the forward
  // transform must see it.
  // Strided FP32 loads ask L2 to fetch 256-byte blocks: a CTA reads 64-128
  // bytes of each row and its neighbours read the rest of the block soon
  // after (about 1 % faster strided passes on GB300; contiguous lines gain
  // nothing).
  template <typename V> __device__ __forceinline__ static V ld(const V* p) {
    if constexpr (!CONTIG && !CG && std::is_same<V, float2>::value) {
      float2 r;
      asm volatile("ld.global.L2::256B.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
      return r;
    } else if constexpr (!CONTIG && !CG && std::is_same<V, float>::value) {
      float r;
      asm volatile("ld.global.L2::256B.f32 %0, [%1];" : "=f"(r) : "l"(p));
      return r;
    } else if constexpr (CG) {
      return __ldcg(p);
    } else {
      return *p;
    }
  }

  __device__ __forceinline__ static float4 ld4(const float4* p) {
    if constexpr (CG) return __ldcg(p);
    else return *p;
  }

  __device__ __forceinline__ C gload(int n) const {
    if (PRED && !valid) return cmk<C>(T(0), T(0));
    if (KIND == K_C2C) {
      if (!GB_SRC(sb0 + n * ssn, 1)) return cmk<C>(T(0), T(0));
      C x = ld(reinterpret_cast<const C*>(src) + sb0 + n * ssn);
      if (inverse) x.y = -x.y;
      return x;
    } else if (KIND == K_R2C) {
      const T* s = reinterpret_cast<const T*>(src);
      if (!CONTIG && pvec && has1) {
        if (!GB_SRC(sb0 + n * ssn, 2)) return cmk<C>(T(0), T(0));
        return ld(reinterpret_cast<const C*>(s + sb0 + n * ssn));
      }
      const T re = GB_SRC(sb0 + n * ssn, 1) ? ld(s + sb0 + n * ssn) : T(0);
      const T im = (has1 && GB_SRC(sb1 + n * ssn, 1)) ? ld(s + sb1 + n * ssn) : T(0);
      return cmk<C>(re, im);
    } else {
      // Hermitian extension of both half spectra (src/fft_generic.f90:318-330)
      const C* s = reinterpret_cast<const C*>(src);
      const bool low = 2 * n <= N;
      const int m = low ? n : N - n;
      C x1 = GB_SRC(sb0 + m * ssn, 1) ? ld(s + sb0 + m * ssn) : cmk<C>(T(0), T(0));
      C x2 = (has1 && GB_SRC(sb1 + m * ssn, 1)) ? ld(s + sb1 + m * ssn) : cmk<C>(T(0), T(0));
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

  // Point n of this line from a tile that a copy engine filled in natural
  // order (slot sidx(n)), as the forward transform must see it.
  __device__ __forceinline__ C sload(const C* S, int n) const {
    C x = S[sidx(n)];
    if (KIND == K_C2C && inverse) x.y = -x.y;
    return x;
  }

  __device__ __forceinline__ void gstore(int n, C v) const {
    if (!valid) return;
    if (KIND == K_C2C) {
      if (inverse) v.y = -v.y;
      if (GB_DST(db0 + n * dsn, 1)) reinterpret_cast<C*>(dst)[db0 + n * dsn] = v;
    } else if (KIND == K_C2R) {
      T* d = reinterpret_cast<T*>(dst);
      if (!CONTIG && pvec && has1) {
        if (GB_DST(db0 + n * dsn, 2)) *reinterpret_cast<C*>(d + db0 + n * dsn) = cmk<C>(v.x, -v.y);
        return;
      }
      if (GB_DST(db0 + n * dsn, 1)) d[db0 + n * dsn] = v.x;
      if (has1 && GB_DST(db1 + n * dsn, 1)) d[db1 + n * dsn] = -v.y;
    }
  }

  // c2r input staging: the two half spectra of this line pair (n/2+1 points
  // each) in shared memory, interleaved: pair slot j holds (X1[j], X2[j]),
  // so that the Hermitian gather reads both with one 16-byte load (FP32).
  struct alignas(16) Pair {
    C a, b;
  };
  __device__ __forceinline__ int sstage(int j) const {
    return CONTIG ? line * (N / 2 + 1) + j : j * L + line;
  }
  // NN, TPL: the line length and threads per line, known at compile time so
  // that every load is issued before the first shared-memory store.
  template <int NN, int TPL>
  __device__ __forceinline__ void stage_c2r(C* S) const {
    constexpr int h = NN / 2 + 1;
    constexpr int J = (h + TPL - 1) / TPL;
    const C* s = reinterpret_cast<const C*>(src);
    Pair* P = reinterpret_cast<Pair*>(S);
    C a[J], b[J];
#pragma unroll
    for (int i = 0; i < J; ++i) {
      const int j = t + i * TPL;
      const bool in = (!PRED || valid) && j < h;
      if constexpr (std::is_same<T, float>::value) {
        if (cvec && has1) {  // the pair's two complex values side by side
          const float4 q = (in && GB_SRC(sb0 + j * ssn, 2)) ? ld4(reinterpret_cast<const float4*>(s + sb0 + j * ssn))
                                                           : make_float4(0.f, 0.f, 0.f, 0.f);
          a[i] = cmk<C>(q.x, q.y);
          b[i] = cmk<C>(q.z, q.w);
          continue;
        }
      }
      a[i] = (in && GB_SRC(sb0 + j * ssn, 1)) ? ld(s + sb0 + j * ssn) : cmk<C>(T(0), T(0));
      b[i] = (in && has1 && GB_SRC(sb1 + j * ssn, 1)) ? ld(s + sb1 + j * ssn) : cmk<C>(T(0), T(0));
    }
#pragma unroll
    for (int i = 0; i < J; ++i) {
      const int j = t + i * TPL;
      if (j < h) P[sstage(j)] = Pair{a[i], b[i]};
    }
  }
  // Point n of the complex line z = x1 + i x2 built from the staged half
  // spectra by the Hermitian extension (src/fft_generic.f90:318-330),
  // conjugated for the inverse-by-conjugation.
  __device__ __forceinline__ C sgather_c2r(const C* S, int n) const {
    const bool low = 2 * n <= N;
    const int m = low ? n : N - n;
    const Pair p = reinterpret_cast<const Pair*>(S)[sstage(m)];
    C x1 = p.a, x2 = p.b;
    if (!low) {
      x1.y = -x1.y;
      x2.y = -x2.y;
    }
    if (n == 0 || 2 * n == N) {  // c2r ignores Im of the DC and Nyquist bins
      x1.y = T(0);
      x2.y = T(0);
    }
    return cmk<C>(x1.x - x2.y, -(x1.y + x2.x));
  }

  // r2c output in pair slots (the c2r staging layout): slot k holds
  // (Z[k], Z[n-k]) for k <= n/2, so that the split below reads both with one
  // 16-byte load (FP32).  put_r2c stores point j of the transformed line.
  __device__ __forceinline__ void put_r2c(C* S, int j, C v) const {
    Pair* P = reinterpret_cast<Pair*>(S);
    if (2 * j <= N) {
      P[sstage(j)].a = v;
      if (j == 0 || 2 * j == N) P[sstage(j)].b = v;
    } else {
      P[sstage(N - j)].b = v;
    }
  }
  __device__ __forceinline__ void store_r2c_pairs(const C* S) const {
    if (!valid) return;
    const Pair* P = reinterpret_cast<const Pair*>(S);
    C* d = reinterpret_cast<C*>(dst);
    const T h = T(0.5);
#pragma unroll 1
    for (int k = t; 2 * k <= N; k += tpl) {
      const Pair p = P[sstage(k)];
      const C zk = p.a, zm = p.b;
      if (GB_DST(db0 + k * dsn, 1)) d[db0 + k * dsn] = cmk<C>((zk.x + zm.x) * h, (zk.y - zm.y) * h);
      if (has1 && GB_DST(db1 + k * dsn, 1)) d[db1 + k * dsn] = cmk<C>((zk.y + zm.y) * h, (zm.x - zk.x) * h);
    }
  }
  // The same with the line length NN and its TPL threads known at compile
  // time: every iteration unrolled.
  template <int NN, int TPL>
  __device__ __forceinline__ void store_r2c_pairs_ct(const C* S) const {
    if (!valid) return;
    const Pair* P = reinterpret_cast<const Pair*>(S);
    C* d = reinterpret_cast<C*>(dst);
    const T h = T(0.5);
    constexpr int J = (NN / 2 + TPL) / TPL;
#pragma unroll
    for (int i = 0; i < J; ++i) {
      const int k = t + i * TPL;
      if (2 * k > NN) break;
      const Pair p = P[sstage(k)];
      const C zk = p.a, zm = p.b;
      const C x1 = cmk<C>((zk.x + zm.x) * h, (zk.y - zm.y) * h);
      const C x2 = cmk<C>((zk.y + zm.y) * h, (zm.x - zk.x) * h);
      if constexpr (std::is_same<T, float>::value) {
        if (cvec && has1) {  // the pair's two complex outputs side by side
          if (GB_DST(db0 + k * dsn, 2))
            *reinterpret_cast<float4*>(d + db0 + k * dsn) = make_float4(x1.x, x1.y, x2.x, x2.y);
          continue;
        }
      }
      if (GB_DST(db0 + k * dsn, 1)) d[db0 + k * dsn] = x1;
      if (has1 && GB_DST(db1 + k * dsn, 1)) d[db1 + k * dsn] = x2;
    }
  }

  // r2c output: separate the two half spectra held in shared memory,
  // X1 = (Z_k + conj Z_{n-k}) / 2, X2 = (Z_k - conj Z_{n-k}) / (2i).
  __device__ __forceinline__ void store_r2c(const C* S) const {
    if (!valid) return;
    C* d = reinterpret_cast<C*>(dst);
    const T h = T(0.5);
#pragma unroll 1
    for (int k = t; 2 * k <= N; k += tpl) {
      const C zk = S[sidx(k)], zm = S[sidx(k == 0 ? 0 : N - k)];
      if (GB_DST(db0 + k * dsn, 1)) d[db0 + k * dsn] = cmk<C>((zk.x + zm.x) * h, (zk.y - zm.y) * h);
      if (has1 && GB_DST(db1 + k * dsn, 1)) d[db1 + k * dsn] = cmk<C>((zk.y + zm.y) * h, (zm.x - zk.x) * h);
    }
  }
};

// ---------------------------------------------------------------------------
// Chained launches of the axis passes (programmatic dependent launch).
// ---------------------------------------------------------------------------
// A pass launched with launch_chained may start while the previous kernel of
// its stream finishes.  Its first action is chained_entry(): wait until that
// kernel has completed and its memory is visible (a no-op for a kernel
// launched without the attribute), then let the next chained pass begin to
// launch.  Every CTA of this grid is then resident or done, so the next
// grid's waiting CTAs cannot keep any of them from running.
__device__ __forceinline__ void chained_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

}  // namespace dev

// Launch of an axis-pass kernel that overlaps its launch with the end of the
// previous kernel in the stream; the kernel must call dev::chained_entry()
// before it touches global memory.  Measured on GB300: stream launches of
// small grids gain 5-25 % (256^3 FP32 round trip 0.142 -> 0.128 ms, 384
// per-grid launches 2.79 -> 2.12 ms), while the same launches replayed from
// a CUDA graph got slower (1.85 -> 2.03 ms), so a launch into a stream that
// is being captured stays a plain one.
template <typename... KArgs, typename... Args>
cudaError_t launch_chained(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                           Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &capture) != cudaSuccess) capture = cudaStreamCaptureStatusActive;
  cfg.attrs = attr;
  cfg.numAttrs = capture == cudaStreamCaptureStatusNone ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<Args&&>(args)...);
}

}  // namespace gbfft
