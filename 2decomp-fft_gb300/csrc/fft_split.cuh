// Split-precision tensor-core axis passes (GBFFT_FORM_SPLIT), FP32 data,
// lengths 256, 512 and 1024.
//
// The radix-16 stages of the power-of-two plan (256 = 16 x 16,
// 512 = 16 x 16 x 2, 1024 = 16 x 16 x 4) run as dense DFT-matrix products
// on the tensor cores; the last radix-2/4 stage, the r2c split and the c2r
// merge stay on the CUDA cores.
//
// One warp-level mma.sync.m16n8k16 (FP16 in, FP32 accumulate) transforms 8
// butterflies: Y[16 x 8] = F16[16 x 16] X[16 x 8], F16[r][k] = W16^{rk},
// with the real and imaginary parts as separate products.  FP16 alone keeps
// 11 bits, so both operands are split, v = hi + lo with hi = fp16(v) and
// lo = fp16(v - hi) (about 22 bits together), and three of the four cross
// products are accumulated in FP32:
//     Y = Fh Xh + Fh Xl + Fl Xh        (Fl Xl, ~2^-22 relative, dropped)
// with the large and the small products in separate accumulators (see
// mma_stage16).
// Before the split each butterfly's 16 inputs are scaled by a power of two
// that brings their largest component just under 1 (exact, undone on the
// outputs), which keeps hi inside FP16's range and lo above its subnormals.
//
// Lines sit in shared memory throughout (two ping-pong buffers): a load phase
// reads global memory, every stage reads one buffer and writes the other,
// a store phase writes global memory.
#pragma once

#include <cuda_fp16.h>

#include "fft_common.cuh"

namespace gbfft {
namespace split {

using namespace dev;

constexpr int kThreads = 256;

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ unsigned pack2(__half lo_index, __half hi_index) {
  __half2 h = __halves2half2(lo_index, hi_index);
  return *reinterpret_cast<unsigned*>(&h);
}

__device__ __forceinline__ void split1(float v, __half& hi, __half& lo) {
  hi = __float2half_rn(v);
  lo = __float2half_rn(v - __half2float(hi));
}

// W16^m = exp(-2 pi i m / 16), m = 0..15
__device__ __forceinline__ float2 w16(int m) {
  const float c8 = 0.92387953251128675613f, s8 = 0.38268343236508977173f, r2 = 0.70710678118654752440f;
  const float cs[16] = {1.f, c8, r2, s8, 0.f, -s8, -r2, -c8, -1.f, -c8, -r2, -s8, 0.f, s8, r2, c8};
  const int mm = m & 15;
  return make_float2(cs[mm], -cs[(mm + 12) & 15]);  // sin(x) = cos(x - pi/2)
}

// A fragments of F16 (rows r = output, columns k = input) for this lane:
// Frh/Frl: real part hi/lo, Fih/Fil: imaginary part hi/lo, and the negated
// imaginary part for the real output.
struct DftFrag {
  unsigned rh[4], rl[4], ih[4], il[4], nih[4], nil[4];
};

__device__ __forceinline__ void dft16_frag(DftFrag& f, int lane) {
  const int g = lane >> 2, t = lane & 3;
  const int rows[4] = {g, g + 8, g, g + 8};
  const int cols[4] = {2 * t, 2 * t, 2 * t + 8, 2 * t + 8};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 w0 = w16(rows[i] * cols[i]), w1 = w16(rows[i] * (cols[i] + 1));
    __half h0, l0, h1, l1;
    split1(w0.x, h0, l0);
    split1(w1.x, h1, l1);
    f.rh[i] = pack2(h0, h1);
    f.rl[i] = pack2(l0, l1);
    split1(w0.y, h0, l0);
    split1(w1.y, h1, l1);
    f.ih[i] = pack2(h0, h1);
    f.il[i] = pack2(l0, l1);
    f.nih[i] = pack2(__hneg(h0), __hneg(h1));
    f.nil[i] = pack2(__hneg(l0), __hneg(l1));
  }
}

// One radix-16 Stockham stage on the tensor cores, shared buffer A -> B.
// Butterfly b (0 <= b < n/16) of a line reads points b + k n/16 (k = 0..15),
// multiplies by W_{16 NS}^{(b mod NS) k} (stage-major table, entry
// NS - 1 + (k - 1) NS + b mod NS), transforms, and writes point
// (b - b mod NS) 16 + b mod NS + r NS for output r.
template <int N, class Ctx>
__device__ __forceinline__ void mma_stage16(const Ctx& c, const DftFrag& F, const float2* A, float2* B, int NS,
                                            int lines) {
  constexpr int NB = N / 16;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = kThreads / 32;
  const int g = lane >> 2, t = lane & 3;
  const int groups = lines * (NB / 8);
  const int ks[4] = {2 * t, 2 * t + 1, 2 * t + 8, 2 * t + 9};
  for (int G = warp; G < groups; G += nwarps) {
    const int line = G / (NB / 8);
    const int b = (G % (NB / 8)) * 8 + g;  // this lane's butterfly (column g)
    const int kb = b & (NS - 1);
    float2 x[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      x[j] = A[c.sidx_at(line, b + ks[j] * NB)];
      if (NS > 1 && ks[j] > 0) x[j] = cmul(x[j], c.twiddle((NS - 1) + (ks[j] - 1) * NS + kb));
    }
    // power-of-two scale of this butterfly (the 4 lanes with the same g)
    float m = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) m = fmaxf(m, fmaxf(fabsf(x[j].x), fabsf(x[j].y)));
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
    int e = 0;
    if (m > 0.f) frexpf(m, &e);
    e = max(-125, min(e, 126));  // keep both 2^-e and 2^e normal floats
    const float sc = ldexpf(1.f, -e), unsc = ldexpf(1.f, e);
    __half rh[4], rl[4], ih[4], il[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      split1(x[j].x * sc, rh[j], rl[j]);
      split1(x[j].y * sc, ih[j], il[j]);
    }
    const unsigned brh[2] = {pack2(rh[0], rh[1]), pack2(rh[2], rh[3])};
    const unsigned brl[2] = {pack2(rl[0], rl[1]), pack2(rl[2], rl[3])};
    const unsigned bih[2] = {pack2(ih[0], ih[1]), pack2(ih[2], ih[3])};
    const unsigned bil[2] = {pack2(il[0], il[1]), pack2(il[2], il[3])};
    // Yr = Fr Xr - Fi Xi,  Yi = Fi Xr + Fr Xi; each as hi*hi + hi*lo + lo*hi.
    // The tensor cores align the terms of one product-sum to the largest
    // and drop the bits below FP32's precision, so a chain of six products
    // into one accumulator loses a few units in the last place at every
    // step.  The two hi*hi products start from zero in accumulators of
    // their own, the four small corrections share a third, and the three
    // are added with rounding at the end.
    float ar[4] = {0.f, 0.f, 0.f, 0.f}, br[4] = {0.f, 0.f, 0.f, 0.f}, cr[4] = {0.f, 0.f, 0.f, 0.f};
    float ai[4] = {0.f, 0.f, 0.f, 0.f}, bi[4] = {0.f, 0.f, 0.f, 0.f}, ci[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(ar, F.rh, brh);
    mma16816(br, F.nih, bih);
    mma16816(cr, F.rh, brl);
    mma16816(cr, F.rl, brh);
    mma16816(cr, F.nih, bil);
    mma16816(cr, F.nil, bih);
    mma16816(ai, F.ih, brh);
    mma16816(bi, F.rh, bih);
    mma16816(ci, F.ih, brl);
    mma16816(ci, F.il, brh);
    mma16816(ci, F.rh, bil);
    mma16816(ci, F.rl, bih);
    float yr[4], yi[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      yr[i] = (ar[i] + br[i]) + cr[i];
      yi[i] = (ai[i] + bi[i]) + ci[i];
    }
    // outputs: rows r = g, g + 8; columns (butterflies) 2t, 2t + 1; each
    // column's scale lives in lanes 4 * column
    const float u0 = __shfl_sync(0xffffffffu, unsc, 8 * t), u1 = __shfl_sync(0xffffffffu, unsc, 8 * t + 4);
    const int bq = (G % (NB / 8)) * 8;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = (i < 2) ? g : g + 8;
      const int col = 2 * t + (i & 1);
      const float u = (i & 1) ? u1 : u0;
      const int bb = bq + col;
      const int k = bb & (NS - 1);
      B[c.sidx_at(line, (bb - k) * 16 + k + r * NS)] = make_float2(yr[i] * u, yi[i] * u);
    }
  }
}

// Plain radix-R stage (the last factor 2 or 4), shared buffer A -> B.
template <int N, int R, class Ctx>
__device__ __forceinline__ void plain_stage(const Ctx& c, const float2* A, float2* B, int NS, int lines) {
  constexpr int NB = N / R;
  for (int w = threadIdx.x; w < lines * NB; w += kThreads) {
    const int line = w / NB, b = w % NB;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = A[c.sidx_at(line, b + r * NB)];
    const int k = b & (NS - 1);
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = cmul(v[r], c.twiddle((NS - 1) + (r - 1) * NS + k));
    dftp<R>(v);
#pragma unroll
    for (int r = 0; r < R; ++r) B[c.sidx_at(line, (b - k) * R + k + r * NS)] = v[r];
  }
}

}  // namespace split
}  // namespace gbfft
