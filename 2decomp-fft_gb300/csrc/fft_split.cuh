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
// Before the split each butterfly's 16 inputs are scaled by a power of two
// that brings their largest component just under 1 (exact, undone on the
// outputs), which keeps hi inside FP16's range and lo above its subnormals.
//
// The tensor cores align the terms of one product-sum to the largest and
// drop the bits below FP32's precision, so a chain of six products into one
// accumulator loses a few units in the last place at every step: the two
// hi*hi products start from zero in accumulators of their own, the four
// small corrections share a third, and the three are added with rounding.
//
// Fragment layout (PTX m16n8k16, .row.col): lane (g = lane / 4, q = lane % 4)
// holds column g of B at rows 2q, 2q+1, 2q+8, 2q+9 and, of the result, rows
// g and g+8 at columns 2q and 2q+1.  A group of 8 butterflies is one B
// matrix: on contiguous lines 8 neighbouring butterflies of one line, on
// strided lines the same butterfly of 8 neighbouring lines (so the loads of
// a group are 64-byte row segments either way).
#pragma once

#include <cuda_fp16.h>

#include "fft_common.cuh"

namespace gbfft {
namespace split {

using namespace dev;

constexpr int kThreads = 256;

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned as_u32(__half2 h) { return *reinterpret_cast<unsigned*>(&h); }

// hi / lo halves of (v0, v1), packed with v0 in the low half
__device__ __forceinline__ void split2(float v0, float v1, unsigned& hi, unsigned& lo) {
  const __half2 h = __floats2half2_rn(v0, v1);
  const float2 b = __half22float2(h);
  hi = as_u32(h);
  lo = as_u32(__floats2half2_rn(v0 - b.x, v1 - b.y));
}

// W16^m = exp(-2 pi i m / 16), m = 0..15
__device__ __forceinline__ float2 w16(int m) {
  const float c8 = 0.92387953251128675613f, s8 = 0.38268343236508977173f, r2 = 0.70710678118654752440f;
  const float cs[16] = {1.f, c8, r2, s8, 0.f, -s8, -r2, -c8, -1.f, -c8, -r2, -s8, 0.f, s8, r2, c8};
  const int mm = m & 15;
  return make_float2(cs[mm], -cs[(mm + 12) & 15]);  // sin(x) = cos(x - pi/2)
}

// A fragments of F16 (rows r = output, columns k = input) for this lane:
// real part hi / lo, imaginary part hi / lo.
struct DftFrag {
  unsigned rh[4], rl[4], ih[4], il[4];
};

__device__ __forceinline__ void dft16_frag(DftFrag& f, int lane) {
  const int g = lane >> 2, q = lane & 3;
  const int rows[4] = {g, g + 8, g, g + 8};
  const int cols[4] = {2 * q, 2 * q, 2 * q + 8, 2 * q + 8};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 w0 = w16(rows[i] * cols[i]), w1 = w16(rows[i] * (cols[i] + 1));
    split2(w0.x, w1.x, f.rh[i], f.rl[i]);
    split2(w0.y, w1.y, f.ih[i], f.il[i]);
  }
}

// One group of 8 radix-16 butterflies: x[j] is this lane's input at row
// k = 2q, 2q+1, 2q+8, 2q+9 (j = 0..3) of column g; y[i] the output at row
// (i < 2 ? g : g + 8), column 2q + (i & 1).  All lanes of the warp call it.
__device__ __forceinline__ void mma_group(const DftFrag& F, const float2 (&x)[4], float2 (&y)[4], int lane) {
  const int q = lane & 3;
  // power-of-two scale of this column's butterfly (the 4 lanes with this g)
  float m = 0.f;
#pragma unroll
  for (int j = 0; j < 4; ++j) m = fmaxf(m, fmaxf(fabsf(x[j].x), fabsf(x[j].y)));
  m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
  m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
  int e = 0;
  if (m > 0.f) frexpf(m, &e);
  e = max(-125, min(e, 126));  // keep both 2^-e and 2^e normal floats
  const float sc = ldexpf(1.f, -e), unsc = ldexpf(1.f, e);
  unsigned rh0, rl0, rh1, rl1, ih0, il0, ih1, il1;
  split2(x[0].x * sc, x[1].x * sc, rh0, rl0);
  split2(x[2].x * sc, x[3].x * sc, rh1, rl1);
  split2(x[0].y * sc, x[1].y * sc, ih0, il0);
  split2(x[2].y * sc, x[3].y * sc, ih1, il1);
  const unsigned neg = 0x80008000u;  // -Xi for the real part
  float yr[4], yi[4];
  {
    float a[4] = {0.f, 0.f, 0.f, 0.f}, b[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(a, F.rh, rh0, rh1);              // Fr Xr, hi hi
    mma16816(b, F.ih, ih0 ^ neg, ih1 ^ neg);  // -Fi Xi, hi hi
    mma16816(c, F.rh, rl0, rl1);
    mma16816(c, F.rl, rh0, rh1);
    mma16816(c, F.ih, il0 ^ neg, il1 ^ neg);
    mma16816(c, F.il, ih0 ^ neg, ih1 ^ neg);
#pragma unroll
    for (int i = 0; i < 4; ++i) yr[i] = (a[i] + b[i]) + c[i];
  }
  {
    float a[4] = {0.f, 0.f, 0.f, 0.f}, b[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(a, F.ih, rh0, rh1);  // Fi Xr, hi hi
    mma16816(b, F.rh, ih0, ih1);  // Fr Xi, hi hi
    mma16816(c, F.ih, rl0, rl1);
    mma16816(c, F.il, rh0, rh1);
    mma16816(c, F.rh, il0, il1);
    mma16816(c, F.rl, ih0, ih1);
#pragma unroll
    for (int i = 0; i < 4; ++i) yi[i] = (a[i] + b[i]) + c[i];
  }
  // each output column's scale lives in lanes 4 * column
  const float u0 = __shfl_sync(0xffffffffu, unsc, 8 * q), u1 = __shfl_sync(0xffffffffu, unsc, 8 * q + 4);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float u = (i & 1) ? u1 : u0;
    y[i] = make_float2(yr[i] * u, yi[i] * u);
  }
}

}  // namespace split
}  // namespace gbfft
