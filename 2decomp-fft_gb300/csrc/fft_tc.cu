// Split-precision strided c2c passes of 1024 points on the 5th-generation
// tensor cores (tcgen05, accumulators in tensor memory); the kernel is a
// template over the line length (512 and 1024 points).
//
// A line of N = 32 Q points (Q = 32 or 16) is transformed as 32 x Q
// (j = n1 + Q n2, k = k2 + 32 k1):
//   stage A  Y[n1][k2] = sum_n2 x[n1 + Q n2] W32^(n2 k2)   GEMM columns (line, n1)
//   twiddle  Y[n1][k2] *= WN^(n1 k2)
//   stage B  X[k2 + 32 k1] = sum_n1 Y[n1][k2] WQ^(n1 k1)  Q-point DFTs
// Each stage is one dense product D = A . B, M = 64 rows of the real form
// (2k + re/im), K = 64 columns (2n + re/im), N = 128 GEMM columns: a tile
// of LT = 128 / Q lines (4 of 1024 points, 8 of 512).  Stage A's A is the
// real form of the 32-point DFT.  Stage B's is the same matrix for Q = 32
// (columns (line, k2)); for Q = 16 it is block-diagonal, two 16-point DFTs,
// and a column holds the pair k2 = 2p, 2p + 1 (columns (line, p), K = 32 h +
// 2 n1 + re/im with h = k2 & 1).  Operands are FP16 hi + lo splits of FP32
// values (about 22 bits); the products hi.hi go to one TMEM accumulator,
// the corrections hi.lo + lo.hi to another, and the epilogue adds the two
// with rounding (one accumulator for all three loses a few bits per step to
// the tensor cores' truncating alignment).  The data of a tile are scaled
// by one power of two before the split (exact; undone after stage B), so
// that hi stays inside FP16's range.
//
// Per CTA (256 threads, at most two CTAs per SM: their TMEM is 2 x 256 of
// the 512 columns), per tile: every thread loads 16 points (the next tile's
// loads are issued before this tile's MMAs), the tile maximum is reduced,
// the stage-A operand is written to shared memory in the K-major
// no-swizzle core-matrix layout, one thread issues 12 MMAs
// (tcgen05.mma.cta_group::1.kind::f16, descriptors built here) and commits
// them to an mbarrier, the epilogue reads both accumulators with
// tcgen05.ld.16x32bx2 (all 32 lanes of a warp busy on the M = 64 layout:
// rows 16q..16q+15 in lanes 32q..32q+15), exchanges re / im between lane
// pairs, twiddles and writes the stage-B operand; stage B likewise, its
// results to a padded output tile and from there to global memory.  Every
// mbarrier wait is bounded; a CTA that gives up sets the pass's status word,
// waits (bounded) once more for the MMAs it committed, frees its TMEM and
// stops (the decision is taken by the whole CTA).
//
// The DFT matrices and the twiddles come from the axis's n-root table
// exp(-2 pi i m / N).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "gbfft_internal.h"

namespace gbfft {
namespace tc {

constexpr int kCols = 128;      // GEMM columns of a tile
constexpr int kThreads = 256;
constexpr uint32_t kLBO = 128, kSBO = 1024;      // K = 64: 8 core matrices along K
constexpr int kABytes = 64 * 64 * 2;              // one DFT matrix, hi or lo: 8 KB
constexpr int kBBytes = kCols * 64 * 2;           // Bh, Bl: 16 KB each
constexpr int kOutPad = 3 * 1024;                 // padded output tile beyond Bh|Bl
constexpr int kTwEntries = 1024;                  // stage twiddles, laid out by epilogue role
constexpr int kSmem = 80 * 1024;  // requested: at most two CTAs an SM (TMEM 2 x 256 columns)
constexpr int kTmemCols = 256;
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(kCols >> 3) << 17) | ((uint32_t)(64 >> 4) << 24);
constexpr long long kWaitLimit = 2000000000ll;  // clock cycles, about a second

static_assert(4 * kABytes + 2 * kBBytes + kOutPad + kTwEntries * 8 + 64 <= kSmem, "shared memory");

// Shape of one line length: N = 32 Q points, LT lines a tile, the output
// tile's pad (slots per row of LT lines; keeps the epilogue's writes at the
// two-way minimum of 8-byte accesses)
template <int N>
struct Shape {
  static constexpr int Q = N / 32;
  static constexpr int LT = kCols / Q;
  __device__ static constexpr int pad(int p) { return Q == 32 ? (p >> 4) : 2 * (p >> 5); }
  static_assert(N == 512 || N == 1024, "tcgen05 passes: 512 or 1024 points");
  static_assert(N * LT + (Q == 32 ? N / 16 : 2 * (N / 32)) <= (2 * kBBytes + kOutPad) / 8, "output tile");
};

std::atomic<long long> g_launches{0};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, K-major, no swizzle: start, leading byte
// offset (K-adjacent core matrices), stride byte offset (8-row groups), the
// fixed 0b001 at bits 46-48
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((kLBO >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((kSBO >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
               ::"r"(d), "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
    if (clock64() - t0 > kWaitLimit) return false;
  }
}

// 16 lanes x 32 bits, two column sets: threads 0-15 columns [c, c+16),
// threads 16-31 columns [c+32, c+48)
__device__ __forceinline__ void tld16x2(uint32_t addr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.16x32bx2.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16], 32;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(addr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (row r, k) of a K-major no-swizzle operand
__device__ __forceinline__ uint32_t core_off(int r, int k) {
  return (uint32_t)((r >> 3) * kSBO + (k >> 3) * kLBO + (r & 7) * 16 + (k & 7) * 2);
}

// four complex values -> their hi and lo halves as one 16-byte chunk each
__device__ __forceinline__ void split4(const float2* z, float f, uint4& hi, uint4& lo) {
  uint32_t hw[4], lw[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float re = z[i].x * f, im = z[i].y * f;
    const __half2 h = __floats2half2_rn(re, im);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(re - hf.x, im - hf.y);
    hw[i] = *reinterpret_cast<const uint32_t*>(&h);
    lw[i] = *reinterpret_cast<const uint32_t*>(&l);
  }
  hi = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  lo = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

struct TileSpace {
  long long tiles_u, nlines;
};

// First element of line u of plane v: lines along x (unit stride) of rows
// s_l apart, or (row_w != 0) the lines of whole (x, y) planes taken flat,
// line u at (u mod row_w, u / row_w) with rows s_r apart
__device__ __forceinline__ long long line_off(long long u, long long v, int row_w, long long s_r, long long s_l) {
  return row_w ? (u % row_w) + (u / row_w) * s_r : u + v * s_l;
}

// The 16 points of thread (line l, column n1, chunk group jg) of a tile:
// n2 = 16 jg .. 16 jg + 15, points n1 + Q n2
template <int N>
__device__ __forceinline__ void load_tile(const PassArgs& a, const TileSpace& ts, long long tile, int ld_l, int ld_n1,
                                          int ld_jg, float2* x) {
  using S = Shape<N>;
  const long long ut = tile % ts.tiles_u, v = tile / ts.tiles_u;
  const long long u = ut * S::LT + ld_l;
  if (u >= ts.nlines) {
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = make_float2(0.f, 0.f);
    return;
  }
  const float2* p = static_cast<const float2*>(a.src) + line_off(u, v, a.row_w, a.s_src_r, a.s_src_l) +
                    (long long)(ld_n1 + 16 * S::Q * ld_jg) * a.s_src_n;
  const long long st = S::Q * a.s_src_n;
#pragma unroll
  for (int j = 0; j < 16; ++j) x[j] = __ldg(p + j * st);
}

// the real form of a DFT of length L as rows (2k + re/im) x columns
// (2n + re/im) entries: W_L^(nk) from the N-root table
__device__ __forceinline__ float dft_entry(const float2* tw, int N, int L, int r, int kk) {
  const int k = r >> 1, n = kk >> 1;
  const float2 wv = tw[(N / L) * ((n * k) % L)];
  return (r & 1) == (kk & 1) ? wv.x : ((r & 1) ? wv.y : -wv.y);
}

__device__ __forceinline__ void put_split(unsigned char* hi, unsigned char* lo, int r, int kk, float v) {
  const __half h = __float2half_rn(v);
  *reinterpret_cast<__half*>(hi + core_off(r, kk)) = h;
  *reinterpret_cast<__half*>(lo + core_off(r, kk)) = __float2half_rn(v - __half2float(h));
}

template <int N>
__global__ void __launch_bounds__(kThreads, 2) tc_pass_kernel(const __grid_constant__ PassArgs a, TileSpace ts) {
  using S = Shape<N>;
  constexpr int Q = S::Q, LT = S::LT;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sAh = smem;                    // 32-point DFT, hi / lo
  unsigned char* sAl = smem + kABytes;
  unsigned char* sA2h = smem + 2 * kABytes;     // stage B's matrix (Q = 16: two 16-point DFTs)
  unsigned char* sA2l = smem + 3 * kABytes;
  unsigned char* sBh = smem + 4 * kABytes;
  unsigned char* sBl = sBh + kBBytes;
  float2* sOut = reinterpret_cast<float2*>(sBh);  // padded output tile; aliases Bh|Bl and the pad
  float2* sTw = reinterpret_cast<float2*>(sBl + kBBytes + kOutPad);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sTw + kTwEntries);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
  float* wmax = reinterpret_cast<float*>(slot + 4);  // 8 warps
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const float2* tw = static_cast<const float2*>(a.tw);  // exp(-2 pi i m / N)
  const long long tiles = ts.tiles_u * (long long)a.nv;

  for (int i = t; i < 64 * 64; i += kThreads) {
    const int r = i >> 6, kk = i & 63;
    put_split(sAh, sAl, r, kk, dft_entry(tw, N, 32, r, kk));
    // stage B of Q = 16: two 16-point DFTs on the diagonal (Q = 32 reuses A)
    if (Q == 16)
      put_split(sA2h, sA2l, r, kk, (r >> 5) == (kk >> 5) ? dft_entry(tw, N, 16, r & 31, kk & 31) : 0.f);
  }
  // stage twiddles WN^(n1 k2) by epilogue role: [q][i][re/im lane][k2 & 7],
  // n1 = (16 e_c) % Q + i, k2 = 8 q + (k2 & 7)
  for (int i = t; i < kTwEntries; i += kThreads) {
    const int kk = i & 7, ec = (i >> 3) & 1, ii = (i >> 4) & 15, qq = i >> 8;
    sTw[i] = tw[((16 * ec) % Q + ii) * (8 * qq + kk)];
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *slot;
  const uint32_t bar_a = smem_u32(bar);
  uint32_t phase = 0;

  // load / convert role: line l, column n1, chunk group jg (chunks 4jg..4jg+3)
  const int ld_l = t % LT, ld_n1 = (t / LT) % Q, ld_jg = t >> 7;
  // epilogue role: TMEM quarter q (rows 16q..16q+15), column half hc, row ->
  // (k, re/im); after the re/im exchange a thread holds 16 columns
  // (n1 or p = n1_0 .. n1_0 + 15) of line e_l
  const int q = w & 3, hc = w >> 2, sl = lane & 15, hi16 = lane >> 4;
  const int e_k = 8 * q + (sl >> 1), e_c = sl & 1;
  const int e_l = (64 * hc + 32 * hi16 + 16 * e_c) / Q, n1_0 = (16 * e_c) % Q;
  const uint32_t t_row = (uint32_t)(32 * q) << 16;

  float2 x[16];
  if ((long long)blockIdx.x < tiles) load_tile<N>(a, ts, blockIdx.x, ld_l, ld_n1, ld_jg, x);
  bool ok = true;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      if (a.inverse) x[i].y = -x[i].y;
      mx = fmaxf(mx, fmaxf(fabsf(x[i].x), fabsf(x[i].y)));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) wmax[w] = mx;
    __syncthreads();  // also: the previous tile's stores have read sOut
    mx = wmax[0];
#pragma unroll
    for (int i = 1; i < 8; ++i) mx = fmaxf(mx, wmax[i]);
    int ex = 0;
    if (mx > 0.f) frexpf(mx, &ex);  // mx in [2^(ex-1), 2^ex)
    const float sc = ldexpf(1.f, 15 - ex), isc = ldexpf(1.f, ex - 15);
    {
      const int col = ld_l * Q + ld_n1;  // stage-A column (l, n1), K = 2 n2 + re/im
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        uint4 h, l;
        split4(x + 4 * m, sc, h, l);
        const uint32_t off = core_off(col, 8 * (4 * ld_jg + m));
        *reinterpret_cast<uint4*>(sBh + off) = h;
        *reinterpret_cast<uint4*>(sBl + off) = l;
      }
    }
    // the next tile's loads are in flight while this one is transformed
    if (tile + gridDim.x < tiles) load_tile<N>(a, ts, tile + gridDim.x, ld_l, ld_n1, ld_jg, x);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
#pragma unroll 1
    for (int stage = 0; stage < 2; ++stage) {
      if (t == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const bool a2 = Q == 16 && stage;
        const uint32_t ah = smem_u32(a2 ? sA2h : sAh), al = smem_u32(a2 ? sA2l : sAl);
        const uint32_t bh = smem_u32(sBh), bl = smem_u32(sBl);
#pragma unroll
        for (int s = 0; s < 4; ++s) mma_f16(tmem, make_desc(ah + 256 * s), make_desc(bh + 256 * s), s > 0);
#pragma unroll
        for (int s = 0; s < 4; ++s) mma_f16(tmem + 128, make_desc(ah + 256 * s), make_desc(bl + 256 * s), s > 0);
#pragma unroll
        for (int s = 0; s < 4; ++s) mma_f16(tmem + 128, make_desc(al + 256 * s), make_desc(bh + 256 * s), 1);
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_a)
                     : "memory");
      }
      // one thread polls the mbarrier (every thread polling would take the
      // shared-memory pipe and issue slots from the SM's other CTA); the
      // barrier releases the rest and carries the decision to all of them
      const bool got = t == 0 ? mbar_wait(bar_a, phase) : true;
      if (__syncthreads_or(!got)) {
        ok = false;
        if (t == 0) {
          if (a.status) atomicExch(a.status, 1);
          // the MMAs this CTA committed may still be writing TMEM: give them
          // a second bounded wait before the columns are freed below
          mbar_wait(bar_a, phase);
        }
        break;
      }
      phase ^= 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float v[32];
      {
        float hh[16], cc[16];
        const uint32_t base = tmem + t_row + (uint32_t)(64 * hc);
        tld16x2(base, hh);
        tld16x2(base + 128, cc);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = hh[i] + cc[i];
        tld16x2(base + 16, hh);
        tld16x2(base + 144, cc);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[16 + i] = hh[i] + cc[i];
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      }
      // the re lane keeps columns 0..15 of its 32, the im lane 16..31
      float2 y[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const float send = e_c ? v[i] : v[16 + i];
        const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
        y[i] = e_c ? make_float2(recv, v[16 + i]) : make_float2(v[i], recv);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      if (stage == 0) {
        // twiddle by WN^(n1 k2), k2 = e_k; scale by 2^-5 (stage A grew the
        // values by at most 32); write the stage-B operand
        const int col = Q == 32 ? e_l * 32 + e_k : e_l * 16 + (e_k >> 1);
        const int chunk0 = Q == 32 ? 4 * e_c : 4 * (e_k & 1);
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          float2 z[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float2 wv = sTw[(q << 8) + ((4 * m + i) << 4) + (e_c << 3) + (e_k & 7)];
            const float2 u = y[4 * m + i];
            z[i] = make_float2(u.x * wv.x - u.y * wv.y, u.x * wv.y + u.y * wv.x);
          }
          uint4 h, l;
          split4(z, 0.03125f, h, l);
          const uint32_t off = core_off(col, 8 * (chunk0 + m));
          *reinterpret_cast<uint4*>(sBh + off) = h;
          *reinterpret_cast<uint4*>(sBl + off) = l;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
      } else {
        // X[k2 + 32 k1]: Q = 32 row k1 = e_k, column k2 = n1_0 + i; Q = 16 row
        // 32 h + 2 k1 + re/im, column p = i (k2 = 2 p + h).  Unscale,
        // conjugate back, into the output tile [point][line]
        __syncthreads();  // stage B has consumed Bh|Bl, every warp has read TMEM
        const float f = 32.f * isc;
        const int kb = Q == 32 ? 32 * e_k : 32 * (8 * (q & 1) + (sl >> 1)) + (q >> 1);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int p = Q == 32 ? kb + n1_0 + i : kb + 2 * i;
          float2 z = make_float2(y[i].x * f, y[i].y * f);
          if (a.inverse) z.y = -z.y;
          sOut[p * LT + e_l + S::pad(p)] = z;
        }
        __syncthreads();
      }
    }
    if (!ok) break;
    {
      const long long ut = tile % ts.tiles_u, vv = tile / ts.tiles_u;
      const long long u = ut * LT + (t % LT);
      if (u < ts.nlines) {
        float2* d = static_cast<float2*>(a.dst) + line_off(u, vv, a.row_w, a.s_dst_r, a.s_dst_l) +
                    (long long)(t / LT) * a.s_dst_n;
        const long long st = (kThreads / LT) * a.s_dst_n;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int i = t + kThreads * j, p = i / LT;
          d[j * st] = sOut[i + S::pad(p)];
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

int sm_count() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      v <= 0)
    v = kSmsDefault;
  return v;
}

}  // namespace tc

bool tc_pass_supported(int prec_bytes, int kind, bool contiguous, const PassArgs& a) {
  // 1024-point lines.  The template also builds 512-point lines (32 x 16,
  // 8-line tiles); on the 1024 x 1024 x 512 grid's flat-plane z pass that
  // measured 1.94 ms against 1.90 for the mma.sync split kernel, so it is
  // not instantiated.
  if (prec_bytes != 4 || kind != K_C2C || contiguous || a.n != 1024) return false;
  if (a.row_w != 0 && a.nv != 1) return false;  // flat planes: one plane of lines a launch
  if (a.nlines <= 0 || a.nv <= 0 || !a.src || !a.dst || !a.tw) return false;
  return (uintptr_t)a.src % 8 == 0 && (uintptr_t)a.dst % 8 == 0;
}

long long tc_launch_counter() { return tc::g_launches.load(); }

namespace tc {
template <int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t stream) {
  TileSpace ts;
  ts.nlines = a.nlines;
  ts.tiles_u = (a.nlines + Shape<N>::LT - 1) / Shape<N>::LT;
  const long long tiles = ts.tiles_u * (long long)a.nv;
  // the shared-memory limit is a per-device attribute: set it every launch
  cudaError_t err = cudaFuncSetAttribute(tc_pass_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
  if (err != cudaSuccess) return err;
  const long long grid = std::min(tiles, 2LL * sm_count());
  tc_pass_kernel<N><<<(unsigned)grid, kThreads, kSmem, stream>>>(a, ts);
  add_launches(1);
  g_launches.fetch_add(1);
  return cudaGetLastError();
}
}  // namespace tc

cudaError_t launch_tc_pass(const PassArgs& a, cudaStream_t stream) {
  if (!tc_pass_supported(4, K_C2C, false, a)) return cudaErrorInvalidValue;
  return tc::launch_n<1024>(a, stream);
}

}  // namespace gbfft
