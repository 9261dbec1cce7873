// Internal declarations shared by the kernels and the host engine of the
// GB300 3D FFT backend.  Nothing here is part of the C ABI (include/gbfft.h).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

struct gbfft_engine_s;

namespace gbfft {

constexpr int kMaxStages = 16;    // radix stages of one axis plan
constexpr int kMaxE = 16;         // complex values a thread holds in one stage
constexpr int kMaxThreads = 512;  // threads in one CTA of an axis pass
constexpr int kMaxN = 8192;       // longest axis a single-tile pass supports
constexpr int kMaxGridY = 65535;  // planes (grid.y) of one strided launch
constexpr int kSmsDefault = 152;  // SMs of a GB300: the occupancy targets of small grids
constexpr int kMaxDevices = 64;   // per-device caches of launch parameters

// What one axis pass does to each line.
enum Kind : int {
  K_C2C = 0,  // complex line -> complex line
  K_R2C = 1,  // two real lines -> two half spectra (n/2+1 values each)
  K_C2R = 2,  // two half spectra -> two real lines
};

// Radices with a hand-written butterfly; any other factor runs through the
// generic direct-sum stage.
__host__ __device__ constexpr bool radix_is_special(int r) {
  return r == 2 || r == 3 || r == 4 || r == 5 || r == 7 || r == 8 || r == 16;
}

// Arguments of one batched-line FFT pass along one axis of a 3D array.
//
// A "line" is one 1D transform.  Two addressings exist:
//   contiguous (the x axis): line l starts at l * s_l, point n at + n * s_n;
//   strided   (the y and z axes): lines are indexed by (u, v) with u the
//     x index (unit stride, so a warp reads neighbouring lines in one
//     transaction) and v the remaining axis; line (u, v) starts at
//     u + v * s_l and point n sits at + n * s_n.
// For K_R2C / K_C2R two neighbouring real lines (2c, 2c+1 along l or u) are
// carried by one complex line c.  All strides are in elements of the
// array's own type (real elements for the real side of r2c/c2r).
// Chirp-z (Bluestein) tables of one axis whose length has a large prime
// factor: the length-n transform is a circular convolution of length m (a
// power of two >= 2n - 1) between the input times a chirp and the
// conjugate chirp, done as two forward m-point FFTs.  Device pointers; the
// struct itself lives on the host, in the engine's axis plan.
struct BlueTables {
  int m;                    // convolution length
  int nst;                  // radix stages of the m-point FFTs
  int radix[kMaxStages];
  const void* chirp;        // w_j = exp(-i pi j^2 / n), j < n
  const void* filt;         // FFT_m of b (b_j = conj w_j at j and m - j, 0 between), divided by m
  const void* twm;          // exp(-2 pi i k / m), k < m
};

// Axes whose largest prime factor exceeds this run the chirp-z path: a
// direct-sum stage costs that many multiply-adds a point.
constexpr int kBluePrime = 256;

struct PassArgs {
  const void* src;
  void* dst;
  const void* tw;  // n complex roots exp(-2 pi i m / n), m = 0..n-1
  long long s_src_n, s_src_l;
  long long s_dst_n, s_dst_l;
  int n;           // transform length
  int nst;         // number of radix stages (0 when n == 1)
  int L;           // complex lines per CTA
  int tpl;         // threads per line
  int inverse;     // 1: backward (+i) transform, done as conj(F(conj(x)))
  int nlines;      // complex lines along l (contiguous) or u (strided)
  int real_lines;  // r2c/c2r: real lines along l or u (may be odd)
  int nv;          // strided: extent of v (grid.y)
  int first_fused; // stage 0 reads global memory directly
  int last_fused;  // last stage writes global memory directly
  int fast;        // 1: compile-time power-of-two kernel, 2: mixed-radix kernel,
                   // 3: split-precision tensor-core kernel (mma.sync), 4:
                   // balanced non-power-of-two plan, 5: split-precision
                   // tcgen05 kernel (fft_tc.cu)
  int pair_vec;    // r2c/c2r on strided lines, bit 0: the two real lines of a
                   // pair are adjacent and aligned (read/write as one pair);
                   // bit 1 (FP32): so are their two complex lines, 16-byte
                   // aligned (one 16-byte access for both)
  int csize;       // fast == 1, one-shot: 0, or launch CTAs in clusters of
                   // csize neighbours (co-scheduled: their row segments
                   // reach DRAM together)
  int csync;       // with csize: the CTAs of a cluster start with a
                   // cluster barrier
  int row_w;       // strided, nv == 1: 0, or the lines are the positions
                   // of whole (x, y) planes taken flat: line u is point
                   // (u % row_w, u / row_w) of the plane and starts at
                   // u % row_w + (u / row_w) * s_src_r (s_dst_r), so that
                   // a tile's row segments are as aligned as the plane
  long long s_src_r, s_dst_r;
  int tma;         // strided FP32 c2c pass (fast == 1) run by the persistent
                   // kernel whose tiles arrive by bulk tensor copies
                   // (fft_tma.cu); needs tma_pass_supported()
  int* status;     // device word set to 1 when a bounded wait of the pass
                   // gave up, 2 when a check of the bounds-checked build
                   // caught an access outside an array (null: not recorded)
  long long src_elems, dst_elems;  // extents of the two arrays in elements of
                                   // each side's type (bounds-checked build)
  const BlueTables* blue;  // host-side tables of the chirp-z path (fft_long.cu),
                           // null unless the axis runs it; never read on the device
  int radix[kMaxStages];
};

// Power-of-two lengths with a compile-time-planned kernel (fft_fast.cuh):
// 16 points per thread, n / 16 threads per line.
__host__ __device__ constexpr bool fast_length(int n) {
  return n >= 16 && n <= 4096 && (n & (n - 1)) == 0;
}
// Radix plan of the power-of-two kernel, for E points per thread.  E = 32
// (strided y/z lines of length 512 or 1024): two stages, 32 x (n/32), one
// exchange.  E = 16 (the default), 8 or 4: radix-E stages, then one stage
// of the remaining factor.  E = 8 (lines of at most 256 points) and E = 4
// (at most 128) give short lines more threads, for grids too small to
// fill the GPU at 16 points a thread.
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }
__host__ __device__ constexpr int fast_points(int n, bool contiguous) {
  return (!contiguous && (n == 512 || n == 1024)) ? 32 : 16;
}
// Points per thread the power-of-two kernel offers for length n.
__host__ __device__ constexpr bool fast_e_ok(int n, int e) {
  return n >= 16 && n <= 4096 && (n & (n - 1)) == 0 &&
         (e == 16 || (e == 32 && (n == 512 || n == 1024)) || (e == 8 && n <= 256) || (e == 4 && n <= 128));
}
// Lengths with more than one power-of-two plan.
__host__ __device__ constexpr bool fast_has_alt(int n) {
  return n == 512 || n == 1024 || (n >= 16 && n <= 256 && (n & (n - 1)) == 0);
}
__host__ __device__ constexpr int fast_nst(int n, int e) {
  return e == 32 ? 2 : ilog2c(n) / ilog2c(e) + (ilog2c(n) % ilog2c(e) ? 1 : 0);
}
__host__ __device__ constexpr int fast_radix(int n, int e, int s) {
  return e == 32 ? (s == 0 ? 32 : n / 32)
                 : (s < ilog2c(n) / ilog2c(e) ? e : (1 << (ilog2c(n) % ilog2c(e))));
}
// Thread limits of the power-of-two kernel, launched with one CTA per SM
// guaranteed: 16 points a thread at most 64 registers (1024 threads, FP32),
// 32 points a thread at most 128 (512 threads).  Smaller tiles of the same
// kernel still run several CTAs per SM.
constexpr int kFastMaxThreadsF32 = 1024;
constexpr int kFastMaxThreadsF64 = 256;
// Mixed-radix lengths with a compile-time-planned kernel (fft_mixed.cuh):
// n = R0 * R1, R0 <= R1 <= 32, the most balanced such split.
__host__ __device__ constexpr int mixed_r0(int n) {
  int best = 0;
  for (int a = 2; a <= 32; ++a)
    if (n % a == 0 && n / a <= 32 && a <= n / a) best = a;
  return best;
}
__host__ __device__ constexpr bool mixed_length(int n) {
  return n == 48 || n == 96 || n == 192 || n == 210 || n == 243 || n == 270 || n == 360 ||
         n == 384 || n == 400;
}
cudaError_t launch_mixed_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);
// Non-power-of-two lengths with a balanced compile-time plan (fft_gen.cuh,
// fast::GenPlan): E points a thread, n / E threads a line.
__host__ __device__ constexpr bool gen_length(int n) {
  return n == 243 || n == 270 || n == 360 || n == 384 || n == 400;
}
__host__ __device__ constexpr int gen_points(int n) {
  return n == 243 ? 9 : (n == 270 || n == 360) ? 30 : n == 384 ? 24 : n == 400 ? 20 : 0;
}
// the plan's radices, stage by stage (0 after the last)
__host__ __device__ constexpr int gen_radix(int n, int s) {
  return n == 243 ? (s < 2 ? 9 : s == 2 ? 3 : 0)
       : n == 270 ? (s == 0 ? 15 : s == 1 ? 6 : s == 2 ? 3 : 0)
       : n == 360 ? (s == 0 ? 10 : s < 3 ? 6 : 0)
       : n == 384 ? (s < 2 ? 8 : s == 2 ? 6 : 0)
       : n == 400 ? (s < 2 ? 20 : 0) : 0;
}
// thread limit: E <= 16 at most 64 registers (1024 threads, FP32), more
// points at most 128 (512 threads); FP64 256 threads
__host__ __device__ constexpr int gen_max_threads(int e, int prec_bytes) {
  return prec_bytes == 8 ? 256 : (e <= 16 ? 1024 : 512);
}
cudaError_t launch_gen_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);
cudaError_t launch_gen_f64(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);
// Split-precision tensor-core passes (fft_split.cuh): FP32 lines of 256,
// 512, 1024 points, 256-thread CTAs of split_lines_per_cta lines.
bool split_length(int n);
int split_lines_per_cta(int n, bool contiguous);
cudaError_t launch_split_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);
cudaError_t launch_mixed_f64(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);

// Thread limit of the power-of-two kernel for E points a thread.
__host__ __device__ constexpr int fast_max_threads(int e, int prec_bytes) {
  return e == 32 ? (prec_bytes == 4 ? 512 : 256) : (prec_bytes == 4 ? kFastMaxThreadsF32 : kFastMaxThreadsF64);
}
// Shared-memory entries of one power-of-two tile of L lines: the exchange
// buffer, or for c2r the staged half spectra (n/2+1 per real line).
__host__ __device__ constexpr long long fast_smem_entries(int n, int L) {
  // rounded up to an even count: buffers laid end to end stay 16-byte
  // aligned (the c2r staging reads 16-byte pairs)
  return ((long long)(n + 2) * L + (((long long)(n + 2) * L) >> 4) + 2) & ~1ll;
}

cudaError_t launch_fast_f32_c2c(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);
cudaError_t launch_fast_f32_real(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);
cudaError_t launch_fast_f64_c2c(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);
cudaError_t launch_fast_f64_real(int kind, bool contiguous, const PassArgs& a, cudaStream_t s);

// The x and y passes of one z-plane run by one fused kernel
// (fft_fused.cuh): ax holds the x pass with ax.nlines = complex x lines per
// plane, ay the y pass (ay.nlines = columns, ay.nv = planes).
struct FusedArgs {
  PassArgs ax;
  PassArgs ay;
  long long nplanes;
  int* sync;    // nplanes + 2 ints: ticket, error flag, per-plane counters
  int threads;  // threads per CTA: 256 or 512 (ax.L, ay.L follow from it)
};

// True when a fused x/y kernel exists for these lengths (x first or y
// first, x kind K_C2C / K_R2C / K_C2R).
bool fused_supported(int prec_bytes, int kindx, bool x_first, int nx, int ny);
// Default threads per CTA of the fused kernel (a tile of L = threads / (n / E)
// lines).
constexpr int kFusedThreads = 256;
// Enqueue a fused x/y pass (zeroes f.sync first).
cudaError_t launch_fused(int prec_bytes, int kindx, bool x_first, const FusedArgs& f, cudaStream_t stream);

// ---- batches: every pass of many grids in one persistent launch ----------
constexpr int kBatchThreads = 256;
// Points a thread of the batch kernel's power-of-two plans (lines of 32..256
// points).  16: with 8 (half the points a tile, more tiles resident per SM)
// the 64-grid batch measured 2.45 ms a forward + backward step against 1.94.
__host__ __device__ constexpr int batch_points(int) { return 16; }
struct BatchDesc {
  PassArgs a;       // a.L = tile lines + 1 (shared-memory layout lines)
  int code;         // 2 * kind + (strided ? 1 : 0)
  int dep;          // descriptor that must be complete first, or -1
  long long lines;  // complex lines of the pass (contiguous) or nu * nv (strided)
  long long nu;     // strided: lines along u (x)
};
// Line lengths the batch kernel runs: 32, 48, 64, 96, 128, 192, 256.
bool batch_length(int n);
// Lines one 256-thread tile holds for a length and contiguity.
int batch_tile_lines(int n, bool contiguous);
cudaError_t launch_batch_f32(const BatchDesc* d_desc, const long long* d_prefix, int ndesc, int* d_sync,
                             long long sync_ints, cudaStream_t stream);

// Self-test of the bounded inter-CTA wait: d_words[0] is the counter,
// d_words[1] receives 1 when the wait gave up.
cudaError_t launch_wait_selftest(int* d_words, int need, long long limit, cudaStream_t stream);

// The unfused passes an engine would run for r2c (which = 0) or c2r
// (which = 1) between the given arrays (the engine's pipeline, without
// launching anything).
struct PassInfo {
  PassArgs a;
  int kind;
  bool contiguous;
};
int engine_precision(struct ::gbfft_engine_s* e);
int engine_passes(struct ::gbfft_engine_s* e, int which, const void* in, void* out, PassInfo* out_passes,
                  int max_passes, int* n);

// Shared memory the runtime-planned pass needs for L lines of length n
// (two padded buffers); the power-of-two pass needs half of it.
size_t pass_smem_bytes(int prec_bytes, int n, int L);

// One real-to-real pass along an axis (dtt.cu): the window of n points
// starting at point `off` of every line is transformed by kind 1..8
// (DCT-I..IV, DST-I..IV) through a complex FFT of length M.
struct DttArgs {
  const void* src;   // real array the window is read from
  void* dst;         // real array it is written to (may be src)
  long long sn;      // element stride between points of a line
  long long sl;      // contiguous: line stride; strided: stride of v
  long long nlines;  // contiguous: lines; strided: extent of u (x positions)
  int nv;            // strided: extent of v (grid.y)
  int naxis;         // points on the axis (copied through outside the window)
  int off, n;        // window: first point, length
  int kind;          // 1..8
  int M;             // FFT length of the extension
  int nst;           // radix stages of M
  int radix[kMaxStages];
  const void* tw;    // exp(-2 pi i m / M), m < M
  const void* twf;   // power-of-two M: stage-major table of the 16-point plan,
                     // which runs instead of the runtime plan (null: runtime plan)
  const void* w4;    // exp(-2 pi i m / (4 n)), m < n
  double c0x, c0y;   // exp(-i pi / (4 n))
  int L, tpl;        // lines a CTA, threads a line
};
size_t dtt_smem_bytes(int prec_bytes, int M, int L);
// power-of-two extension lengths with a compile-time plan for the r2r pass
__host__ __device__ constexpr bool dtt_fast_length(int M) { return M >= 32 && M <= 2048 && (M & (M - 1)) == 0; }
// Extension lengths with the compile-time two-stage plan M = R0 * R1
// (mixed_r0): 126 = 9 * 14 and 510 = 17 * 30, the default windows of every
// kind on axes of 64 and 256 points (FP32; the engine keeps FP64 on the
// runtime plan).
__host__ __device__ constexpr bool dtt_mixed_length(int M) { return M == 126 || M == 510; }
cudaError_t launch_dtt_pass(int prec_bytes, bool contiguous, const DttArgs& a, cudaStream_t stream);

// TMA-staged strided c2c passes (fft_tma.cu): FP32 lines of 1024 points
// whose source and destination rows and planes lie multiples of 16 bytes
// apart and start 16-byte aligned, on the axis's own compile-time plan
// (a.tpl = n / 16 or n / 32; the stage-major twiddle table is the axis's).
bool tma_pass_supported(int prec_bytes, int kind, bool contiguous, const PassArgs& a);
cudaError_t launch_tma_pass(const PassArgs& a, cudaStream_t stream);
long long tma_launch_counter();

// Split-precision strided c2c passes of 1024 FP32 points on tcgen05 with
// TMEM accumulators (fft_tc.cu): a.fast == 5, a.tw the n-root table,
// a.status the engine's status word.
bool tc_pass_supported(int prec_bytes, int kind, bool contiguous, const PassArgs& a);
cudaError_t launch_tc_pass(const PassArgs& a, cudaStream_t stream);
long long tc_launch_counter();

// Axis passes whose lines do not fit one shared-memory tile, or whose
// length has a prime factor above kBluePrime (fft_long.cu): one kernel per
// radix stage through `scratch`, which must hold two copies of the pass's
// lines -- of m points each on the chirp-z path (long_pass_scratch_bytes).
// Lines are per row (row_w = 0); a.nst / a.radix are the axis's stages,
// a.tw its n-root table, a.blue the chirp-z tables when set.
size_t long_pass_scratch_bytes(int prec_bytes, bool contiguous, const PassArgs& a);
cudaError_t launch_long_pass(int prec_bytes, int kind, bool contiguous, const PassArgs& a, void* scratch,
                             size_t scratch_bytes, cudaStream_t stream);

// Enqueue one axis pass.  prec_bytes = 4 (float) or 8 (double).
cudaError_t launch_axis_pass(int prec_bytes, int kind, bool contiguous,
                             const PassArgs& a, cudaStream_t stream);

// Enqueue an identity-layout copy of `bytes` bytes (the one-rank transpose).
cudaError_t launch_copy(const void* src, void* dst, size_t bytes,
                        cudaStream_t stream);

// Every device allocation of the library: cudaMalloc, unless a test armed
// gbfft_debug_fail_alloc for this one (then cudaErrorMemoryAllocation,
// nothing allocated).
cudaError_t dev_malloc(void** p, size_t bytes);
// ... and every free of one (counts the live allocations)
cudaError_t dev_free(void* p);

// Record an error message for gbfft_last_error_string(); returns `code`.
int set_error(int code, const char* msg);

// Count of kernels this library has enqueued (for the benchmark's report).
long long launch_counter();
void add_launches(long long n);

}  // namespace gbfft
