// One persistent launch for every pass of a batch of independent FFT grids.
//
// The multiple-grids use of the reference (src/fft_common.f90:381-479: the
// application selects grid 1, transforms, selects grid 2, ...) runs one grid
// after another, three batched 1D passes each.  Here the passes of all grids
// are cut into tiles and run by one persistent kernel:
//   * descriptors are ordered stage by stage (pass 0 of every grid, then pass
//     1 of every grid, ...), tiles are dealt out by a ticket counter;
//   * a tile of pass p of grid g first waits until all tiles of pass p-1 of
//     grid g are done (per-descriptor completion counters); those tiles hold
//     earlier tickets, were claimed by running CTAs and wait for nothing
//     later, so the wait always ends.  It is still bounded (kSpinLimit polls,
//     then an error flag and the tile goes on);
//   * every load goes through L2 only (ld.global.cg): a pass reads what
//     another CTA of this kernel wrote.
// Each tile is one 256-thread CTA running the compile-time kernel of its
// line length: power-of-two lengths 32..256 and the mixed lengths 48, 96,
// 192.  Strided passes flatten their (u, v) lines so that small grids fill a
// tile.
#include "fft_fast.cuh"
#include "fft_sync.cuh"
#include "fft_mixed.cuh"
#include "gbfft_internal.h"

namespace gbfft {

namespace {

using namespace dev;

constexpr int kBT = kBatchThreads;
constexpr long long kSpinLimit = 1ll << 24;

// Lines of one tile: all threads that make up whole lines.
template <int TPL>
constexpr int tile_lines() {
  return kBT / TPL;
}

template <typename T, int KIND, bool CONTIG, int N>
__device__ __forceinline__ void run_tile(const BatchDesc& D, Cx<T>* Sm, long long tile) {
  constexpr bool MIXED = !((N & (N - 1)) == 0);
  constexpr int TPL = MIXED ? N / mixed_r0(N) : N / batch_points(N);
  constexpr int LE = tile_lines<TPL>();
  const int tid = threadIdx.x;
  int t, line;
  if (CONTIG) {
    t = tid % TPL;
    line = tid / TPL;
  } else {
    // strided: lines fastest across the lanes (coalesced along x)
    line = tid % LE;
    t = tid / LE;
    if (tid >= LE * TPL) {
      line = LE;  // spare threads: a padding line
      t = 0;
    }
  }
  LineCtx<T, KIND, CONTIG, true> c;
  const long long first = tile * LE;
  const long long idx = first + (line < LE ? line : 0);
  if (CONTIG) {
    c.init_at(D.a, t, line, idx, 0, line < LE ? D.lines : 0);
  } else {
    // flattened (u, v): u = idx mod nu (x index), v = idx / nu
    const long long u = idx % D.nu, v = idx / D.nu;
    c.init_at(D.a, t, line, u, v, (line < LE && idx < D.lines) ? D.nu : 0);
  }
  if constexpr (MIXED) {
    mixed::run_mixed<N>(c, Sm);
  } else {
    constexpr int E = batch_points(N);
    Cx<T> v[E];
    fast::run_stages<N, E, 0>(c, Sm, v);
    if constexpr (KIND == K_R2C) c.store_r2c_pairs(Sm);
  }
}

template <typename T, int KIND, bool CONTIG>
__device__ __forceinline__ bool dispatch_n(const BatchDesc& D, Cx<T>* Sm, long long tile) {
  switch (D.a.n) {
    case 32: run_tile<T, KIND, CONTIG, 32>(D, Sm, tile); return true;
    case 48: run_tile<T, KIND, CONTIG, 48>(D, Sm, tile); return true;
    case 64: run_tile<T, KIND, CONTIG, 64>(D, Sm, tile); return true;
    case 96: run_tile<T, KIND, CONTIG, 96>(D, Sm, tile); return true;
    case 128: run_tile<T, KIND, CONTIG, 128>(D, Sm, tile); return true;
    case 192: run_tile<T, KIND, CONTIG, 192>(D, Sm, tile); return true;
    case 256: run_tile<T, KIND, CONTIG, 256>(D, Sm, tile); return true;
    default: return false;
  }
}

// Four 256-thread CTAs per SM (at most 64 registers a thread): tiles are
// short, so occupancy hides their load / exchange / store phases.  The
// kernel spills a few hundred bytes a thread at 64 registers; the 64-grid
// forward + backward batch still measured fastest so (with one ticket a
// tile and no look-ahead: 1.94 ms, against 2.32 ms with three CTAs per SM,
// 80 registers, and 3.15 ms with two, 128 registers and no spills).
template <typename T>
__global__ void __launch_bounds__(kBT, 4)
    batch_kernel(const BatchDesc* __restrict__ desc, const long long* __restrict__ prefix, int ndesc,
                 int* sync) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned int s_ticket;
  Cx<T>* Sm = reinterpret_cast<Cx<T>*>(smem_raw);
  // Thread 0 claims each ticket one tile ahead (the atomic's latency then
  // overlaps a tile), and signals a tile's completion at the start of the
  // next one, while the other warps already load it.  A CTA's tickets only
  // grow, so its descriptor index only moves forward.  The wait stays
  // deadlock-free: the smallest unfinished ticket is always one a CTA is
  // running (a CTA holds its claimed ticket only behind a smaller one), and
  // a CTA signals its last tile before it waits for anything.
  unsigned int next = 0;
  if (threadIdx.x == 0) next = atomicAdd(reinterpret_cast<unsigned int*>(sync), 1u);
  int lo = -1;  // descriptor of the previous tile (-1: none yet)
  for (;;) {
    if (threadIdx.x == 0) s_ticket = next;
    // every thread's stores of the previous tile, and its reads of the
    // shared tile, come before this barrier
    __syncthreads();
    const long long tk = (long long)s_ticket;
    const bool more = tk < __ldg(prefix + ndesc);
    if (threadIdx.x == 0) {
      if (lo >= 0) {
        __threadfence();  // cumulative through the barrier: the whole CTA's stores
        atomicAdd(sync + 2 + lo, 1);
      }
      if (more) next = atomicAdd(reinterpret_cast<unsigned int*>(sync), 1u);
    }
    if (!more) break;
    // descriptor i with prefix[i] <= tk < prefix[i + 1]
    if (lo < 0) lo = 0;
    while (__ldg(prefix + lo + 1) <= tk) ++lo;
    const BatchDesc& D = desc[lo];
    const long long tile = tk - prefix[lo];
    if (D.dep >= 0) {
      if (threadIdx.x == 0)
        bounded_wait(sync + 2 + D.dep, (int)(prefix[D.dep + 1] - prefix[D.dep]), kSpinLimit, sync + 1, 1);
      __syncthreads();
    }
    bool ok;
    switch (D.code) {
      case 0: ok = dispatch_n<T, K_C2C, true>(D, Sm, tile); break;
      case 1: ok = dispatch_n<T, K_C2C, false>(D, Sm, tile); break;
      case 2: ok = dispatch_n<T, K_R2C, true>(D, Sm, tile); break;
      case 3: ok = dispatch_n<T, K_R2C, false>(D, Sm, tile); break;
      case 4: ok = dispatch_n<T, K_C2R, true>(D, Sm, tile); break;
      default: ok = dispatch_n<T, K_C2R, false>(D, Sm, tile); break;
    }
    if (!ok && threadIdx.x == 0) atomicExch(sync + 1, 2);
  }
}

int g_grid[kMaxDevices] = {0};  // resident CTAs of the batch kernel, per device

// One thread waits for counter[0] >= need with a poll limit (self-test of
// the bounded wait).
__global__ void wait_selftest_kernel(int* words, int need, long long limit) {
  if (threadIdx.x == 0) bounded_wait(words, need, limit, words + 1, 1);
}

}  // namespace

cudaError_t launch_wait_selftest(int* d_words, int need, long long limit, cudaStream_t stream) {
  wait_selftest_kernel<<<1, 32, 0, stream>>>(d_words, need, limit);
  add_launches(1);
  return cudaGetLastError();
}

bool batch_length(int n) {
  return n == 32 || n == 48 || n == 64 || n == 96 || n == 128 || n == 192 || n == 256;
}

int batch_tile_lines(int n, bool contiguous) {
  const bool mixed = (n & (n - 1)) != 0;
  const int tpl = mixed ? n / mixed_r0(n) : n / batch_points(n);
  (void)contiguous;
  return kBT / tpl;
}

size_t batch_smem_bytes() {
  // largest tile: lines of every supported length, plus one padding line
  long long best = 0;
  for (int n : {32, 48, 64, 96, 128, 192, 256})
    for (int c = 0; c < 2; ++c) {
      const long long e = fast_smem_entries(n, batch_tile_lines(n, c != 0) + 1);
      if (e > best) best = e;
    }
  return (size_t)best * sizeof(float2);
}

cudaError_t launch_batch_f32(const BatchDesc* d_desc, const long long* d_prefix, int ndesc, int* d_sync,
                             long long sync_ints, cudaStream_t stream) {
  auto kern = batch_kernel<float>;
  const size_t smem = batch_smem_bytes();
  // the shared-memory limit is a per-device attribute: set it every launch;
  // the resident CTA count is cached per device
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (g_grid[dev] == 0) {
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBT, smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_grid[dev] = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  e = cudaMemsetAsync(d_sync, 0, (size_t)sync_ints * sizeof(int), stream);
  if (e != cudaSuccess) return e;
  kern<<<g_grid[dev], kBT, smem, stream>>>(d_desc, d_prefix, ndesc, d_sync);
  add_launches(1);
  return cudaGetLastError();
}

}  // namespace gbfft
