// TMA-staged strided c2c passes (FP32 y passes; lines of 1024 points).
//
// The one-shot strided kernel (fft_fast.cuh) holds its whole tile in
// registers from its global loads to its first exchange, so an SM has at
// most two tiles of loads in flight, and its 8-byte global stores queue up
// behind one another at the end of every tile.  Here the transform itself
// issues no global memory instruction at all:
//  * one persistent CTA per SM walks the tiles blockIdx.x, + gridDim.x, ...
//    (a tile: L neighbouring lines of one plane, L * n * 8 = 64 KB);
//  * a producer warp moves every tile with bulk tensor copies
//    (cp.async.bulk.tensor.3d, one per 256 points of the line): loads into
//    one of three shared-memory buffers, completed on that buffer's `full`
//    mbarrier, and, once the consumers have left the transformed tile in
//    the buffer and arrived on its `empty` mbarrier, stores back to global
//    memory from it before the buffer takes the tile three ahead -- so two
//    tiles are loading while one is transformed;
//  * the consumer threads run the power-of-two plan's stages in place in the
//    buffer: stage 0 reads point n of line l at n * L + l (the copy's dense
//    layout), the exchanges between stages use the same slots with bit 3
//    of the slot XOR-ed with the bit of n that separates the half-warp's two
//    butterflies (L = 8; with 16 or 32 lines a half-warp holds one point of
//    16 lines and needs none), which keeps every stage free of bank
//    conflicts without pad slots, and the last stage writes the dense
//    layout again for the store; the stage-major twiddles sit in shared
//    memory;
//  * every wait on an mbarrier is bounded (about two seconds of clock); a
//    thread that gives up records GBFFT_ERR_TIMEOUT in the engine's status
//    word, and the producer waits (bounded) for its copies still in flight
//    and for its stores before the CTA ends.
//
// Where it pays (GB300, FP32): y passes of 1024 points, whose one-shot tiles
// are 64-byte row segments held in 128 registers a thread -- 0.645 ms
// against 0.82 for a 1024 x 1024 x 512 grid's y pass (rows padded to 64
// bytes), 6.7 TB/s.  The same kernel on 512- and 256-point lines and on z
// passes (every row of a tile in another plane) measured slower than the
// one-shot kernel, which already streams those at 6.3-6.8 TB/s, so the
// engine uses it for 1024-point y passes only.
//
// The tensor maps describe the source and destination arrays as
// (u, n, v) = (line, point, plane) -- y passes -- or as (u, v, n) when v has
// the smaller stride (z passes, whose v is the row), with byte strides that
// must be multiples of 16: rows of an even number of complex values (the
// padded work area, or the rows of an even-length axis), both arrays
// 16-byte aligned.  Tiles start at u = k L, so the innermost copy
// coordinate is a multiple of 64 bytes.  Lines past the last one read as
// zeros and are clipped from the stores (the tensor maps' bounds).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cstring>
#include <mutex>

#include "fft_fast.cuh"

namespace gbfft {
namespace tma {

using namespace dev;

struct TmaParams {
  CUtensorMap src;    // source array as (u, n, v), or (u, v, n) when v is
                      // the smaller stride (z passes: v is the row)
  CUtensorMap dst;    // destination array, the same dimension order
  PassArgs a;
  long long tiles_u;  // tiles along u
  long long tiles;    // tiles of the pass
  int v_inner;        // 1: the maps' dimensions are (u, v, n)
};

// Lines of one 64 KB tile, by line length.
__host__ __device__ constexpr int tma_lines(int n) { return 8192 / n; }
constexpr int kStages = 3;
constexpr int kBoxRows = 256;                    // points of a line one tensor copy moves
constexpr long long kWaitCycles = 4000000000ll;  // about two seconds at 2 GHz
constexpr int kConsBarrier = 1;                  // named barrier of the consumer threads

__host__ __device__ constexpr size_t tma_buf_bytes(int n) { return (size_t)n * tma_lines(n) * sizeof(float2); }
__host__ __device__ constexpr size_t tma_smem_bytes(int n) {
  // buffers, stage-major twiddles (n - 1 entries, rounded up), mbarriers
  return kStages * tma_buf_bytes(n) + (size_t)n * sizeof(float2) + 64;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for the phase with this parity to complete, for at most kWaitCycles.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (clock64() - t0 < kWaitCycles)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int c0, int c1, int c2) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory reads of every committed store are done
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// every committed store is done (its global writes performed)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
template <int COUNT>
__device__ __forceinline__ void cons_sync() {
  asm volatile("bar.sync %0, %1;" ::"n"(kConsBarrier), "n"(COUNT) : "memory");
}
// consumer-wide OR of a predicate (and a barrier)
template <int COUNT>
__device__ __forceinline__ bool cons_any(bool q) {
  unsigned r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "barrier.cta.red.or.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((unsigned)q), "n"(kConsBarrier), "n"(COUNT)
      : "memory");
  return r != 0;
}

// Exchange slot of point n of line `line`: dense (n * L + line) with bit 3
// flipped by bit SB of n when L = 8 (SB = log2 of the first radix).
template <int L, int SB>
__device__ __forceinline__ int xslot(int n, int line) {
  const int a = n * L + line;
  if constexpr (L == 8) return a ^ (((n >> SB) & 1) << 3);
  else return a;
}

// Stage S of plan P on the tile in buffer B (in place), thread t of line
// `line`: stage 0 reads the dense layout, the last stage writes it.
template <class P, int S, int L, int COUNT>
__device__ __forceinline__ void run_stages(float2* B, const float2* tws, int t, int line, bool inv,
                                           float2 (&v)[P::E]) {
  constexpr int N = P::N, E = P::E, TPL = P::TPL;
  if constexpr (S < P::NST) {
    constexpr int R = P::radix(S), NS = P::ns(S), MB = E / R, NB = N / R;
    constexpr bool LAST = S == P::NST - 1;
    constexpr int SB = ilog2c(P::radix(0));
#pragma unroll
    for (int m = 0; m < MB; ++m)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = t + m * TPL + r * NB;
        if constexpr (S == 0) {
          float2 x = B[n * L + line];
          if (inv) x.y = -x.y;
          v[m * R + r] = x;
        } else {
          v[m * R + r] = B[xslot<L, SB>(n, line)];
        }
      }
    // every point of the tile is in registers before this stage's outputs
    // overwrite the buffer
    cons_sync<COUNT>();
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int b = t + m * TPL;
      const int k = b % NS;
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[m * R + r] = cmul(v[m * R + r], tws[(NS - 1) + (r - 1) * NS + k]);
      }
      dftg<R>(&v[m * R]);
    }
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int b = t + m * TPL;
      const int k = b % NS;
      const int base = (b - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = base + r * NS;
        if constexpr (LAST) {
          float2 x = v[m * R + r];
          if (inv) x.y = -x.y;
          B[n * L + line] = x;
        } else {
          B[xslot<L, SB>(n, line)] = v[m * R + r];
        }
      }
    }
    if constexpr (!LAST) cons_sync<COUNT>();
    run_stages<P, S + 1, L, COUNT>(B, tws, t, line, inv, v);
  }
}

// E points a thread: the axis plan's (32: two stages for 512 and 1024
// points; 16: radix-16 stages and a last one of 2, 4 or 8).
template <int N, int E>
__global__ void __launch_bounds__(tma_lines(N) * (N / E) + 32, 1)
    tma_pass_kernel(const __grid_constant__ TmaParams p) {
  using P = fast::P2Plan<N, E>;
  constexpr int L = tma_lines(N);
  constexpr int CONS = L * (N / E);  // consumer threads; one producer warp follows
  constexpr size_t kBuf = tma_buf_bytes(N);
  constexpr unsigned kTileBytes = (unsigned)kBuf;
  constexpr int kRows = N < kBoxRows ? N : kBoxRows;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float2* tws = reinterpret_cast<float2*>(smem_raw + kStages * kBuf);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + kStages * kBuf + (size_t)N * sizeof(float2));
  uint64_t* empty = full + kStages;
  const int tid = threadIdx.x;
  const long long ntiles = p.tiles;
  const long long stride = gridDim.x;
  auto buf = [&](int s) { return reinterpret_cast<float2*>(smem_raw + (size_t)s * kBuf); };
  auto coords = [&](long long tile, int j, int& c0, int& c1, int& c2) {
    c0 = (int)(tile % p.tiles_u) * L;
    const int v = (int)(tile / p.tiles_u);
    c1 = p.v_inner ? v : j;
    c2 = p.v_inner ? j : v;
  };

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CONS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  {
    const float2* tw = reinterpret_cast<const float2*>(p.a.tw);
    for (int i = tid; i < N - 1; i += blockDim.x) tws[i] = tw[i];
  }
  __syncthreads();

  if (tid >= CONS) {
    // ---- producer warp: lane 0 issues every copy ----
    if (tid != CONS) return;
    auto load = [&](long long tile, int s) {
      mbar_expect_tx(&full[s], kTileBytes);
#pragma unroll
      for (int j = 0; j < N; j += kRows) {
        int c0, c1, c2;
        coords(tile, j, c0, c1, c2);
        tma_load_3d(buf(s) + (size_t)j * L, &p.src, &full[s], c0, c1, c2);
      }
    };
    auto store = [&](long long tile, int s) {
#pragma unroll
      for (int j = 0; j < N; j += kRows) {
        int c0, c1, c2;
        coords(tile, j, c0, c1, c2);
        tma_store_3d(&p.dst, buf(s) + (size_t)j * L, c0, c1, c2);
      }
      bulk_commit();
    };
    long long count = 0;  // tiles loaded
    bool failed = false;
    for (long long tile = blockIdx.x; tile < ntiles; tile += stride, ++count) {
      const int s = (int)(count % kStages);
      const long long k = count / kStages;
      if (k > 0) {
        // the tile three back left this buffer transformed: store it, and
        // load the next one once the store has read it
        if (!mbar_wait_bounded(&empty[s], (unsigned)((k - 1) & 1))) {
          failed = true;
          break;
        }
        store(tile - kStages * stride, s);
        bulk_wait_read_all();
      }
      load(tile, s);
    }
    // store the last tiles as the consumers finish them
    const long long first = count > kStages ? count - kStages : 0;
    for (long long c = first; c < count && !failed; ++c) {
      const int s = (int)(c % kStages);
      if (!mbar_wait_bounded(&empty[s], (unsigned)((c / kStages) & 1))) {
        failed = true;
        break;
      }
      store(blockIdx.x + c * stride, s);
    }
    if (failed) {
      if (p.a.status) atomicExch(p.a.status, 1);
      // let the loads still in flight land before the CTA ends
      for (long long c = first; c < count; ++c)
        mbar_wait_bounded(&full[(int)(c % kStages)], (unsigned)((c / kStages) & 1));
    }
    bulk_wait_all();
    return;
  }

  // ---- consumers ----
  const int line = tid % L, t = tid / L;
  const bool inv = p.a.inverse != 0;
  long long i = 0;
  for (long long tile = blockIdx.x; tile < ntiles; tile += stride, ++i) {
    const int s = (int)(i % kStages);
    const bool ok = mbar_wait_bounded(&full[s], (unsigned)((i / kStages) & 1));
    if (cons_any<CONS>(!ok)) {
      if (tid == 0 && p.a.status) atomicExch(p.a.status, 1);
      return;
    }
    float2 v[E];
    run_stages<P, 0, L, CONS>(buf(s), tws, t, line, inv, v);
    // the transformed tile is in the buffer: hand it to the producer's store
    fence_proxy_async();
    mbar_arrive(&empty[s]);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

std::atomic<long long> g_tma_launches{0};

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

// Tensor map of one side (base, strides s_n / s_l in complex elements) with
// the pass's dimensions in increasing stride.
bool encode(CUtensorMap* map, const void* base, long long s_n, long long s_l, const PassArgs& a, int n, int L,
            bool v_inner) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t rows = (cuuint64_t)(n < kBoxRows ? n : kBoxRows);
  const cuuint64_t dims[3] = {(cuuint64_t)a.nlines, v_inner ? (cuuint64_t)a.nv : (cuuint64_t)n,
                              v_inner ? (cuuint64_t)n : (cuuint64_t)a.nv};
  const long long lo = v_inner ? s_l : s_n, hi = v_inner ? s_n : s_l;
  const cuuint64_t strides[2] = {(cuuint64_t)lo * sizeof(float2), (cuuint64_t)hi * sizeof(float2)};
  const cuuint32_t box[3] = {(cuuint32_t)L, v_inner ? 1u : (cuuint32_t)rows, v_inner ? (cuuint32_t)rows : 1u};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int N, int E>
cudaError_t launch_ne(const PassArgs& in, cudaStream_t stream) {
  constexpr int L = tma_lines(N);
  TmaParams p;
  std::memset(&p, 0, sizeof p);
  p.a = in;
  p.a.L = L;
  p.a.tpl = N / E;
  p.v_inner = in.s_src_l < in.s_src_n ? 1 : 0;
  if (!encode(&p.src, in.src, in.s_src_n, in.s_src_l, in, N, L, p.v_inner) ||
      !encode(&p.dst, in.dst, in.s_dst_n, in.s_dst_l, in, N, L, p.v_inner))
    return cudaErrorInvalidValue;
  p.tiles_u = (in.nlines + L - 1) / L;
  p.tiles = p.tiles_u * in.nv;
  if (p.tiles <= 0) return cudaSuccess;
  const size_t smem = tma_smem_bytes(N);
  auto kern = tma_pass_kernel<N, E>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  const long long grid = p.tiles < sm_count() ? p.tiles : sm_count();
  kern<<<(unsigned)grid, L * (N / E) + 32, smem, stream>>>(p);
  add_launches(1);
  g_tma_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

// a.tpl = n / E says which plan the axis has (the twiddle table follows it)
template <int N>
cudaError_t launch_n(const PassArgs& in, cudaStream_t stream) {
  if (in.tpl == N / 16) return launch_ne<N, 16>(in, stream);
  if constexpr (N >= 512) {
    if (in.tpl == N / 32) return launch_ne<N, 32>(in, stream);
  }
  return cudaErrorInvalidValue;
}

// One side's strides admit a tensor map: multiples of 16 bytes, the smaller
// one holding a row of lines, the larger one all of the smaller dimension.
bool side_ok(const void* base, long long s_n, long long s_l, const PassArgs& a) {
  const size_t cb = sizeof(float2);
  if ((uintptr_t)base % 16 != 0) return false;
  if ((s_n * cb) % 16 != 0 || (s_l * cb) % 16 != 0) return false;
  const bool v_inner = s_l < s_n;
  const long long lo = v_inner ? s_l : s_n, hi = v_inner ? s_n : s_l;
  const long long n_lo = v_inner ? a.nv : a.n;
  return lo >= a.nlines && hi >= lo * n_lo && (unsigned long long)hi * cb < (1ull << 40);
}

}  // namespace tma

bool tma_pass_supported(int prec_bytes, int kind, bool contiguous, const PassArgs& a) {
  if (prec_bytes != 4 || kind != K_C2C || contiguous || a.row_w != 0) return false;
  if (a.n != 1024) return false;
  if (a.tpl != a.n / 16 && a.tpl != a.n / 32) return false;
  if (a.nlines <= 0 || a.nv <= 0 || a.nlines > (1ll << 31) || a.nv > (1ll << 31)) return false;
  if (!a.src || !a.dst || !a.tw) return false;
  if ((a.s_src_l < a.s_src_n) != (a.s_dst_l < a.s_dst_n)) return false;
  if (!tma::side_ok(a.src, a.s_src_n, a.s_src_l, a) || !tma::side_ok(a.dst, a.s_dst_n, a.s_dst_l, a)) return false;
  return tma::encode_fn() != nullptr;
}

long long tma_launch_counter() { return tma::g_tma_launches.load(); }

cudaError_t launch_tma_pass(const PassArgs& a, cudaStream_t stream) {
  if (a.n != 1024) return cudaErrorNotSupported;
  return tma::launch_n<1024>(a, stream);
}

}  // namespace gbfft
