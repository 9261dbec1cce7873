// Fused x/y passes per z-plane: the two in-plane axis passes of a 3D FFT run
// in one persistent kernel, plane by plane, so that each intermediate plane
// is written to and read back from L2 instead of making a round trip
// through HBM.
//
// At one rank the reference runs the x and y transforms as two complete
// passes over the array (src/fft_common_3d.f90:27-58 and :133-159, with
// transposes that are copies in between).  Here the work of both passes is
// cut into tiles (L lines of one axis within one plane, one CTA of TH = 256
// or 512 threads a tile) and dealt out through a ticket counter in a fixed order:
//
//   slot k:  phase-1 tiles of plane k,  then phase-2 tiles of plane k - LAG
//
// Phase 1 is the axis the transform does first (x for a forward
// PHYSICAL_IN_X transform); phase 2 is the other axis.  A phase-1 tile
// publishes its completion (stores, __threadfence, then an atomic increment
// of the plane's counter); a phase-2 tile first waits until its plane's
// counter reaches the number of phase-1 tiles, then reads the plane through
// L2 only (ld.global.cg, so no stale L1 line is used).
//
// Why it cannot deadlock: a tile only ever waits for phase-1 tiles of its own
// plane, which hold earlier tickets, were therefore claimed by CTAs that are
// already running, and themselves wait for nothing.  The wait is still
// bounded: after kSpinLimit polls it records an error in the status word and
// goes on (the result is then wrong, but the GPU is not held).
//
// With LAG = 2 about five planes are in flight, a few MB of L2.
#pragma once

#include "fft_fast.cuh"
#include "fft_sync.cuh"

namespace gbfft {
namespace fused {

using namespace dev;
using fast::run_stages;

constexpr int kLag = 2;
constexpr long long kSpinLimit = 1ll << 24;  // ~1-2 s of polling

template <typename T, int KIND, bool CG, int N, int TH>
__device__ __forceinline__ void x_tile(const PassArgs& a, Cx<T>* Sm, long long plane, int item) {
  constexpr int EX = fast_points(N, true), TX = N / EX, LX = TH / TX;
  const int tid = threadIdx.x;
  const int t = tid % TX, line = tid / TX;
  const long long per_plane = a.nlines;  // complex x lines in one plane
  const long long first = plane * per_plane;
  LineCtx<T, KIND, true, CG> c;
  c.init_at(a, t, line, first + (long long)item * LX + line, 0, first + per_plane);
  Cx<T> v[EX];
  run_stages<N, EX, 0>(c, Sm, v);
  if constexpr (KIND == K_R2C) c.store_r2c_pairs(Sm);
}

template <typename T, bool CG, int N, int TH>
__device__ __forceinline__ void y_tile(const PassArgs& a, Cx<T>* Sm, long long plane, int item) {
  constexpr int EY = fast_points(N, false), TY = N / EY, LY = TH / TY;
  const int tid = threadIdx.x;
  const int line = tid % LY, t = tid / LY;
  LineCtx<T, K_C2C, false, CG> c;
  c.init_at(a, t, line, (long long)item * LY + line, plane, a.nlines);
  Cx<T> v[EY];
  run_stages<N, EY, 0>(c, Sm, v);
}

// sync[0]: ticket counter, sync[1]: error flag, sync[2 + p]: phase-1 tiles
// of plane p completed.  The host zeroes it before every launch.
// 256 threads: two CTAs an SM (at most 128 registers); 512: one.
template <typename T, int KINDX, bool XFIRST, int NX, int NY, int TH>
__global__ void __launch_bounds__(TH, TH == 256 ? 2 : 1) fused_xy_kernel(const __grid_constant__ FusedArgs f) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_ticket;
  Cx<T>* Sm = reinterpret_cast<Cx<T>*>(smem_raw);
  constexpr int LX = TH / (NX / fast_points(NX, true));
  constexpr int LY = TH / (NY / fast_points(NY, false));
  const int items_x = (int)((f.ax.nlines + LX - 1) / LX);
  const int items_y = (f.ay.nlines + LY - 1) / LY;
  const int n1 = XFIRST ? items_x : items_y;  // phase-1 tiles per plane
  const int n2 = XFIRST ? items_y : items_x;
  const long long P = f.nplanes;
  const long long lag = P < kLag ? P : kLag;
  const long long head = lag * n1;                    // slots 0..lag-1
  const long long body = (P - lag) * (long long)(n1 + n2);
  const long long total = head + body + lag * n2;     // slots P..P+lag-1
  int* sync = f.sync;

  for (;;) {
    __syncthreads();  // previous tile done with shared memory and s_ticket
    if (threadIdx.x == 0) s_ticket = (long long)atomicAdd(reinterpret_cast<unsigned int*>(sync), 1u);
    __syncthreads();
    const long long tk = s_ticket;
    if (tk >= total) break;
    bool phase1;
    long long plane;
    int item;
    if (tk < head) {
      phase1 = true;
      plane = tk / n1;
      item = (int)(tk % n1);
    } else if (tk < head + body) {
      const long long r = tk - head;
      const long long k = lag + r / (n1 + n2);
      const int o = (int)(r % (n1 + n2));
      phase1 = o < n1;
      plane = phase1 ? k : k - lag;
      item = phase1 ? o : o - n1;
    } else {
      const long long r = tk - head - body;
      phase1 = false;
      plane = (P - lag) + r / n2;
      item = (int)(r % n2);
    }
    if (phase1) {
      if constexpr (XFIRST)
        x_tile<T, KINDX, false, NX, TH>(f.ax, Sm, plane, item);
      else
        y_tile<T, false, NY, TH>(f.ay, Sm, plane, item);
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(sync + 2 + plane, 1);
    } else {
      if (threadIdx.x == 0) bounded_wait(sync + 2 + plane, n1, kSpinLimit, sync + 1, 1);
      __syncthreads();
      if constexpr (XFIRST)
        y_tile<T, true, NY, TH>(f.ay, Sm, plane, item);
      else
        x_tile<T, KINDX, true, NX, TH>(f.ax, Sm, plane, item);
    }
  }
}

template <int NX, int NY, int TH>
constexpr size_t smem_bytes(int cbytes) {
  constexpr long long ex = fast_smem_entries(NX, TH / (NX / fast_points(NX, true)));
  constexpr long long ey = fast_smem_entries(NY, TH / (NY / fast_points(NY, false)));
  return (size_t)(ex > ey ? ex : ey) * (size_t)cbytes;
}

template <typename T, int KINDX, bool XFIRST, int NX, int NY, int TH>
cudaError_t launch(const FusedArgs& f, cudaStream_t stream) {
  auto kern = fused_xy_kernel<T, KINDX, XFIRST, NX, NY, TH>;
  const size_t smem = smem_bytes<NX, NY, TH>((int)sizeof(Cx<T>));
  // the shared-memory limit is a per-device attribute: set it every launch;
  // the resident CTA count is cached per device and instantiation
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  static int grid[kMaxDevices] = {0};
  if (grid[dev] == 0) {
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TH, smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    grid[dev] = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  const size_t sync_bytes = (size_t)(f.nplanes + 2) * sizeof(int);
  e = cudaMemsetAsync(f.sync, 0, sync_bytes, stream);
  if (e != cudaSuccess) return e;
  kern<<<grid[dev], TH, smem, stream>>>(f);
  add_launches(1);
  return cudaGetLastError();
}

}  // namespace fused
}  // namespace gbfft
