// Pack and unpack of the multi-rank pencil transposes: mem_split_* and
// mem_merge_* of src/transpose_{x_to_y,y_to_z,z_to_y,y_to_x}.f90 as one
// kernel each.
//
// A transpose between pencils on several ranks packs the local array into
// one send buffer of per-peer blocks, exchanges the buffers (ALLTOALL(V) on
// the column or row communicator: src/transpose_x_to_y.f90:96-129,
// src/transpose_y_to_z.f90:94-156), and unpacks the received blocks into
// the destination pencil.  Every pack and unpack of the reference is the
// same operation on an (n1, n2, n3) array split along one dimension d into
// blocks of widths dist[m]: block m -- the sub-array of indices
// [start_m, start_m + dist[m]) along d, in Fortran order -- sits at
// displacement disp[m] of the buffer:
//   mem_split_xy, mem_merge_yx: d = x;   mem_merge_xy, mem_split_yz,
//   mem_merge_zy, mem_split_yx: d = y;   mem_merge_yz, mem_split_zy: d = z
// (src/transpose_x_to_y.f90:266-441 and the siblings' mem_split_* /
// mem_merge_*).  The reference's GPU build runs one cudaMemcpy2D per block;
// here one launch moves every element, one thread per element (4-, 8- or
// 16-byte words: real or complex, single or double), the array side read or
// written in its own order (coalesced), the buffer side in runs of the block
// width.  Copies are bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "gbfft.h"
#include "gbfft_internal.h"

namespace gbfft {
namespace {

struct BlockArgs {
  const void* src;
  void* dst;
  long long n1, n2, n3;
  int d;        // split dimension 0, 1, 2
  int nblocks;
  int pack;     // 1: array -> buffer, 0: buffer -> array
  long long start[GBFFT_MAX_PEERS];  // 0-based first index of block m along d
  long long width[GBFFT_MAX_PEERS];
  long long disp[GBFFT_MAX_PEERS];   // element offset of block m in the buffer
};

template <typename W>
__global__ void __launch_bounds__(256) block_copy_kernel(const __grid_constant__ BlockArgs a) {
  const W* src = static_cast<const W*>(a.src);
  W* dst = static_cast<W*>(a.dst);
  const long long total = a.n1 * a.n2 * a.n3;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    long long idx[3];
    idx[0] = e % a.n1;
    const long long r = e / a.n1;
    idx[1] = r % a.n2;
    idx[2] = r / a.n2;
    // block of idx[d]: the last block starting at or before it
    const long long x = idx[a.d];
    int lo = 0, hi = a.nblocks - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.start[mid] <= x) lo = mid;
      else hi = mid - 1;
    }
    long long ext[3] = {a.n1, a.n2, a.n3};
    ext[a.d] = a.width[lo];
    idx[a.d] = x - a.start[lo];
    const long long b = a.disp[lo] + idx[0] + ext[0] * (idx[1] + ext[1] * idx[2]);
    if (a.pack) dst[b] = src[e];
    else dst[e] = src[b];
  }
}

std::atomic<int> g_sms{0};
int sm_count() {
  int v = g_sms.load();
  if (v) return v;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      v <= 0)
    v = 152;
  g_sms.store(v);
  return v;
}

// the split dimension of each pack / unpack, by transpose kind
int split_dim(int kind, bool pack) {
  switch (kind) {
    case GBFFT_X_TO_Y: return pack ? 0 : 1;
    case GBFFT_Y_TO_Z: return pack ? 1 : 2;
    case GBFFT_Z_TO_Y: return pack ? 2 : 1;
    case GBFFT_Y_TO_X: return pack ? 1 : 0;
    default: return -1;
  }
}

int run(bool pack, int kind, int is_complex, int prec, const void* src, void* dst, int n1, int n2, int n3,
        int nblocks, const int* dist, const int* disp, size_t buf_elems, void* stream) {
  const int d = split_dim(kind, pack);
  if (d < 0) return set_error(GBFFT_ERR_INVALID, "bad transpose kind");
  if (prec != GBFFT_PREC_SINGLE && prec != GBFFT_PREC_DOUBLE)
    return set_error(GBFFT_ERR_INVALID, "Invalid value for precision (4 or 8)");
  if (n1 <= 0 || n2 <= 0 || n3 <= 0 || !src || !dst || !dist || !disp)
    return set_error(GBFFT_ERR_INVALID, "bad argument");
  if (nblocks < 1 || nblocks > GBFFT_MAX_PEERS)
    return set_error(GBFFT_ERR_UNSUPPORTED, "number of peers outside 1..GBFFT_MAX_PEERS");
  const size_t esz = (is_complex ? 2 : 1) * (size_t)prec;
  if ((uintptr_t)src % esz || (uintptr_t)dst % esz)
    return set_error(GBFFT_ERR_INVALID, "array not aligned to its element size");
  BlockArgs a;
  std::memset(&a, 0, sizeof a);
  a.src = src;
  a.dst = dst;
  a.n1 = n1;
  a.n2 = n2;
  a.n3 = n3;
  a.d = d;
  a.nblocks = nblocks;
  a.pack = pack ? 1 : 0;
  const long long ext = d == 0 ? n1 : d == 1 ? n2 : n3;
  const long long plane = (long long)n1 * n2 * n3 / ext;  // elements of a unit-width block
  long long s = 0;
  for (int m = 0; m < nblocks; ++m) {
    if (dist[m] < 0 || disp[m] < 0) return set_error(GBFFT_ERR_INVALID, "negative block width or displacement");
    // every block inside the buffer: nothing is launched otherwise
    if ((unsigned long long)disp[m] + (unsigned long long)dist[m] * plane > buf_elems)
      return set_error(GBFFT_ERR_INVALID, "a block reaches past the end of the buffer");
    a.start[m] = s;
    a.width[m] = dist[m];
    a.disp[m] = disp[m];
    s += dist[m];
  }
  if (s != ext) return set_error(GBFFT_ERR_INVALID, "block widths do not add up to the split dimension");
  const long long total = (long long)n1 * n2 * n3;
  const long long want = (total + 255) / 256;
  const unsigned grid = (unsigned)std::max(1ll, std::min(want, (long long)sm_count() * 16));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (esz == 4) block_copy_kernel<unsigned><<<grid, 256, 0, st>>>(a);
  else if (esz == 8) block_copy_kernel<uint2><<<grid, 256, 0, st>>>(a);
  else block_copy_kernel<uint4><<<grid, 256, 0, st>>>(a);
  add_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GBFFT_ERR_CUDA, cudaGetErrorString(e));
  return GBFFT_OK;
}

}  // namespace
}  // namespace gbfft

extern "C" int gbfft_transpose_pack(int kind, int is_complex, int prec, const void* d_src, int n1, int n2, int n3,
                                    int npeers, const int* dist, const int* disp, void* d_send, size_t send_elems,
                                    void* stream) {
  return gbfft::run(true, kind, is_complex, prec, d_src, d_send, n1, n2, n3, npeers, dist, disp, send_elems, stream);
}

extern "C" int gbfft_transpose_unpack(int kind, int is_complex, int prec, const void* d_recv, int n1, int n2, int n3,
                                      int npeers, const int* dist, const int* disp, size_t recv_elems, void* d_dst,
                                      void* stream) {
  return gbfft::run(false, kind, is_complex, prec, d_recv, d_dst, n1, n2, n3, npeers, dist, disp, recv_elems, stream);
}
