// Box copy between two 3D arrays: the device data movement of the halo-cell
// update (src/halo.f90, src/halo_common.f90, halo_exchange_{x,y,z}_body.f90).
//
// update_halo copies a pencil into the interior of a larger array with
// `level` halo cells on its two distributed axes, then fills the halos by
// exchanging slabs with the neighbouring ranks.  On the GPU every one of
// those steps is a copy of a box of (w1, w2, w3) elements from one array at
// (o1, o2, o3) to another at (p1, p2, p3), both Fortran-ordered: the copy
// into the interior, the packing of the slabs a rank sends (into a
// contiguous buffer: an array of the box's own shape) and the unpacking of
// the slabs it receives.  One kernel, one thread per element, 4-, 8- or
// 16-byte words (real or complex, single or double), the destination
// written in its own order.  The host rejects a box that leaves either
// array before anything is launched.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "gbfft.h"
#include "gbfft_internal.h"

namespace gbfft {
namespace {

struct BoxArgs {
  const void* src;
  void* dst;
  long long s1, s2, d1, d2;  // leading extents of the two arrays
  long long o1, o2, o3, p1, p2, p3;
  long long w1, w2, w3;
};

template <typename W>
__global__ void __launch_bounds__(256) box_copy_kernel(const __grid_constant__ BoxArgs a) {
  const W* src = static_cast<const W*>(a.src);
  W* dst = static_cast<W*>(a.dst);
  const long long total = a.w1 * a.w2 * a.w3;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % a.w1, r = e / a.w1, j = r % a.w2, k = r / a.w2;
    dst[(a.p1 + i) + a.d1 * ((a.p2 + j) + a.d2 * (a.p3 + k))] =
        src[(a.o1 + i) + a.s1 * ((a.o2 + j) + a.s2 * (a.o3 + k))];
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

bool inside(const int* off, const int* w, const int* n) {
  for (int d = 0; d < 3; ++d)
    if (off[d] < 0 || w[d] < 0 || (long long)off[d] + w[d] > n[d]) return false;
  return true;
}

}  // namespace
}  // namespace gbfft

extern "C" int gbfft_box_copy(int is_complex, int prec, const void* d_src, const int* src_dims, const int* src_off,
                              void* d_dst, const int* dst_dims, const int* dst_off, const int* box, void* stream) {
  using namespace gbfft;
  if (prec != GBFFT_PREC_SINGLE && prec != GBFFT_PREC_DOUBLE)
    return set_error(GBFFT_ERR_INVALID, "Invalid value for precision (4 or 8)");
  if (!d_src || !d_dst || !src_dims || !src_off || !dst_dims || !dst_off || !box)
    return set_error(GBFFT_ERR_INVALID, "bad argument");
  for (int d = 0; d < 3; ++d)
    if (src_dims[d] <= 0 || dst_dims[d] <= 0) return set_error(GBFFT_ERR_INVALID, "array extents must be positive");
  if (!inside(src_off, box, src_dims) || !inside(dst_off, box, dst_dims))
    return set_error(GBFFT_ERR_INVALID, "box outside the source or destination array");
  const size_t esz = (is_complex ? 2 : 1) * (size_t)prec;
  if ((uintptr_t)d_src % esz || (uintptr_t)d_dst % esz)
    return set_error(GBFFT_ERR_INVALID, "array not aligned to its element size");
  const long long total = (long long)box[0] * box[1] * box[2];
  if (total == 0) return GBFFT_OK;
  BoxArgs a;
  a.src = d_src;
  a.dst = d_dst;
  a.s1 = src_dims[0];
  a.s2 = src_dims[1];
  a.d1 = dst_dims[0];
  a.d2 = dst_dims[1];
  a.o1 = src_off[0];
  a.o2 = src_off[1];
  a.o3 = src_off[2];
  a.p1 = dst_off[0];
  a.p2 = dst_off[1];
  a.p3 = dst_off[2];
  a.w1 = box[0];
  a.w2 = box[1];
  a.w3 = box[2];
  const unsigned grid = (unsigned)std::max(1ll, std::min((total + 255) / 256, (long long)sm_count() * 16));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (esz == 4) box_copy_kernel<unsigned><<<grid, 256, 0, st>>>(a);
  else if (esz == 8) box_copy_kernel<uint2><<<grid, 256, 0, st>>>(a);
  else box_copy_kernel<uint4><<<grid, 256, 0, st>>>(a);
  add_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GBFFT_ERR_CUDA, cudaGetErrorString(e));
  return GBFFT_OK;
}
