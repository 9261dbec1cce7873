// Allocation-free 3D c2r: gbfft_exec_c2r_noalloc.
//
// Who needs it: code that runs where device allocation is not allowed --
// inside a region that must not call cudaMalloc (a memory pool owned by
// another runtime, an application that reserved all device memory up front,
// a library callback that may not allocate or synchronise the device).  The
// regular path allocates at gbfft_engine_create (twiddle tables and the c2r
// work area); this entry point takes no engine and allocates nothing.
//
// What it uses instead: one file-scope static __device__ array of
// GBFFT_NOALLOC_SCRATCH_BYTES (64 MiB).  Every GPU that loads this library
// holds that array until the process exits.  A call places its twiddle
// tables and the complex intermediate (the c2r work area: the spectral array
// after the first two c2c passes) in it, so one call handles spectral arrays
// up to roughly 64 MiB minus its tables; larger sizes are rejected with
// GBFFT_ERR_INVALID.
//
// Sharing: every call on a device uses the same array and leaves its own
// contents there.  Nothing in the array needs to start at zero (each call
// writes its tables and its whole work area before reading them), but calls
// whose GPU work overlaps -- on different streams, or from different host
// threads -- race on the array and corrupt each other's results.
//
// Set-up: host code cannot use the array's name as a device address, so the
// first call on each device (with that device current) asks the runtime for
// the array's device address with cudaGetSymbolAddress and caches it.  Make
// that first call before any stream capture on that device.
//
// When the array is reserved: the CUDA runtime loads a library's device code
// lazily by default (CUDA_MODULE_LOADING=LAZY), so the 64 MiB are most likely
// reserved by that first call, not when the library is loaded.  A caller that
// will reserve all device memory, or enter a region where nothing may
// allocate, should make one call first (any small grid will do) or run with
// CUDA_MODULE_LOADING=EAGER.  The cached address belongs to the device's
// primary context: calling cudaDeviceReset between calls is not supported.
#include <atomic>
#include <cstdint>
#include <cmath>
#include <cstdio>

#include "gbfft.h"
#include "gbfft_internal.h"

namespace {

using gbfft::PassArgs;

constexpr size_t kScratchBytes = (size_t)GBFFT_NOALLOC_SCRATCH_BYTES;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::atomic<void*> g_scratch_addr[kMaxDevices];

int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gbfft::set_error(GBFFT_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return gbfft::set_error(GBFFT_ERR_UNSUPPORTED, "device index too large");
  void* p = g_scratch_addr[dev].load();
  if (!p) {
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      char msg[160];
      std::snprintf(msg, sizeof msg, "cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
      return gbfft::set_error(GBFFT_ERR_CUDA, msg);
    }
    g_scratch_addr[dev].store(p);
  }
  *out = p;
  return GBFFT_OK;
}

// exp(-2 pi i m / n), m = 0..n-1, written into the scratch array.
template <typename T>
__global__ void twiddle_kernel(T* tw, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  double s, c;
  sincospi(2.0 * (double)m / (double)n, &s, &c);
  tw[2 * m] = (T)c;
  tw[2 * m + 1] = (T)(-s);
}

struct Plan {
  int n, nst, tpl;
  int radix[gbfft::kMaxStages];
};

bool make_plan(int n, Plan& p) {
  int r[32];
  int cnt = 0, m = n, p2 = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++p2;
  }
  while (p2 >= 4) {
    r[cnt++] = 16;
    p2 -= 4;
  }
  if (p2 == 3) r[cnt++] = 8;
  if (p2 == 2) r[cnt++] = 4;
  if (p2 == 1) r[cnt++] = 2;
  for (int q : {7, 5, 3})
    while (m % q == 0) {
      r[cnt++] = q;
      m /= q;
    }
  for (int q = 11; (long long)q * q <= m && cnt < 31; q += 2)
    while (m % q == 0 && cnt < 31) {
      r[cnt++] = q;
      m /= q;
    }
  if (m > 1) r[cnt++] = m;
  if (cnt > gbfft::kMaxStages) return false;
  p.n = n;
  p.nst = cnt;
  for (int i = 0; i < gbfft::kMaxStages; ++i) p.radix[i] = i < cnt ? r[i] : 0;
  int tpl = (n + 7) / 8;
  if (tpl > gbfft::kMaxThreads) tpl = gbfft::kMaxThreads;
  p.tpl = tpl < 1 ? 1 : tpl;
  return true;
}

void tile(const Plan& p, int prec, bool contiguous, long long nlines, PassArgs& a) {
  int tpl = p.tpl, L;
  if (contiguous) {
    L = 256 / tpl;
    if (L < 1) L = 1;
  } else {
    const int min_l = 64 / (2 * prec);
    L = 512 / tpl;
    if (L > 32) L = 32;
    if (L < min_l) L = min_l;
    while (L * tpl > gbfft::kMaxThreads && tpl > 32) tpl /= 2;
    while (L > 1 && L * tpl > gbfft::kMaxThreads) L /= 2;
  }
  while (L > 1 && gbfft::pass_smem_bytes(prec, p.n, L) > 100 * 1024) L /= 2;
  if (L > 1 && nlines < L) {
    int l2 = 1;
    while (l2 < nlines) l2 *= 2;
    L = l2;
  }
  a.L = L < 1 ? 1 : L;
  a.tpl = tpl;
  a.n = p.n;
  a.nst = p.nst;
  for (int i = 0; i < gbfft::kMaxStages; ++i) a.radix[i] = p.radix[i];
  a.first_fused = 0;
  a.last_fused = 0;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" int gbfft_exec_c2r_noalloc(int format, int nx, int ny, int nz, int prec, const void* d_in,
                                      void* d_out, void* stream) {
  if (nx <= 0) return gbfft::set_error(GBFFT_ERR_INVALID, "Invalid value for nx");
  if (ny <= 0) return gbfft::set_error(GBFFT_ERR_INVALID, "Invalid value for ny");
  if (nz <= 0) return gbfft::set_error(GBFFT_ERR_INVALID, "Invalid value for nz");
  if (format != GBFFT_PHYSICAL_IN_X && format != GBFFT_PHYSICAL_IN_Z)
    return gbfft::set_error(GBFFT_ERR_INVALID, "Invalid value for pencil");
  if (prec != GBFFT_PREC_SINGLE && prec != GBFFT_PREC_DOUBLE)
    return gbfft::set_error(GBFFT_ERR_INVALID, "Invalid value for precision (4 or 8)");
  if (!d_in || !d_out) return gbfft::set_error(GBFFT_ERR_INVALID, "null array pointer");
  // the kernels load and store whole elements: a complex input aligned to
  // 2 * prec bytes, a real output to prec bytes (as gbfft_exec_c2r)
  if ((uintptr_t)d_in % (2 * (uintptr_t)prec) != 0 || (uintptr_t)d_out % (uintptr_t)prec != 0)
    return gbfft::set_error(GBFFT_ERR_INVALID, "array not aligned to its element size");
  const int lens[3] = {nx, ny, nz};
  Plan plan[3];
  for (int d = 0; d < 3; ++d) {
    if (lens[d] > gbfft::kMaxN || gbfft::pass_smem_bytes(prec, lens[d], 1) > 200 * 1024 ||
        !make_plan(lens[d], plan[d]))
      return gbfft::set_error(GBFFT_ERR_UNSUPPORTED, "axis length does not fit one shared-memory tile");
  }
  const size_t cs = 2 * (size_t)prec;
  const int s1 = format == GBFFT_PHYSICAL_IN_X ? nx / 2 + 1 : nx;
  const int s3 = format == GBFFT_PHYSICAL_IN_Z ? nz / 2 + 1 : nz;
  const size_t spec_bytes = (size_t)s1 * ny * s3 * cs;
  const size_t real_bytes = (size_t)nx * ny * nz * prec;
  size_t tw_off[3], off = 0;
  for (int d = 0; d < 3; ++d) {
    tw_off[d] = off;
    off += align256((size_t)lens[d] * cs);
  }
  const size_t work_off = off;
  if (work_off + spec_bytes > kScratchBytes) {
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "c2r of %d x %d x %d needs %zu bytes of scratch; the static scratch holds %zu bytes "
                  "(64 MiB)",
                  nx, ny, nz, work_off + spec_bytes, kScratchBytes);
    return gbfft::set_error(GBFFT_ERR_INVALID, msg);
  }
  {
    const char* a = (const char*)d_in;
    const char* b = (const char*)d_out;
    if (a < b + real_bytes && b < a + spec_bytes)
      return gbfft::set_error(GBFFT_ERR_INVALID, "In-place c2r transform is not yet available");
  }
  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  unsigned char* sb = (unsigned char*)base;
  cudaStream_t st = (cudaStream_t)stream;

  for (int d = 0; d < 3; ++d) {
    const int n = lens[d];
    const int blocks = (n + 255) / 256;
    if (prec == 8)
      twiddle_kernel<double><<<blocks, 256, 0, st>>>((double*)(sb + tw_off[d]), n);
    else
      twiddle_kernel<float><<<blocks, 256, 0, st>>>((float*)(sb + tw_off[d]), n);
    gbfft::add_launches(1);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gbfft::set_error(GBFFT_ERR_CUDA, cudaGetErrorString(e));

  void* W = sb + work_off;
  // two c2c passes into the work area, in the reference's order
  // (src/fft_common_3d.f90:216-283), then the c2r pass into d_out
  const int order_x[2] = {2, 1}, order_z[2] = {0, 1};
  const int* order = format == GBFFT_PHYSICAL_IN_X ? order_x : order_z;
  const void* cur = d_in;
  for (int i = 0; i < 2; ++i) {
    const int ax = order[i];
    PassArgs a = {};
    a.src = cur;
    a.dst = W;
    a.inverse = 1;
    a.tw = sb + tw_off[ax];
    bool contiguous;
    if (ax == 0) {
      contiguous = true;
      a.s_src_n = a.s_dst_n = 1;
      a.s_src_l = a.s_dst_l = s1;
      a.nlines = ny * s3;
      a.nv = 1;
    } else if (ax == 1) {
      contiguous = false;
      a.s_src_n = a.s_dst_n = s1;
      a.s_src_l = a.s_dst_l = (long long)s1 * ny;
      a.nlines = s1;
      a.nv = s3;
    } else {
      contiguous = false;
      a.s_src_n = a.s_dst_n = (long long)s1 * ny;
      a.s_src_l = a.s_dst_l = s1;
      a.nlines = s1;
      a.nv = ny;
    }
    tile(plan[ax], prec, contiguous, a.nlines, a);
    e = gbfft::launch_axis_pass(prec, gbfft::K_C2C, contiguous, a, st);
    if (e != cudaSuccess) return gbfft::set_error(GBFFT_ERR_CUDA, cudaGetErrorString(e));
    cur = W;
  }
  PassArgs a = {};
  a.src = cur;
  a.dst = d_out;
  a.inverse = 1;
  bool contiguous;
  int ax;
  if (format == GBFFT_PHYSICAL_IN_X) {
    ax = 0;
    contiguous = true;
    a.s_src_n = a.s_dst_n = 1;
    a.s_src_l = s1;
    a.s_dst_l = nx;
    a.real_lines = ny * nz;
    a.nv = 1;
  } else {
    ax = 2;
    contiguous = false;
    a.s_src_n = a.s_dst_n = (long long)nx * ny;
    a.s_src_l = a.s_dst_l = nx;
    a.real_lines = nx;
    a.nv = ny;
  }
  a.nlines = (a.real_lines + 1) / 2;
  a.tw = sb + tw_off[ax];
  tile(plan[ax], prec, contiguous, a.nlines, a);
  e = gbfft::launch_axis_pass(prec, gbfft::K_C2R, contiguous, a, st);
  if (e != cudaSuccess) return gbfft::set_error(GBFFT_ERR_CUDA, cudaGetErrorString(e));
  return GBFFT_OK;
}
