// Host side of the GB300 3D FFT backend: plans, engines and the C ABI of
// include/gbfft.h.
//
// An engine is one FFT grid of the reference's multiple-grids API
// (decomp_2d_fft_engine, src/fft_common.f90:141-242).  At one rank the
// reference runs, per direction, three batched 1D transforms separated by
// transposes that are plain copies (src/fft_common_3d.f90, src/fft_cufft.f90:
// 676-1170).  Here the copies disappear: each axis pass reads its source and
// writes its destination directly, and the buffers are chosen so that no
// extra pass and no input-preserving copy (the reference's wk1) is needed:
//   r2c:  in -> out -> out -> out              (out is the work array)
//   c2c:  in -> out -> out -> out              (in is never modified)
//   c2r:  in -> W -> W -> out, W = in when inplace, else the engine's work
//         area (the complex intermediate does not fit in the real output).
#include <dlfcn.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <utility>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gbfft.h"
#include "gbfft_internal.h"

using namespace gbfft;

namespace {

thread_local std::string g_err;
std::atomic<int> g_warnings{0};
// gbfft_debug_fail_alloc: allocations to let through before one fails (-1:
// none fails)
std::atomic<long long> g_fail_alloc{-1};
// NVTX ranges around transforms and passes (gbfft_set_nvtx, GBFFT_NVTX=1)
std::atomic<int> g_nvtx{-1};
bool nvtx_on() {
  int v = g_nvtx.load();
  if (v < 0) {
    const char* env = std::getenv("GBFFT_NVTX");
    v = (env && env[0] && env[0] != '0') ? 1 : 0;
    g_nvtx.store(v);
  }
  return v == 1;
}
// a named range of the transform (the reference's profiler regions
// "fft_r2c" / "fft_c2r" / "fft_c2c", src/fft_common_3d.f90:22,114) or pass
struct Range {
  bool on;
  explicit Range(const char* name) : on(nvtx_on()) {
    if (on) nvtxRangePushA(name);
  }
  ~Range() {
    if (on) nvtxRangePop();
  }
};
const char* kPassNames[GBFFT_PASS_KINDS] = {"pass r2c", "pass c2r", "pass c2c x", "pass c2c y", "pass c2c z",
                                            "pass x+y fused"};

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return GBFFT_ERR_CUDA;
}

constexpr unsigned kMagic = 0x47424646u;  // "GBFF"

struct AxisPlan {
  int n = 1;
  int nst = 0;
  int radix[kMaxStages] = {0};
  int tpl = 1;        // threads per line
  int fast_e = 16;    // points per thread of the power-of-two kernel
  bool big = false;   // lines do not fit one shared-memory tile: the
                      // multi-kernel long-axis path (fft_long.cu)
  bool blue = false;  // a prime factor above kBluePrime: the chirp-z path
                      // of fft_long.cu (implies big)
  void* d_tw = nullptr;   // exp(-2 pi i m / n), m = 0..n-1
  void* d_twf = nullptr;  // stage-major table of the power-of-two kernel
  void* d_twfb = nullptr;   // the same for the batch kernel's plan
                            // (batch_points), when the axis runs another
  void* d_chirp = nullptr;  // chirp-z tables (bt points at them)
  void* d_filt = nullptr;
  void* d_twm = nullptr;
  BlueTables bt{};
};

// Largest prime factor of an axis's length, from its radix stages (the
// power-of-two radices 16/8/4 count as 2).
int largest_prime(const AxisPlan& p) {
  int q = 1;
  for (int i = 0; i < p.nst; ++i) {
    const int r = p.radix[i];
    q = std::max(q, (r == 16 || r == 8 || r == 4) ? 2 : r);
  }
  return q;
}

// Split n into radix stages: 16s, then one 8/4/2 for the rest of the powers
// of two, then 7s, 5s, 3s, then any other prime as a generic stage.  Largest
// radices first.  Any length factorises; whether its lines fit one tile is
// decided by the caller.
bool factorize(int n, AxisPlan& p, std::string& why) {
  std::vector<int> r;
  int m = n;
  int p2 = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++p2;
  }
  while (p2 >= 4) {
    r.push_back(16);
    p2 -= 4;
  }
  if (p2 == 3) r.push_back(8);
  if (p2 == 2) r.push_back(4);
  if (p2 == 1) r.push_back(2);
  for (int q : {7, 5, 3}) {
    while (m % q == 0) {
      r.push_back(q);
      m /= q;
    }
  }
  for (int q = 11; (long long)q * q <= m; q += 2) {
    while (m % q == 0) {
      r.push_back(q);
      m /= q;
    }
  }
  if (m > 1) r.push_back(m);
  if ((int)r.size() > kMaxStages) {
    why = "too many radix stages";
    return false;
  }
  p.n = n;
  p.nst = (int)r.size();
  for (int i = 0; i < p.nst; ++i) p.radix[i] = r[i];
  // threads per line: about 8 points per thread, at most one CTA's worth
  int tpl = (n + 7) / 8;
  if (tpl > kMaxThreads) tpl = kMaxThreads;
  if (tpl < 1) tpl = 1;
  p.tpl = tpl;
  return true;
}

// Twiddle table exp(-2 pi i m / n), m = 0..n-1, evaluated in long double and
// rounded once to the working precision.
std::vector<double> twiddles(int n) {
  std::vector<double> t(2 * (size_t)n);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < n; ++m) {
    // reduce to the first half turn for accuracy
    long double a = two_pi * (long double)m / (long double)n;
    long double c = cosl(a), s = sinl(a);
    if (4 * m == n) { c = 0; s = 1; }
    if (2 * m == n) { c = -1; s = 0; }
    if (4 * m == 3 * n) { c = 0; s = -1; }
    t[2 * m] = (double)c;
    t[2 * m + 1] = (double)(-s);
  }
  return t;
}

// Stage-major twiddles of the power-of-two kernel: stage s of radix R after
// NS points holds W_{NS R}^{k r} at (NS - 1) + (r - 1) NS + k, for
// r = 1..R-1, k = 0..NS-1 (n - 1 entries in all).
std::vector<double> stage_twiddles(const std::vector<int>& radices) {
  int n = 1;
  for (int r : radices) n *= r;
  std::vector<double> t(2 * (size_t)n, 0.0);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  int ns = 1;
  for (size_t s = 0; s < radices.size(); ++s) {
    const int R = radices[s];
    for (int r = 1; r < R; ++r)
      for (int k = 0; k < ns; ++k) {
        const long long m = ((long long)k * r) % ((long long)ns * R);
        const long double a = two_pi * (long double)m / (long double)(ns * R);
        const size_t i = (size_t)(ns - 1) + (size_t)(r - 1) * ns + k;
        t[2 * i] = (double)cosl(a);
        t[2 * i + 1] = (double)(-sinl(a));
      }
    ns *= R;
  }
  return t;
}

int upload_table(void** dst, const std::vector<double>& t, int prec) {
  const size_t bytes = t.size() / 2 * 2 * (size_t)prec;
  cudaError_t e = dev_malloc(dst, bytes);
  if (e != cudaSuccess) {
    *dst = nullptr;
    return fail(GBFFT_ERR_ALLOC, std::string("cudaMalloc(twiddles): ") + cudaGetErrorString(e));
  }
  if (prec == 8) {
    e = cudaMemcpy(*dst, t.data(), bytes, cudaMemcpyHostToDevice);
  } else {
    std::vector<float> f(t.size());
    for (size_t i = 0; i < t.size(); ++i) f[i] = (float)t[i];
    e = cudaMemcpy(*dst, f.data(), bytes, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(twiddles)");
  return GBFFT_OK;
}

// Radices of an axis's compile-time plan (power of two: fast_e points a
// thread; balanced non-power-of-two plan when fast_e = gen_points(n); the
// two-stage mixed-radix plan otherwise); empty when the axis has none.
std::vector<int> plan_radices(const AxisPlan& p) {
  std::vector<int> radices;
  if (fast_length(p.n)) {
    for (int s = 0; s < fast_nst(p.n, p.fast_e); ++s) radices.push_back(fast_radix(p.n, p.fast_e, s));
  } else if (gen_length(p.n) && p.fast_e == gen_points(p.n)) {
    for (int s = 0; gen_radix(p.n, s) > 0; ++s) radices.push_back(gen_radix(p.n, s));
  } else if (mixed_length(p.n)) {
    radices = {mixed_r0(p.n), p.n / mixed_r0(p.n)};
  }
  return radices;
}

// Forward DFT of a (power-of-two length) in place, iterative radix 2, in
// double with roots evaluated in long double: the chirp-z filter.
void host_fft_pow2(std::vector<double>& a) {
  const size_t m = a.size() / 2;
  for (size_t i = 1, j = 0; i < m; ++i) {
    size_t bit = m >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(a[2 * i], a[2 * j]);
      std::swap(a[2 * i + 1], a[2 * j + 1]);
    }
  }
  const std::vector<double> root = twiddles((int)m);  // exp(-2 pi i k / m)
  for (size_t len = 2; len <= m; len <<= 1) {
    const size_t half = len / 2, step = m / len;
    for (size_t i = 0; i < m; i += len)
      for (size_t k = 0; k < half; ++k) {
        const double wr = root[2 * k * step], wi = root[2 * k * step + 1];
        double* u = &a[2 * (i + k)];
        double* v = &a[2 * (i + k + half)];
        const double tr = v[0] * wr - v[1] * wi, ti = v[0] * wi + v[1] * wr;
        v[0] = u[0] - tr;
        v[1] = u[1] - ti;
        u[0] += tr;
        u[1] += ti;
      }
  }
}

// Chirp-z tables of an axis: w_j = exp(-i pi j^2 / n) (j^2 reduced mod 2n
// exactly), FFT_m(b) / m with b_j = b_(m-j) = conj w_j, the m roots, and
// the radix plan of m (16s, then one 8/4/2).
int upload_blue(AxisPlan& p, int prec) {
  const int n = p.n;
  long long m = 1;
  while (m < 2LL * n - 1) m <<= 1;
  if (m > (1LL << 24)) return fail(GBFFT_ERR_UNSUPPORTED, "axis too long for the chirp-z path");
  const long double pi = 3.141592653589793238462643383279502884L;
  std::vector<double> w(2 * (size_t)n), b(2 * (size_t)m, 0.0);
  for (long long j = 0; j < n; ++j) {
    const unsigned long long e = ((unsigned long long)j * (unsigned long long)j) % (2ULL * (unsigned long long)n);
    const long double a = pi * (long double)e / (long double)n;
    const double c = (double)cosl(a), sn = (double)sinl(a);
    w[2 * j] = c;
    w[2 * j + 1] = -sn;
    b[2 * j] = c;
    b[2 * j + 1] = sn;
    if (j > 0) {
      b[2 * (m - j)] = c;
      b[2 * (m - j) + 1] = sn;
    }
  }
  host_fft_pow2(b);
  for (double& v : b) v /= (double)m;
  int rc = upload_table(&p.d_chirp, w, prec);
  if (rc == GBFFT_OK) rc = upload_table(&p.d_filt, b, prec);
  if (rc == GBFFT_OK) rc = upload_table(&p.d_twm, twiddles((int)m), prec);
  if (rc != GBFFT_OK) return rc;
  BlueTables& t = p.bt;
  t.m = (int)m;
  t.nst = 0;
  int lg = 0;
  while ((1LL << lg) < m) ++lg;
  for (; lg >= 4; lg -= 4) t.radix[t.nst++] = 16;
  if (lg > 0) t.radix[t.nst++] = 1 << lg;
  t.chirp = p.d_chirp;
  t.filt = p.d_filt;
  t.twm = p.d_twm;
  return GBFFT_OK;
}

// The batch kernel runs batch_points(n) points a thread on power-of-two
// lines of at most 256 points: an axis on another plan also keeps that
// plan's stage-major table.
int upload_batch_table(AxisPlan& p, int prec) {
  if (!fast_length(p.n) || p.n > 256 || p.fast_e == batch_points(p.n) || p.d_twfb) return GBFFT_OK;
  AxisPlan q = p;
  q.fast_e = batch_points(p.n);
  return upload_table(&p.d_twfb, stage_twiddles(plan_radices(q)), prec);
}

int upload_twiddles(AxisPlan& p, int prec) {
  int rc = upload_table(&p.d_tw, twiddles(p.n), prec);
  const std::vector<int> radices = plan_radices(p);
  if (rc == GBFFT_OK && !radices.empty()) rc = upload_table(&p.d_twf, stage_twiddles(radices), prec);
  if (rc == GBFFT_OK && p.blue) rc = upload_blue(p, prec);
  if (rc == GBFFT_OK) rc = upload_batch_table(p, prec);
  return rc;
}

// ---- tuning cache -------------------------------------------------------
// Text file, one shape per line:
//   prec format nx ny nz key=value ...
// keys: r2c c2r c2c_x c2c_y c2c_z xy_fused (lines per CTA of that pass),
// fuse (0/1), e_y e_z (points per thread of the strided y / z plan).
struct TuneEntry {
  int prec = 0, format = 0, nx = 0, ny = 0, nz = 0;
  int fuse = -1;
  int L[GBFFT_PASS_KINDS] = {0};
  int csize[GBFFT_PASS_KINDS] = {0};
  int csync[GBFFT_PASS_KINDS] = {0};
  int e[3] = {0, 0, 0};
  int pad = -1, flat = -1;
  int tma = -1;
};

std::mutex g_tune_mu;
bool g_tune_loaded = false;
std::string g_tune_path_override;
bool g_tune_path_set = false;
std::vector<TuneEntry> g_tune;

std::string default_tune_path() {
  const char* env = std::getenv("GBFFT_TUNE_CACHE");
  if (env) return env;
  Dl_info info;
  if (dladdr(reinterpret_cast<void*>(&gbfft_engine_create), &info) && info.dli_fname) {
    std::string so = info.dli_fname;  // .../2decomp-fft_gb300/lib/libgbfft.so
    size_t a = so.rfind('/');
    if (a != std::string::npos) {
      size_t b = so.rfind('/', a == 0 ? 0 : a - 1);
      if (b != std::string::npos) return so.substr(0, b) + "/tune_cache.txt";
    }
  }
  return "";
}

void load_tune_locked() {
  g_tune.clear();
  g_tune_loaded = true;
  const std::string path = g_tune_path_set ? g_tune_path_override : default_tune_path();
  if (path.empty()) return;
  std::ifstream f(path);
  std::string line;
  static const char* names[GBFFT_PASS_KINDS] = {"r2c", "c2r", "c2c_x", "c2c_y", "c2c_z", "xy_fused"};
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream in(line);
    TuneEntry t;
    if (!(in >> t.prec >> t.format >> t.nx >> t.ny >> t.nz)) continue;
    std::string kv;
    while (in >> kv) {
      const size_t eq = kv.find('=');
      if (eq == std::string::npos) continue;
      const std::string k = kv.substr(0, eq);
      const int v = std::atoi(kv.c_str() + eq + 1);
      if (k == "fuse") t.fuse = v;
      else if (k == "e_x") t.e[0] = v;
      else if (k == "e_y") t.e[1] = v;
      else if (k == "e_z") t.e[2] = v;
      else if (k == "pad") t.pad = v;
      else if (k == "flat") t.flat = v;
      else if (k == "tma") t.tma = v;
      for (int i = 0; i < GBFFT_PASS_KINDS; ++i) {
        if (k == names[i]) t.L[i] = v;
        if (k == std::string("cl_") + names[i]) t.csize[i] = v;
        if (k == std::string("cls_") + names[i]) t.csync[i] = v;
      }
    }
    g_tune.push_back(t);
  }
}

TuneEntry lookup_tune(int prec, int format, int nx, int ny, int nz) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (!g_tune_loaded) load_tune_locked();
  for (const TuneEntry& t : g_tune)
    if (t.prec == prec && t.format == format && t.nx == nx && t.ny == ny && t.nz == nz) return t;
  return TuneEntry();
}

}  // namespace

struct ProfRec {
  int kind;
  cudaEvent_t start, stop;
  double bytes;
};

struct gbfft_engine_s {
  unsigned magic = kMagic;
  bool profiling = false;
  std::vector<ProfRec> prof;          // launches not yet resolved
  long long prof_n[GBFFT_PASS_KINDS] = {0};
  double prof_ms[GBFFT_PASS_KINDS] = {0};
  double prof_bytes[GBFFT_PASS_KINDS] = {0};
  int format = GBFFT_PHYSICAL_IN_X;
  int nx = 0, ny = 0, nz = 0;
  int inplace = 0;
  int skip[3] = {0, 0, 0};
  int prec = 8;
  int form = GBFFT_FORM_PLAIN;
  int ph[3] = {0, 0, 0};
  int sp[3] = {0, 0, 0};
  AxisPlan ax[3];
  int tile_L[GBFFT_PASS_KINDS] = {0};  // tuned lines per CTA, 0 = built-in
  int csize[GBFFT_PASS_KINDS] = {0};   // cluster launch of the one-shot kernel, 0 = none
  int csync[GBFFT_PASS_KINDS] = {0};   // with it, a cluster barrier at the start
  bool fuse = false;                   // fuse x/y passes per plane when possible
  int* d_sync = nullptr;               // fused kernel's ticket/status/plane counters
  long long sync_planes = 0;
  void* work = nullptr;
  size_t work_bytes = 0;
  // Row layout: `pad` -- 1: the work area's rows of complex values start on
  // kRowAlignBytes boundaries (its row pitch is sp[0] rounded up) and every
  // r2c / c2r pass but the last writes there, so that the strided passes
  // store whole 32-byte sectors; 2: the same for c2r only (r2c works in its
  // output); 0: unpadded.  `flat` -- z passes whose output rows are
  // unpadded and not so aligned take the lines of each (x, y) plane flat
  // (segments aligned as the plane is).
  int pad = 0;
  bool flat = true;
  // strided FP32 c2c passes of 256, 512 and 1024 points whose source rows
  // allow it run the persistent kernel fed by bulk tensor copies
  bool tma = true;
  int* d_status = nullptr;  // set to 1 by a bounded wait that gave up
  // two buffers of the grid's size for axes on the long-axis path
  void* long_scratch = nullptr;
  size_t long_scratch_bytes = 0;
};

namespace {

bool valid_engine(gbfft_engine_t e) { return e != nullptr && e->magic == kMagic; }

void drop_profile(gbfft_engine_t e) {
  for (auto& r : e->prof) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  e->prof.clear();
}

void release(gbfft_engine_t e) {
  drop_profile(e);
  for (auto& a : e->ax) {
    for (void** q : {&a.d_tw, &a.d_twf, &a.d_twfb, &a.d_chirp, &a.d_filt, &a.d_twm}) {
      if (*q) dev_free(*q);
      *q = nullptr;
    }
  }
  if (e->work) dev_free(e->work);
  e->work = nullptr;
  if (e->d_sync) dev_free(e->d_sync);
  e->d_sync = nullptr;
  if (e->d_status) dev_free(e->d_status);
  e->d_status = nullptr;
  if (e->long_scratch) dev_free(e->long_scratch);
  e->long_scratch = nullptr;
}

size_t cbytes(const gbfft_engine_s* e) { return 2 * (size_t)e->prec; }

// Row pitch (complex elements) of the work area.
constexpr size_t kRowAlignBytes = 64;
long long padded_pitch(const gbfft_engine_s* e) {
  const long long q = (long long)(kRowAlignBytes / cbytes(e));
  return (e->sp[0] + q - 1) / q * q;
}
// pitch of the work area's rows for c2r (r2c uses the work area only with pad 1)
long long work_pitch(const gbfft_engine_s* e) { return e->pad ? padded_pitch(e) : e->sp[0]; }
// Rows of n elements of `bytes` each whose tiles of 16 lines start on
// 32-byte sectors and fill each row: taken per row, a z pass over them is
// as aligned as a flat one.
bool rows_aligned(long long n, size_t bytes) { return (n * (long long)bytes) % 32 == 0 && n % 16 == 0; }

// Lines per CTA for a pass with the given plan.
int lines_per_cta(const AxisPlan& p, int prec, bool contiguous, long long nlines, int* tpl_out,
                  int forced_L) {
  int tpl = p.tpl;
  int L;
  if (forced_L > 0) {
    L = forced_L;
    if (!contiguous)
      while (L * tpl > kMaxThreads && tpl > 32) tpl /= 2;
    *tpl_out = tpl;
    return L;
  }
  if (contiguous) {
    L = 256 / tpl;
    if (L < 1) L = 1;
  } else {
    // a warp row should cover at least 64 contiguous bytes of x
    const int min_l = (int)(64 / (2 * prec));
    L = 512 / tpl;
    if (L > 32) L = 32;
    if (L < min_l) L = min_l;
    while (L * tpl > kMaxThreads && tpl > 32) tpl /= 2;
    while (L > 1 && L * tpl > kMaxThreads) L /= 2;
  }
  while (L > 1 && pass_smem_bytes(prec, p.n, L) > 100 * 1024) L /= 2;
  *tpl_out = tpl;
  if (L > 1 && nlines < L) {
    int l2 = 1;
    while (l2 < nlines) l2 *= 2;
    L = l2;
  }
  return L < 1 ? 1 : L;
}

// Lines per CTA for the power-of-two kernel (n / fast_points(n) threads per
// line).
int fast_lines_per_cta(int n, int prec, bool contiguous, long long nlines, int forced_L, int e,
                       long long nv = 1) {
  const int tpl = n / e;
  if (forced_L > 0) return forced_L;
  const int maxt = fast_max_threads(e, prec);
  int L;
  if (contiguous) {
    // lines of at most 32 threads run warp-synchronous: 4 warps per CTA;
    // longer lines: one line (pair) per CTA, so that many small CTAs per SM
    // overlap their load, exchange and store phases
    L = tpl > 32 ? 1 : 128 / tpl;
  } else {
    const int min_l = (int)(64 / (2 * prec));
    L = 512 / tpl;
    if (L > 32) L = 32;
    if (L < min_l) L = min_l;
  }
  while (L > 1 && L * tpl > maxt) L /= 2;
  while (L > 1 && (size_t)fast_smem_entries(n, L) * 2 * prec > 100 * 1024) L /= 2;
  if (L < 1) L = 1;
  // small grids: fewer lines a CTA until there are two CTAs per SM (strided
  // tiles keep at least 64-byte row segments)
  const int min_keep = contiguous ? 1 : (int)(64 / (2 * prec));
  while (L > min_keep && ((nlines + L - 1) / L) * nv < 2LL * kSmsDefault) L /= 2;
  if (L > 1 && nlines < L) {
    int l2 = 1;
    while (l2 < nlines) l2 *= 2;
    L = l2;
  }
  return L;
}

// Fill the plan-dependent fields of a pass.
// Lines per CTA for the mixed-radix kernel (R1 = n / mixed_r0(n) threads a
// line, at most 256 threads a CTA).
int mixed_lines_per_cta(int n, int prec, bool contiguous, long long nlines, int forced_L) {
  const int tpl = n / mixed_r0(n);
  if (forced_L > 0) return forced_L;
  int L = contiguous ? 192 / tpl : 256 / tpl;
  if (!contiguous) {
    const int min_l = (int)(64 / (2 * prec));
    if (L < min_l) L = min_l;
  }
  while (L > 1 && L * tpl > 256) --L;
  while (L > 1 && (size_t)fast_smem_entries(n, L) * 2 * prec > 100 * 1024) --L;
  if (L < 1) L = 1;
  if (L > 1 && nlines < L) L = (int)nlines;
  return L;
}

// Lines a CTA of the balanced non-power-of-two kernel: contiguous lines 128
// threads a CTA (at least one line); strided lines enough for 64-byte row
// segments and about 512 threads; within the thread and 100 KB shared-memory
// limits.
int gen_lines_per_cta(int n, int prec, bool contiguous, long long nlines, int forced_L) {
  const int e = gen_points(n), tpl = n / e, maxt = gen_max_threads(e, prec);
  int L;
  if (forced_L > 0) {
    L = forced_L;
  } else if (contiguous) {
    L = tpl >= 128 ? 1 : 128 / tpl;
  } else {
    L = 512 / tpl;
    if (L > 32) L = 32;
    const int min_l = (int)(64 / (2 * prec));
    if (L < min_l) L = min_l;
  }
  while (L > 1 && L * tpl > maxt) --L;
  while (L > 1 && (size_t)fast_smem_entries(n, L) * 2 * prec > (forced_L > 0 ? 200 : 100) * 1024) --L;
  if (L < 1) L = 1;
  if (forced_L <= 0 && L > 1 && nlines < L) L = (int)nlines;
  return L;
}

void fill_plan(PassArgs& a, const AxisPlan& p, int prec, bool contiguous, int kind, int forced_L,
               bool split = false, int csize = 0, int csync = 0) {
  a.blue = p.blue ? &p.bt : nullptr;
  if (split && split_length(p.n)) {
    a.n = p.n;
    a.nst = 0;
    a.tw = p.d_twf;
    a.fast = 3;
    a.L = split_lines_per_cta(p.n, contiguous);
    a.tpl = 256 / a.L;
    a.first_fused = 0;
    a.last_fused = 0;
    (void)forced_L;
    (void)kind;
    return;
  }
  if (gen_length(p.n) && p.fast_e == gen_points(p.n)) {
    a.n = p.n;
    a.nst = 0;
    a.tw = p.d_twf;
    a.fast = 4;
    a.tpl = p.n / p.fast_e;
    a.L = gen_lines_per_cta(p.n, prec, contiguous, a.nlines, forced_L);
    a.first_fused = 1;
    a.last_fused = kind != K_R2C;
    return;
  }
  if (mixed_length(p.n)) {
    a.n = p.n;
    a.nst = 0;
    a.tw = p.d_twf;
    a.fast = 2;
    a.tpl = p.n / mixed_r0(p.n);
    a.L = mixed_lines_per_cta(p.n, prec, contiguous, a.nlines, forced_L);
    a.first_fused = 1;
    a.last_fused = kind != K_R2C;
    return;
  }
  if (fast_length(p.n)) {
    a.n = p.n;
    a.nst = 0;
    a.tw = p.d_twf;
    a.fast = 1;
    const int fe = p.fast_e;  // only axis 0 runs contiguous lines
    a.tpl = p.n / fe;
    a.L = fast_lines_per_cta(p.n, prec, contiguous, a.nlines, forced_L, fe, contiguous ? 1 : a.nv);
    a.first_fused = 1;
    a.last_fused = kind != K_R2C;
    a.csize = csize > 1 ? csize : 0;
    a.csync = a.csize ? csync : 0;
    return;
  }
  a.n = p.n;
  a.nst = p.nst;
  for (int i = 0; i < kMaxStages; ++i) a.radix[i] = i < p.nst ? p.radix[i] : 0;
  a.tw = p.d_tw;
  a.L = lines_per_cta(p, prec, contiguous, a.nlines, &a.tpl, forced_L);
  a.first_fused = 0;
  a.last_fused = 0;
  (void)kind;
}

struct Pass {
  PassArgs a;
  int kind;
  bool contiguous;
  int prof_kind;   // GBFFT_PASS_*
  double bytes;    // algorithmic bytes: one read + one write of the array
  bool fused = false;  // x and y passes of each z-plane in one kernel
  bool big = false;    // long-axis path (one kernel per radix stage)
  FusedArgs f;
  int fused_kindx = 0;
  bool fused_xfirst = true;
};

// c2c along `axis` of a complex (n1, n2, n3) array whose rows of n1 values
// lie `pin` (source) and `pout` (destination) elements apart.  A z pass
// into unpadded rows takes each plane's lines flat when the engine says so.
Pass c2c_pass(const gbfft_engine_s* e, int axis, int n1, int n2, int n3, const void* src, void* dst,
              int inverse, long long pin, long long pout) {
  Pass P;
  PassArgs& a = P.a;
  std::memset(&a, 0, sizeof(a));
  a.src = src;
  a.dst = dst;
  a.inverse = inverse;
  P.kind = K_C2C;
  if (axis == 0) {
    P.contiguous = true;
    a.s_src_n = a.s_dst_n = 1;
    a.s_src_l = pin;
    a.s_dst_l = pout;
    a.nlines = n2 * n3;
    a.nv = 1;
  } else if (axis == 1) {
    P.contiguous = false;
    a.s_src_n = pin;
    a.s_dst_n = pout;
    a.s_src_l = pin * n2;
    a.s_dst_l = pout * n2;
    a.nlines = n1;
    a.nv = n3;
  } else {
    P.contiguous = false;
    a.s_src_n = pin * n2;
    a.s_dst_n = pout * n2;
    a.s_src_l = pin;
    a.s_dst_l = pout;
    a.nlines = n1;
    a.nv = n2;
    if (e->flat && pout == n1 && !rows_aligned(n1, cbytes(e)) && !e->ax[axis].big) {
      a.nlines = n1 * n2;
      a.nv = 1;
      a.row_w = n1;
      a.s_src_r = pin;
      a.s_dst_r = pout;
    }
  }
  fill_plan(a, e->ax[axis], e->prec, P.contiguous, K_C2C, e->tile_L[GBFFT_PASS_C2C_X + axis],
            e->form != GBFFT_FORM_PLAIN, e->csize[GBFFT_PASS_C2C_X + axis],
            e->csync[GBFFT_PASS_C2C_X + axis]);
  // 1024-point FP32 y passes over rows a tensor map can describe: the
  // persistent kernel whose tiles arrive by bulk tensor copies (its plan
  // shares the axis's stage-major twiddle table).  Shorter lines and z
  // passes stay on the one-shot kernel, which is as fast or faster there.
  // the tcgen05 form: strided 1024-point c2c passes on the 5th-generation
  // tensor cores (its DFT matrix and twiddles come from the n-root table)
  if (e->form == GBFFT_FORM_SPLIT_TC && e->d_status && a.fast == 3) {
    PassArgs t = a;
    t.tw = e->ax[axis].d_tw;
    if (tc_pass_supported(e->prec, K_C2C, P.contiguous, t)) {
      a.tw = t.tw;
      a.fast = 5;
      a.status = e->d_status;
    }
  }
  if (e->tma && e->d_status && axis == 1 && a.fast == 1 && tma_pass_supported(e->prec, K_C2C, P.contiguous, a)) {
    a.tma = 1;
    a.status = e->d_status;
    a.csize = 0;
    a.csync = 0;
  }
  P.big = e->ax[axis].big;
  P.prof_kind = GBFFT_PASS_C2C_X + axis;
  P.bytes = 2.0 * (double)n1 * n2 * n3 * (double)cbytes(e);
  return P;
}

// r2c (kind K_R2C) or c2r (K_C2R) along the engine's real axis; the
// complex side's rows lie `cp` elements apart.  Along z into unpadded rows
// the lines of each plane are taken flat when the engine says so.
Pass real_pass(const gbfft_engine_s* e, int kind, const void* src, void* dst, long long cp) {
  Pass P;
  PassArgs& a = P.a;
  std::memset(&a, 0, sizeof(a));
  a.src = src;
  a.dst = dst;
  P.kind = kind;
  const int nx = e->nx, ny = e->ny, nz = e->nz;
  long long real_s_n, real_s_l, cplx_s_n, cplx_s_l;
  bool flat = false;
  if (e->format == GBFFT_PHYSICAL_IN_X) {
    P.contiguous = true;
    real_s_n = cplx_s_n = 1;
    real_s_l = nx;
    cplx_s_l = cp;
    a.real_lines = ny * nz;
    a.nv = 1;
  } else {
    P.contiguous = false;
    real_s_n = (long long)nx * ny;
    cplx_s_n = cp * ny;
    real_s_l = nx;
    cplx_s_l = cp;
    a.real_lines = nx;
    a.nv = ny;
    // the output rows: complex (pitch cp) for r2c, real (nx) for c2r
    flat = e->flat && !e->ax[2].big &&
           (kind == K_C2R ? !rows_aligned(nx, (size_t)e->prec) : (cp == nx && !rows_aligned(nx, cbytes(e))));
    if (flat) {
      a.real_lines = nx * ny;
      a.nv = 1;
      a.row_w = nx;
    }
  }
  a.nlines = (a.real_lines + 1) / 2;
  if (kind == K_R2C) {
    a.s_src_n = real_s_n;
    a.s_src_l = real_s_l;
    a.s_dst_n = cplx_s_n;
    a.s_dst_l = cplx_s_l;
    a.inverse = 0;
  } else {
    a.s_src_n = cplx_s_n;
    a.s_src_l = cplx_s_l;
    a.s_dst_n = real_s_n;
    a.s_dst_l = real_s_l;
    a.inverse = 1;
  }
  if (flat) {
    a.s_src_r = a.s_src_l;
    a.s_dst_r = a.s_dst_l;
  }
  // strided pairs are neighbouring x positions: 8-byte aligned when nx is
  // even (every line then starts at an even real index)
  const void* real_ptr = kind == K_R2C ? src : dst;
  a.pair_vec = (!P.contiguous && nx % 2 == 0 && ((uintptr_t)real_ptr % (2 * (size_t)e->prec)) == 0) ? 1 : 0;
  // FP32 complex pairs: both complex lines of a pair side by side, 16-byte
  // aligned (every pair starts at an even complex index of an even pitch)
  const void* cplx_ptr = kind == K_R2C ? dst : src;
  if (a.pair_vec && e->prec == GBFFT_PREC_SINGLE && cp % 2 == 0 && ((uintptr_t)cplx_ptr % 16) == 0)
    a.pair_vec |= 2;
  const int axis = e->format == GBFFT_PHYSICAL_IN_X ? 0 : 2;
  fill_plan(a, e->ax[axis], e->prec, P.contiguous, kind,
            e->tile_L[kind == K_R2C ? GBFFT_PASS_R2C : GBFFT_PASS_C2R], e->form != GBFFT_FORM_PLAIN,
            e->csize[kind == K_R2C ? GBFFT_PASS_R2C : GBFFT_PASS_C2R],
            e->csync[kind == K_R2C ? GBFFT_PASS_R2C : GBFFT_PASS_C2R]);
  P.big = e->ax[axis].big;
  P.prof_kind = kind == K_R2C ? GBFFT_PASS_R2C : GBFFT_PASS_C2R;
  P.bytes = (double)nx * ny * nz * e->prec +
            (double)e->sp[0] * e->sp[1] * e->sp[2] * (double)cbytes(e);
  return P;
}

// Replace an adjacent x pass / y pass (either order, each feeding the next)
// by one fused x/y kernel when one exists for the lengths.  `planes` is the
// z extent of the array the two passes work on.
void fuse_xy(const gbfft_engine_s* e, std::vector<Pass>& ps, long long planes) {
  if (!e->d_sync || planes > e->sync_planes || e->form != GBFFT_FORM_PLAIN) return;
  for (size_t i = 0; i + 1 < ps.size(); ++i) {
    Pass& p0 = ps[i];
    Pass& p1 = ps[i + 1];
    const bool x0 = p0.contiguous && (p0.prof_kind == GBFFT_PASS_C2C_X || p0.prof_kind == GBFFT_PASS_R2C ||
                                      p0.prof_kind == GBFFT_PASS_C2R);
    const bool x1 = p1.contiguous && (p1.prof_kind == GBFFT_PASS_C2C_X || p1.prof_kind == GBFFT_PASS_R2C ||
                                      p1.prof_kind == GBFFT_PASS_C2R);
    const bool y0 = p0.prof_kind == GBFFT_PASS_C2C_Y, y1 = p1.prof_kind == GBFFT_PASS_C2C_Y;
    if (!((x0 && y1) || (y0 && x1))) continue;
    const bool xfirst = x0;
    Pass& px = xfirst ? p0 : p1;
    Pass& py = xfirst ? p1 : p0;
    if (p1.a.src != p0.a.dst) continue;
    if (!fast_length(px.a.n) || !fast_length(py.a.n)) continue;
    if (px.a.fast != 1 || py.a.fast != 1 || px.a.csize || py.a.csize) continue;
    if (px.a.tma || py.a.tma) continue;
    if (e->ax[1].fast_e != fast_points(py.a.n, false)) continue;  // the fused kernel's y plan
    if (e->ax[0].fast_e != fast_points(px.a.n, true)) continue;   // and its x plan
    if (!fused_supported(e->prec, px.kind, xfirst, px.a.n, py.a.n)) continue;
    long long per_plane;
    if (px.kind == K_C2C) {
      per_plane = px.a.nlines / planes;  // x lines of a c2c pass: n2 per plane
    } else {
      if (e->ny % 2) continue;  // line pairs must not straddle planes
      per_plane = e->ny / 2;
    }
    if (per_plane * planes != px.a.nlines) continue;
    Pass F = px;
    F.fused = true;
    F.fused_kindx = px.kind;
    F.fused_xfirst = xfirst;
    // tile shape: tile_L[XY] y lines a tile (threads = lines x y threads a line)
    const int ty = py.a.n / fast_points(py.a.n, false);
    const int th = e->tile_L[GBFFT_PASS_XY] ? e->tile_L[GBFFT_PASS_XY] * ty : kFusedThreads;
    F.f.threads = th;
    F.f.ax = px.a;
    F.f.ax.nlines = (int)per_plane;
    F.f.ax.tpl = px.a.n / fast_points(px.a.n, true);
    F.f.ax.L = th / F.f.ax.tpl;
    F.f.ay = py.a;
    F.f.ay.tpl = ty;
    F.f.ay.L = th / ty;
    F.f.nplanes = planes;
    F.f.sync = e->d_sync;
    F.prof_kind = GBFFT_PASS_XY;
    F.bytes = px.bytes + py.bytes;
    ps[i] = F;
    ps.erase(ps.begin() + i + 1);
    return;
  }
}

// Arrays of one transform (base, bytes), for the extents the bounds-checked
// build checks every access against.
struct Extent {
  const void* p;
  size_t bytes;
};

int run_passes(gbfft_engine_s* e, const std::vector<Pass>& ps, cudaStream_t st,
               std::initializer_list<Extent> arrays = {}) {
  for (const Pass& pc : ps) {
    Pass p = pc;
    // every pass reports to the engine's status word; the checked build
    // also needs each side's extent in elements of that side's type
    if (!p.a.status) p.a.status = e->d_status;
    const size_t cb = cbytes(e), rb = (size_t)e->prec;
    const size_t se = p.kind == K_R2C ? rb : cb, de = p.kind == K_C2R ? rb : cb;
    for (const Extent& x : arrays) {
      if (x.p == p.a.src) p.a.src_elems = (long long)(x.bytes / se);
      if (x.p == p.a.dst) p.a.dst_elems = (long long)(x.bytes / de);
    }
    if (e->work == p.a.src) p.a.src_elems = (long long)(e->work_bytes / se);
    if (e->work == p.a.dst) p.a.dst_elems = (long long)(e->work_bytes / de);
    Range range(p.fused ? "pass x+y fused" : kPassNames[p.prof_kind]);
    ProfRec rec{p.prof_kind, nullptr, nullptr, p.bytes};
    if (e->profiling) {
      if (cudaEventCreate(&rec.start) != cudaSuccess || cudaEventCreate(&rec.stop) != cudaSuccess)
        return fail(GBFFT_ERR_CUDA, "cudaEventCreate");
      cudaEventRecord(rec.start, st);
    }
    cudaError_t err = p.fused ? launch_fused(e->prec, p.fused_kindx, p.fused_xfirst, p.f, st)
                      : p.big ? launch_long_pass(e->prec, p.kind, p.contiguous, p.a, e->long_scratch,
                                                 e->long_scratch_bytes, st)
                              : launch_axis_pass(e->prec, p.kind, p.contiguous, p.a, st);
    if (e->profiling) {
      cudaEventRecord(rec.stop, st);
      e->prof.push_back(rec);
    }
    if (err != cudaSuccess) return cuda_fail(err, "axis pass launch");
  }
  return GBFFT_OK;
}

// Arrays must be aligned to their element: prec bytes for real arrays,
// 2 * prec for complex ones (the kernels move whole elements).
bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

bool overlap(const void* a, size_t na, const void* b, size_t nb) {
  const char* pa = (const char*)a;
  const char* pb = (const char*)b;
  return pa < pb + nb && pb < pa + na;
}

void warn_skip(int code) {
  g_warnings.fetch_add(1);
  std::fprintf(stderr, "gbfft warning %d: r2c / c2r transform can not be skipped\n", code);
}

}  // namespace

namespace {

// The passes of a 3D r2c (src/fft_common_3d.f90:121-189): the r2c pass
// along the real axis into `out`, then the c2c passes on `out`.
// Arguments of an engine: the same checks and order as
// src/fft_common.f90:157-166, :210-216, and the backend's own limits.
int check_engine_args(int format, int nx, int ny, int nz, int prec, int form) {
  if (nx <= 0) return fail(GBFFT_ERR_INVALID, "Invalid value for nx");
  if (ny <= 0) return fail(GBFFT_ERR_INVALID, "Invalid value for ny");
  if (nz <= 0) return fail(GBFFT_ERR_INVALID, "Invalid value for nz");
  if (format != GBFFT_PHYSICAL_IN_X && format != GBFFT_PHYSICAL_IN_Z)
    return fail(GBFFT_ERR_INVALID, "Invalid value for pencil");
  if (prec != GBFFT_PREC_SINGLE && prec != GBFFT_PREC_DOUBLE)
    return fail(GBFFT_ERR_INVALID, "Invalid value for precision (4 or 8)");
  if (form != GBFFT_FORM_PLAIN && form != GBFFT_FORM_SPLIT && form != GBFFT_FORM_SPLIT_TC)
    return fail(GBFFT_ERR_INVALID, "Invalid value for form");
  if (form != GBFFT_FORM_PLAIN && prec != GBFFT_PREC_SINGLE)
    return fail(GBFFT_ERR_UNSUPPORTED, "the split tensor-core form works on single-precision data");
  const long long cells = (long long)nx * ny * nz;
  if (cells > (1LL << 40)) return fail(GBFFT_ERR_UNSUPPORTED, "grid too large");
  if ((long long)ny * nz > 0x7fffffffLL || (long long)nx * ny > 0x7fffffffLL)
    return fail(GBFFT_ERR_UNSUPPORTED, "line count exceeds 2^31");
  return GBFFT_OK;
}

// The host half of gbfft_engine_create: fields, the axis plans and the
// tuning-cache line, no device memory (the caller uploads the twiddle tables
// and allocates the work area).  Arguments are already validated.
int engine_init_host(gbfft_engine_s* e, int format, int nx, int ny, int nz, int inplace, const int* skip, int prec,
                     int form, TuneEntry* tune_out) {
  e->format = format;
  e->nx = nx;
  e->ny = ny;
  e->nz = nz;
  e->inplace = inplace ? 1 : 0;
  for (int i = 0; i < 3; ++i) e->skip[i] = skip ? (skip[i] ? 1 : 0) : 0;
  e->prec = prec;
  e->form = form;
  e->ph[0] = nx;
  e->ph[1] = ny;
  e->ph[2] = nz;
  e->sp[0] = format == GBFFT_PHYSICAL_IN_X ? nx / 2 + 1 : nx;
  e->sp[1] = ny;
  e->sp[2] = format == GBFFT_PHYSICAL_IN_Z ? nz / 2 + 1 : nz;
  const TuneEntry tune = lookup_tune(prec, format, nx, ny, nz);
  const int lens[3] = {nx, ny, nz};
  for (int d = 0; d < 3; ++d) {
    std::string why;
    if (!factorize(lens[d], e->ax[d], why)) return fail(GBFFT_ERR_UNSUPPORTED, why);
    // lines longer than one shared-memory tile take the long-axis path
    e->ax[d].big = lens[d] > kMaxN || pass_smem_bytes(prec, lens[d], 1) > 200 * 1024;
    // a large prime factor: the chirp-z transform (O(n log n)) instead of a
    // direct-sum stage (O(p) a point)
    // (up to convolutions of 2^24 points: the host tables take 32 bytes a
    // point; longer axes keep the direct-sum stages)
    e->ax[d].blue = largest_prime(e->ax[d]) > kBluePrime && 2LL * lens[d] - 1 <= (1LL << 24);
    if (e->ax[d].blue) e->ax[d].big = true;
    e->ax[d].fast_e = fast_points(lens[d], d == 0);  // axis 0 runs contiguous lines
    if (fast_length(lens[d]) && lens[d] <= 256) {
      // short lines of a small grid: fewer points a thread until the pass
      // has about 16 warps per SM (lines of a full-grid pass: grid / n)
      const double lines = (double)nx * ny * nz / lens[d];
      int pe = 16;
      while (pe > 4 && fast_e_ok(lens[d], pe / 2) && lines * (lens[d] / pe) < 512.0 * kSmsDefault) pe /= 2;
      e->ax[d].fast_e = pe;
    }
    if (gen_length(lens[d])) e->ax[d].fast_e = gen_points(lens[d]);
    if (fast_has_alt(lens[d]) && tune.e[d] > 0 && fast_e_ok(lens[d], tune.e[d])) e->ax[d].fast_e = tune.e[d];
    if (gen_length(lens[d]) && (tune.e[d] == gen_points(lens[d]) || tune.e[d] == 2))
      e->ax[d].fast_e = tune.e[d];
    if (form != GBFFT_FORM_PLAIN && split_length(lens[d])) e->ax[d].fast_e = 16;  // radix-16 stages for the tensor cores
  }
  *tune_out = tune;
  return GBFFT_OK;
}

// Tuned tile shapes, launch forms, fusion and row layout for this shape,
// when the cache has them (host settings only).
void apply_tune(gbfft_engine_s* e, const TuneEntry& tune) {
  for (int k = 0; k < GBFFT_PASS_KINDS; ++k)
    if (tune.L[k] > 0 && gbfft_engine_set_tile(e, k, tune.L[k]) != GBFFT_OK) e->tile_L[k] = 0;
  for (int k = 0; k < GBFFT_PASS_KINDS; ++k)
    if (tune.csize[k] > 0 && gbfft_engine_set_cluster(e, k, tune.csize[k], tune.csync[k]) != GBFFT_OK) {
      e->csize[k] = 0;
      e->csync[k] = 0;
    }
  if (tune.fuse >= 0) e->fuse = tune.fuse != 0;
  if (tune.pad >= 0 && tune.pad <= 2) e->pad = tune.pad;
  if (tune.flat >= 0) e->flat = tune.flat != 0;
  if (tune.tma >= 0) e->tma = tune.tma != 0;
}

// The passes of a 3D c2c (src/fft_common_3d.f90:9-116): x, y, z (forward
// in PHYSICAL_IN_X, backward in PHYSICAL_IN_Z) or z, y, x, the first from
// `in` to `out`, the others in place in `out`; none when every axis is
// skipped (the call is then a copy).
std::vector<Pass> c2c_passes(gbfft_engine_s* e, const void* d_in, void* d_out, int isign) {
  const int n1 = e->nx, n2 = e->ny, n3 = e->nz;
  const bool x_first = (e->format == GBFFT_PHYSICAL_IN_X && isign == GBFFT_FORWARD) ||
                       (e->format == GBFFT_PHYSICAL_IN_Z && isign == GBFFT_BACKWARD);
  const int order_f[3] = {0, 1, 2}, order_b[3] = {2, 1, 0};
  const int* order = x_first ? order_f : order_b;
  const int inv = isign == GBFFT_BACKWARD ? 1 : 0;
  std::vector<Pass> ps;
  const void* cur = d_in;
  for (int i = 0; i < 3; ++i) {
    const int ax = order[i];
    if (e->skip[ax]) continue;
    ps.push_back(c2c_pass(e, ax, n1, n2, n3, cur, d_out, inv, n1, n1));
    cur = d_out;
  }
  return ps;
}

// With the padded layout every pass but the last writes the work area (rows
// padded to aligned starts) and the last one writes `out`; otherwise all
// passes work in `out`, which needs no work area.
std::vector<Pass> r2c_passes(gbfft_engine_s* e, const void* d_in, void* d_out) {
  std::vector<Pass> ps;
  const int s1 = e->sp[0], s2 = e->sp[1], s3 = e->sp[2];
  const int order_x[2] = {1, 2}, order_z[2] = {1, 0};
  const int* order = e->format == GBFFT_PHYSICAL_IN_X ? order_x : order_z;
  int axes[2], na = 0;
  for (int i = 0; i < 2; ++i)
    if (!e->skip[order[i]]) axes[na++] = order[i];
  void* W = (!e->inplace && e->pad == 1) ? e->work : nullptr;
  const long long wp = W ? work_pitch(e) : s1;
  void* mid = W ? W : d_out;
  ps.push_back(real_pass(e, K_R2C, d_in, na ? mid : d_out, na ? wp : s1));
  const void* cur = na ? mid : d_out;
  long long cp = na ? wp : s1;
  for (int i = 0; i < na; ++i) {
    const bool last = i == na - 1;
    ps.push_back(c2c_pass(e, axes[i], s1, s2, s3, cur, last ? d_out : mid, 0, cp, last ? s1 : wp));
    cur = last ? d_out : mid;
    cp = last ? s1 : wp;
  }
  return ps;
}

// The passes of a 3D c2r (src/fft_common_3d.f90:194-296): c2c passes into
// the work array W (the input itself when OVERWRITE), then the c2r pass.
std::vector<Pass> c2r_passes(gbfft_engine_s* e, void* d_in, void* d_out) {
  std::vector<Pass> ps;
  void* W = e->inplace ? d_in : e->work;
  const int s1 = e->sp[0], s2 = e->sp[1], s3 = e->sp[2];
  const long long wp = e->inplace ? s1 : work_pitch(e);
  const void* cur = d_in;
  long long cp = s1;
  const int order_x[2] = {2, 1};  // PHYSICAL_IN_X: z then y, then c2r along x
  const int order_z[2] = {0, 1};  // PHYSICAL_IN_Z: x then y, then c2r along z
  const int* order = e->format == GBFFT_PHYSICAL_IN_X ? order_x : order_z;
  for (int i = 0; i < 2; ++i) {
    const int ax = order[i];
    if (e->skip[ax]) continue;
    ps.push_back(c2c_pass(e, ax, s1, s2, s3, cur, W, 1, cp, wp));
    cur = W;
    cp = wp;
  }
  ps.push_back(real_pass(e, K_C2R, cur, d_out, cp));
  return ps;
}

}  // namespace

int gbfft::engine_passes(gbfft_engine_s* e, int which, const void* in, void* out, PassInfo* out_passes,
                         int max_passes, int* n) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (which == 1 && !(e->inplace ? in : e->work)) return fail(GBFFT_ERR_STATE, "engine has no work area");
  std::vector<Pass> ps =
      which == 0 ? r2c_passes(e, in, out) : c2r_passes(e, const_cast<void*>(in), out);
  if ((int)ps.size() > max_passes) return fail(GBFFT_ERR_INVALID, "too many passes");
  for (size_t i = 0; i < ps.size(); ++i) {
    PassInfo q{ps[i].a, ps[i].kind, ps[i].contiguous};
    // the batch kernel's power-of-two plans are batch_points(n) points a thread
    if (q.a.fast == 1)
      for (const AxisPlan& ax : e->ax)
        if (q.a.tw == ax.d_twf && ax.d_twfb) {
          q.a.tw = ax.d_twfb;
          q.a.tpl = q.a.n / batch_points(q.a.n);
        }
    out_passes[i] = q;
  }
  *n = (int)ps.size();
  return GBFFT_OK;
}

int gbfft::engine_precision(gbfft_engine_s* e) { return valid_engine(e) ? e->prec : 0; }

std::atomic<long long> g_live_allocs{0};

cudaError_t gbfft::dev_free(void* p) {
  if (!p) return cudaSuccess;
  cudaError_t e = cudaFree(p);
  if (e == cudaSuccess) g_live_allocs.fetch_sub(1);
  return e;
}

long long gbfft_debug_live_allocations(void) { return g_live_allocs.load(); }

cudaError_t gbfft::dev_malloc(void** p, size_t bytes) {
  long long v = g_fail_alloc.load();
  while (v >= 0) {
    const long long next = v == 0 ? -1 : v - 1;
    if (g_fail_alloc.compare_exchange_weak(v, next)) {
      if (v == 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) g_live_allocs.fetch_add(1);
  return e;
}

int gbfft::set_error(int code, const char* msg) {
  g_err = msg ? msg : "";
  return code;
}

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* gbfft_last_error_string(void) { return g_err.c_str(); }

int gbfft_warning_count(void) { return g_warnings.load(); }

int gbfft_version(int* major, int* minor) {
  if (major) *major = 0;
  if (minor) *minor = 1;
  return GBFFT_OK;
}

long long gbfft_launch_count(void) { return launch_counter(); }

long long gbfft_tma_pass_count(void) { return tma_launch_counter(); }
long long gbfft_tc_pass_count(void) { return tc_launch_counter(); }

int gbfft_debug_fail_alloc(long long nth) {
  if (nth < -1) return fail(GBFFT_ERR_INVALID, "bad argument");
  g_fail_alloc.store(nth);
  return GBFFT_OK;
}

int gbfft_set_nvtx(int enable) {
  g_nvtx.store(enable ? 1 : 0);
  return GBFFT_OK;
}

int gbfft_debug_bounds_build(void) {
#ifdef GB_DEBUG_BOUNDS
  return 1;
#else
  return 0;
#endif
}

int gbfft_malloc(void** d_ptr, size_t bytes) {
  if (!d_ptr) return fail(GBFFT_ERR_INVALID, "gbfft_malloc: null output pointer");
  *d_ptr = nullptr;
  if (bytes == 0) return GBFFT_OK;
  cudaError_t e = dev_malloc(d_ptr, bytes);
  if (e != cudaSuccess) {
    *d_ptr = nullptr;
    g_err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return GBFFT_ERR_ALLOC;
  }
  return GBFFT_OK;
}

int gbfft_free(void* d_ptr) {
  if (!d_ptr) return GBFFT_OK;
  cudaError_t e = dev_free(d_ptr);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFree");
  return GBFFT_OK;
}

int gbfft_engine_create(int format, int nx, int ny, int nz, int inplace, const int* skip, int prec,
                        int form, gbfft_engine_t* engine) {
  if (!engine) return fail(GBFFT_ERR_INVALID, "engine output pointer is null");
  *engine = nullptr;
  int rc = check_engine_args(format, nx, ny, nz, prec, form);
  if (rc != GBFFT_OK) return rc;
  gbfft_engine_s* e = new (std::nothrow) gbfft_engine_s();
  if (!e) return fail(GBFFT_ERR_ALLOC, "host allocation failed");
  TuneEntry tune;
  rc = engine_init_host(e, format, nx, ny, nz, inplace, skip, prec, form, &tune);
  if (rc != GBFFT_OK) {
    delete e;
    return rc;
  }
  for (int d = 0; d < 3; ++d) {
    rc = upload_twiddles(e->ax[d], prec);
    if (rc != GBFFT_OK) {
      release(e);
      delete e;
      return rc;
    }
  }
  // work area: the complex intermediate of r2c and c2r with padded rows,
  // unless the transforms must work in the arrays they are given
  if (!e->inplace) {
    e->work_bytes = (size_t)padded_pitch(e) * e->sp[1] * e->sp[2] * cbytes(e);
    cudaError_t err = dev_malloc(&e->work, e->work_bytes);
    if (err != cudaSuccess) {
      e->work = nullptr;
      release(e);
      delete e;
      g_err = std::string("cudaMalloc(work area): ") + cudaGetErrorString(err);
      return GBFFT_ERR_ALLOC;
    }
  }
  // counters of the fused x/y kernel: one per z-plane plus ticket and status
  if (prec == GBFFT_PREC_SINGLE && fast_length(nx) && fast_length(ny)) {
    e->sync_planes = nz;
    cudaError_t err = dev_malloc((void**)&e->d_sync, (size_t)(nz + 2) * sizeof(int));
    if (err != cudaSuccess) {
      e->d_sync = nullptr;
      release(e);
      delete e;
      g_err = std::string("cudaMalloc(counters): ") + cudaGetErrorString(err);
      return GBFFT_ERR_ALLOC;
    }
    cudaMemset(e->d_sync, 0, (size_t)(nz + 2) * sizeof(int));
  }
  {
    cudaError_t err = dev_malloc((void**)&e->d_status, 4 * sizeof(int));
    if (err != cudaSuccess) {
      e->d_status = nullptr;
      release(e);
      delete e;
      g_err = std::string("cudaMalloc(status word): ") + cudaGetErrorString(err);
      return GBFFT_ERR_ALLOC;
    }
    cudaMemset(e->d_status, 0, 4 * sizeof(int));
  }
  // scratch of the long-axis path: two copies of the largest pass's lines,
  // at most the whole grid in complex values (any engine may run c2c)
  if (e->ax[0].big || e->ax[1].big || e->ax[2].big) {
    // the chirp-z path keeps lines of m points: at most grid / n lines of a pass
    const size_t grid = (size_t)nx * ny * nz;
    size_t pts = grid;
    for (const AxisPlan& a : e->ax)
      if (a.blue) pts = std::max(pts, grid / (size_t)a.n * (size_t)a.bt.m);
    e->long_scratch_bytes = 2 * pts * cbytes(e);
    cudaError_t err = dev_malloc(&e->long_scratch, e->long_scratch_bytes);
    if (err != cudaSuccess) {
      e->long_scratch = nullptr;
      release(e);
      delete e;
      g_err = std::string("cudaMalloc(long-axis scratch): ") + cudaGetErrorString(err);
      return GBFFT_ERR_ALLOC;
    }
  }
  apply_tune(e, tune);
  g_err.clear();
  *engine = e;
  return GBFFT_OK;
}

int gbfft_engine_destroy(gbfft_engine_t e) {
  if (!e) return GBFFT_OK;
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  release(e);
  e->magic = 0;
  delete e;
  return GBFFT_OK;
}

int gbfft_engine_get_sizes(gbfft_engine_t e, int ph[3], int sp[3]) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  for (int i = 0; i < 3; ++i) {
    if (ph) ph[i] = e->ph[i];
    if (sp) sp[i] = e->sp[i];
  }
  return GBFFT_OK;
}

int gbfft_engine_work_bytes(gbfft_engine_t e, size_t* bytes) {
  if (!valid_engine(e) || !bytes) return fail(GBFFT_ERR_INVALID, "bad argument");
  *bytes = e->work_bytes + e->long_scratch_bytes;
  return GBFFT_OK;
}

int gbfft_exec_r2c(gbfft_engine_t e, const void* d_in, void* d_out, void* stream) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (!d_in || !d_out) return fail(GBFFT_ERR_INVALID, "null array pointer");
  const size_t rb = (size_t)e->nx * e->ny * e->nz * e->prec;
  const size_t cb = (size_t)e->sp[0] * e->sp[1] * e->sp[2] * cbytes(e);
  if (overlap(d_in, rb, d_out, cb))
    return fail(GBFFT_ERR_INVALID, "In-place r2c transform is not yet available");
  if (!aligned(d_in, e->prec) || !aligned(d_out, cbytes(e)))
    return fail(GBFFT_ERR_INVALID, "array not aligned to its element size");
  cudaStream_t st = (cudaStream_t)stream;
  if ((e->format == GBFFT_PHYSICAL_IN_X && e->skip[0]) || (e->format == GBFFT_PHYSICAL_IN_Z && e->skip[2]))
    warn_skip(e->format == GBFFT_PHYSICAL_IN_X ? 1 : 2);
  Range range("fft_r2c");
  std::vector<Pass> ps = r2c_passes(e, d_in, d_out);
  if (e->fuse) fuse_xy(e, ps, e->sp[2]);
  return run_passes(e, ps, st, {{d_in, rb}, {d_out, cb}});
}

int gbfft_exec_c2r(gbfft_engine_t e, void* d_in, void* d_out, void* stream) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (!d_in || !d_out) return fail(GBFFT_ERR_INVALID, "null array pointer");
  const size_t rb = (size_t)e->nx * e->ny * e->nz * e->prec;
  const size_t cb = (size_t)e->sp[0] * e->sp[1] * e->sp[2] * cbytes(e);
  if (overlap(d_in, cb, d_out, rb))
    return fail(GBFFT_ERR_INVALID, "In-place c2r transform is not yet available");
  if (!aligned(d_in, cbytes(e)) || !aligned(d_out, e->prec))
    return fail(GBFFT_ERR_INVALID, "array not aligned to its element size");
  cudaStream_t st = (cudaStream_t)stream;
  if (!(e->inplace ? d_in : e->work)) return fail(GBFFT_ERR_STATE, "engine has no work area");
  if (e->format == GBFFT_PHYSICAL_IN_X && e->skip[0]) warn_skip(3);
  if (e->format == GBFFT_PHYSICAL_IN_Z && e->skip[2]) warn_skip(4);
  Range range("fft_c2r");
  std::vector<Pass> ps = c2r_passes(e, d_in, d_out);
  if (e->fuse) fuse_xy(e, ps, e->sp[2]);
  return run_passes(e, ps, st, {{d_in, cb}, {d_out, rb}});
}

int gbfft_exec_c2c(gbfft_engine_t e, void* d_in, void* d_out, int isign, void* stream) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (!d_in || !d_out) return fail(GBFFT_ERR_INVALID, "null array pointer");
  if (isign != GBFFT_FORWARD && isign != GBFFT_BACKWARD)
    return fail(GBFFT_ERR_INVALID, "Invalid value for isign");
  cudaStream_t st = (cudaStream_t)stream;
  const int n1 = e->nx, n2 = e->ny, n3 = e->nz;
  const size_t bytes = (size_t)n1 * n2 * n3 * cbytes(e);
  if (d_in != d_out && overlap(d_in, bytes, d_out, bytes))
    return fail(GBFFT_ERR_INVALID, "input and output partially overlap");
  if (!aligned(d_in, cbytes(e)) || !aligned(d_out, cbytes(e)))
    return fail(GBFFT_ERR_INVALID, "array not aligned to its element size");
  Range range("fft_c2c");
  std::vector<Pass> ps = c2c_passes(e, d_in, d_out, isign);
  if (ps.empty()) {
    cudaError_t err = launch_copy(d_in, d_out, bytes, st);
    if (err != cudaSuccess) return cuda_fail(err, "copy launch");
    return GBFFT_OK;
  }
  if (e->fuse) fuse_xy(e, ps, n3);
  return run_passes(e, ps, st, {{d_in, bytes}, {d_out, bytes}});
}

int gbfft_transpose(int kind, int is_complex, int prec, const void* d_src, void* d_dst, int n1, int n2,
                    int n3, void* stream) {
  if (kind < GBFFT_X_TO_Y || kind > GBFFT_Y_TO_X) return fail(GBFFT_ERR_INVALID, "Invalid transpose kind");
  if (prec != GBFFT_PREC_SINGLE && prec != GBFFT_PREC_DOUBLE)
    return fail(GBFFT_ERR_INVALID, "Invalid value for precision (4 or 8)");
  if (n1 < 0 || n2 < 0 || n3 < 0) return fail(GBFFT_ERR_INVALID, "negative size");
  const size_t bytes = (size_t)n1 * n2 * n3 * (size_t)prec * (is_complex ? 2 : 1);
  if (bytes == 0) return GBFFT_OK;
  if (!d_src || !d_dst) return fail(GBFFT_ERR_INVALID, "null array pointer");
  if (d_src != d_dst && overlap(d_src, bytes, d_dst, bytes))
    return fail(GBFFT_ERR_INVALID, "source and destination partially overlap");
  cudaError_t err = launch_copy(d_src, d_dst, bytes, (cudaStream_t)stream);
  if (err != cudaSuccess) return cuda_fail(err, "transpose copy launch");
  return GBFFT_OK;
}

int gbfft_engine_set_profiling(gbfft_engine_t e, int enable) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  drop_profile(e);
  for (int k = 0; k < GBFFT_PASS_KINDS; ++k) {
    e->prof_n[k] = 0;
    e->prof_ms[k] = 0;
    e->prof_bytes[k] = 0;
  }
  e->profiling = enable != 0;
  return GBFFT_OK;
}

int gbfft_engine_set_tile(gbfft_engine_t e, int kind, int lines) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (kind < 0 || kind >= GBFFT_PASS_KINDS) return fail(GBFFT_ERR_INVALID, "bad pass kind");
  if (lines < 0 || lines > 64) return fail(GBFFT_ERR_INVALID, "lines per CTA out of range");
  if (lines == 0) {
    e->tile_L[kind] = 0;
    return GBFFT_OK;
  }
  if (kind == GBFFT_PASS_XY) {
    // fused x/y kernel: y lines a tile, 256 or 512 threads a CTA
    const int ty = fast_length(e->ny) ? e->ny / fast_points(e->ny, false) : 0;
    if (ty == 0 || (lines * ty != 256 && lines * ty != 512))
      return fail(GBFFT_ERR_INVALID, "fused tiles have 256 or 512 threads");
    e->tile_L[kind] = lines;
    return GBFFT_OK;
  }
  int axis;
  if (kind == GBFFT_PASS_R2C || kind == GBFFT_PASS_C2R)
    axis = e->format == GBFFT_PHYSICAL_IN_X ? 0 : 2;
  else
    axis = kind - GBFFT_PASS_C2C_X;
  const AxisPlan& p = e->ax[axis];
  if (gen_length(p.n) && p.fast_e == gen_points(p.n)) {
    const int tpl_g = p.n / p.fast_e;
    if (lines * tpl_g > gen_max_threads(p.fast_e, e->prec))
      return fail(GBFFT_ERR_INVALID, "tile exceeds the kernel's thread limit");
    if ((size_t)fast_smem_entries(p.n, lines) * 2 * (size_t)e->prec > 200 * 1024)
      return fail(GBFFT_ERR_INVALID, "tile exceeds the shared-memory limit");
    e->tile_L[kind] = lines;
    return GBFFT_OK;
  }
  if (mixed_length(p.n)) {
    const int tpl_m = p.n / mixed_r0(p.n);
    if (lines * tpl_m > 256) return fail(GBFFT_ERR_INVALID, "tile exceeds the kernel's thread limit");
    if ((size_t)fast_smem_entries(p.n, lines) * 2 * (size_t)e->prec > 200 * 1024)
      return fail(GBFFT_ERR_INVALID, "tile exceeds the shared-memory limit");
    e->tile_L[kind] = lines;
    return GBFFT_OK;
  }
  const bool fast = fast_length(p.n);
  const bool contiguous = (kind == GBFFT_PASS_C2C_X) ||
                          ((kind == GBFFT_PASS_R2C || kind == GBFFT_PASS_C2R) &&
                           e->format == GBFFT_PHYSICAL_IN_X);
  const int fe = p.fast_e;
  int tpl = fast ? p.n / fe : p.tpl;
  const int maxt = fast ? fast_max_threads(fe, e->prec) : kMaxThreads;
  if (!fast && !contiguous)
    while (lines * tpl > kMaxThreads && tpl > 32) tpl /= 2;
  if (lines * tpl > maxt) return fail(GBFFT_ERR_INVALID, "tile exceeds the kernel's thread limit");
  const size_t smem = fast ? (size_t)fast_smem_entries(p.n, lines) * 2 * (size_t)e->prec
                            : pass_smem_bytes(e->prec, p.n, lines);
  if (smem > 200 * 1024) return fail(GBFFT_ERR_INVALID, "tile exceeds the shared-memory limit");
  e->tile_L[kind] = lines;
  return GBFFT_OK;
}

int gbfft_engine_set_cluster(gbfft_engine_t e, int kind, int ctas, int sync) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (kind < 0 || kind >= GBFFT_PASS_KINDS) return fail(GBFFT_ERR_INVALID, "bad pass kind");
  if (ctas != 0 && ctas != 2 && ctas != 4 && ctas != 8)
    return fail(GBFFT_ERR_INVALID, "cluster size must be 0, 2, 4 or 8");
  e->csize[kind] = ctas;
  e->csync[kind] = ctas ? (sync != 0) : 0;
  return GBFFT_OK;
}

int gbfft_engine_get_cluster(gbfft_engine_t e, int* ctas, int* sync) {
  if (!valid_engine(e) || !ctas || !sync) return fail(GBFFT_ERR_INVALID, "bad argument");
  for (int k = 0; k < GBFFT_PASS_KINDS; ++k) {
    ctas[k] = e->csize[k];
    sync[k] = e->csync[k];
  }
  return GBFFT_OK;
}

int gbfft_engine_status(gbfft_engine_t e) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  int flag = 0;
  if (e->d_status) {
    cudaError_t err = cudaMemcpy(&flag, e->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMemcpy(status)");
    if (flag == 2) return fail(GBFFT_ERR_BOUNDS, "a bounds check caught an access outside its array (skipped)");
    if (flag) return fail(GBFFT_ERR_TIMEOUT, "a pass gave up waiting for its bulk tensor copies");
  }
  if (!e->d_sync) return GBFFT_OK;
  cudaError_t err = cudaMemcpy(&flag, e->d_sync + 1, sizeof(int), cudaMemcpyDeviceToHost);
  if (err != cudaSuccess) return cuda_fail(err, "cudaMemcpy(status)");
  if (flag) return fail(GBFFT_ERR_TIMEOUT, "a fused pass gave up waiting for its plane");
  return GBFFT_OK;
}

int gbfft_engine_set_tma(gbfft_engine_t e, int enable) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  e->tma = enable != 0;
  return GBFFT_OK;
}

int gbfft_engine_get_tma(gbfft_engine_t e, int* enable) {
  if (!valid_engine(e) || !enable) return fail(GBFFT_ERR_INVALID, "bad argument");
  *enable = e->tma ? 1 : 0;
  return GBFFT_OK;
}

int gbfft_selftest_bounded_wait(int counter_value, int need, long long poll_limit, int* timed_out) {
  if (!timed_out || poll_limit < 1 || poll_limit > (1ll << 26)) return fail(GBFFT_ERR_INVALID, "bad argument");
  int* d = nullptr;
  cudaError_t err = dev_malloc((void**)&d, 2 * sizeof(int));
  if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc");
  int h[2] = {counter_value, 0};
  err = cudaMemcpy(d, h, sizeof h, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = launch_wait_selftest(d, need, poll_limit, nullptr);
  if (err == cudaSuccess) err = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  dev_free(d);
  if (err != cudaSuccess) return cuda_fail(err, "bounded-wait self-test");
  *timed_out = h[1];
  return GBFFT_OK;
}

int gbfft_tune_cache_path(const char* path) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_path_set = path != nullptr;
  g_tune_path_override = path ? path : "";
  g_tune_loaded = false;
  return GBFFT_OK;
}

int gbfft_engine_set_plan(gbfft_engine_t e, int axis, int points) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (axis < 0 || axis > 2) return fail(GBFFT_ERR_INVALID, "bad axis");
  AxisPlan& p = e->ax[axis];
  if (e->form != GBFFT_FORM_PLAIN && split_length(p.n))
    return fail(GBFFT_ERR_UNSUPPORTED, "the split form has one plan");
  if (gen_length(p.n)) {
    if (points != gen_points(p.n) && points != 2)
      return fail(GBFFT_ERR_INVALID, "points per thread must be the balanced plan's or 2 (two-stage plan)");
  } else {
    if (!fast_has_alt(p.n)) return fail(GBFFT_ERR_UNSUPPORTED, "this axis length has one plan");
    if (!fast_e_ok(p.n, points))
      return fail(GBFFT_ERR_INVALID, "points per thread must be 32 or 16 (512 and 1024 points) or 16, 8, 4 "
                                     "(8: at most 256 points, 4: at most 128)");
  }
  if (p.fast_e == points) return GBFFT_OK;
  void* old = p.d_twf;
  const int old_e = p.fast_e;
  p.fast_e = points;
  p.d_twf = nullptr;
  int rc = upload_table(&p.d_twf, stage_twiddles(plan_radices(p)), e->prec);
  if (rc != GBFFT_OK) {
    p.fast_e = old_e;
    p.d_twf = old;
    return rc;
  }
  cudaDeviceSynchronize();  // no pass still reads the old table
  if (old) dev_free(old);
  if ((rc = upload_batch_table(p, e->prec)) != GBFFT_OK) return rc;
  for (int k = 0; k < GBFFT_PASS_KINDS; ++k) e->tile_L[k] = 0;  // tiles were sized for the old plan
  return GBFFT_OK;
}

int gbfft_engine_get_tuning(gbfft_engine_t e, int* fuse, int* tiles, int* points) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (fuse) *fuse = e->fuse ? 1 : 0;
  if (tiles)
    for (int k = 0; k < GBFFT_PASS_KINDS; ++k) tiles[k] = e->tile_L[k];
  if (points)
    for (int d = 0; d < 3; ++d)
      points[d] = (fast_length(e->ax[d].n) || gen_length(e->ax[d].n)) ? e->ax[d].fast_e : 0;
  return GBFFT_OK;
}

int gbfft_engine_set_layout(gbfft_engine_t e, int pad, int flat) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (pad < 0 || pad > 2) return fail(GBFFT_ERR_INVALID, "pad must be 0, 1 or 2");
  e->pad = pad;
  e->flat = flat != 0;
  return GBFFT_OK;
}

int gbfft_engine_get_layout(gbfft_engine_t e, int* pad, int* flat) {
  if (!valid_engine(e) || !pad || !flat) return fail(GBFFT_ERR_INVALID, "bad argument");
  *pad = e->pad;
  *flat = e->flat ? 1 : 0;
  return GBFFT_OK;
}

int gbfft_plan_describe(int format, int nx, int ny, int nz, int inplace, const int* skip, int prec, int pad,
                        int flat, int which, gbfft_pass_desc_t* out, int max_passes, int* n_passes) {
  if (!n_passes || (max_passes > 0 && !out)) return fail(GBFFT_ERR_INVALID, "null output pointer");
  *n_passes = 0;
  int rc = check_engine_args(format, nx, ny, nz, prec, GBFFT_FORM_PLAIN);
  if (rc != GBFFT_OK) return rc;
  if (which < 0 || which > 3) return fail(GBFFT_ERR_INVALID, "which must be 0 (r2c), 1 (c2r), 2 or 3 (c2c)");
  if (pad < -1 || pad > 2) return fail(GBFFT_ERR_INVALID, "pad must be -1, 0, 1 or 2");
  gbfft_engine_s e;  // no device memory: tables and work area are never touched
  TuneEntry tune;
  rc = engine_init_host(&e, format, nx, ny, nz, inplace, skip, prec, GBFFT_FORM_PLAIN, &tune);
  if (rc != GBFFT_OK) return rc;
  apply_tune(&e, tune);
  if (pad >= 0) e.pad = pad;
  if (flat >= 0) e.flat = flat != 0;
  // stand-in addresses of the three arrays, never dereferenced (aligned like
  // device allocations, so that the vector-access choices are the real ones)
  char* const in = reinterpret_cast<char*>(uintptr_t(1) << 40);
  char* const outp = in + (uintptr_t(1) << 40);
  char* const work = outp + (uintptr_t(1) << 40);
  e.work = e.inplace ? nullptr : work;
  std::vector<Pass> ps;
  if (which == 0) ps = r2c_passes(&e, in, outp);
  else if (which == 1) ps = c2r_passes(&e, in, outp);
  else ps = c2c_passes(&e, in, outp, which == 2 ? GBFFT_FORWARD : GBFFT_BACKWARD);
  e.work = nullptr;
  auto buffer = [&](const void* p) { return p == in ? 0 : p == outp ? 1 : p == work ? 2 : -1; };
  for (size_t i = 0; i < ps.size() && (int)i < max_passes; ++i) {
    const PassArgs& a = ps[i].a;
    gbfft_pass_desc_t& d = out[i];
    d.kind = ps[i].kind;
    d.contiguous = ps[i].contiguous ? 1 : 0;
    d.n = a.n;
    d.nlines = a.nlines;
    d.real_lines = a.real_lines;
    d.nv = a.nv;
    d.row_w = a.row_w;
    d.s_src_n = a.s_src_n;
    d.s_src_l = a.s_src_l;
    d.s_src_r = a.s_src_r;
    d.s_dst_n = a.s_dst_n;
    d.s_dst_l = a.s_dst_l;
    d.s_dst_r = a.s_dst_r;
    d.src = buffer(a.src);
    d.dst = buffer(a.dst);
  }
  *n_passes = (int)ps.size();
  return GBFFT_OK;
}

int gbfft_engine_set_fusion(gbfft_engine_t e, int enable) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  e->fuse = enable != 0;
  return GBFFT_OK;
}

int gbfft_engine_profile_read(gbfft_engine_t e, int kind, long long* launches, double* ms,
                              double* bytes) {
  if (!valid_engine(e)) return fail(GBFFT_ERR_INVALID, "not an engine");
  if (kind < 0 || kind >= GBFFT_PASS_KINDS) return fail(GBFFT_ERR_INVALID, "bad pass kind");
  for (auto& r : e->prof) {
    cudaError_t err = cudaEventSynchronize(r.stop);
    if (err != cudaSuccess) return cuda_fail(err, "cudaEventSynchronize");
    float t = 0;
    cudaEventElapsedTime(&t, r.start, r.stop);
    e->prof_n[r.kind] += 1;
    e->prof_ms[r.kind] += t;
    e->prof_bytes[r.kind] += r.bytes;
  }
  drop_profile(e);
  if (launches) *launches = e->prof_n[kind];
  if (ms) *ms = e->prof_ms[kind];
  if (bytes) *bytes = e->prof_bytes[kind];
  return GBFFT_OK;
}

}  // extern "C"

// ===========================================================================
// Real-to-real transforms (decomp_2d_dtt_3d_r2r, src/fft_fftw3_f03.f90:
// 341-471 configuration, 1555-1656 the 1D passes, 1959-2023 the 3D driver)
// ===========================================================================

namespace {

constexpr unsigned kDttMagic = 0x47424454u;  // "GBDT"

struct DttAxis {
  int kind = 0, off = 0, n = 0, M = 0;
  AxisPlan plan;        // radix stages of M
  void* tw = nullptr;   // exp(-2 pi i m / M)
  void* twf = nullptr;  // power-of-two M: stage-major table of the 16-point plan
  void* w4 = nullptr;   // exp(-2 pi i m / (4 n)), m < n
  double c0x = 1, c0y = 0;
};

}  // namespace

struct gbfft_dtt_s {
  unsigned magic = kDttMagic;
  int format = GBFFT_PHYSICAL_IN_X;
  int nx = 0, ny = 0, nz = 0, prec = 8;
  int skip[3] = {0, 0, 0};
  int cfg[15] = {0};
  DttAxis ax[2][3];  // [forward, backward][x, y, z]
};

namespace {

bool valid_dtt(gbfft_dtt_t d) { return d != nullptr && d->magic == kDttMagic; }

void release_dtt(gbfft_dtt_t d) {
  for (auto& dir : d->ax)
    for (DttAxis& a : dir) {
      if (a.tw) dev_free(a.tw);
      if (a.twf) dev_free(a.twf);
      if (a.w4) dev_free(a.w4);
      a.tw = a.twf = a.w4 = nullptr;
    }
}

// The reference's configuration: dtt_assign_default (windows),
// dtt_invert (backward kinds); src/fft_fftw3_f03.f90:341-455.
int dtt_config(const int* in, int nin, int* c) {
  if (!in || nin < 3) return fail(GBFFT_ERR_INVALID, "Invalid argument");
  for (int k = 0; k < 3; ++k)
    if (in[k] < 1 || in[k] > 8) return fail(GBFFT_ERR_INVALID, "Invalid argument");
  for (int k = 0; k < 15; ++k) c[k] = 0;
  if (nin == 12) {
    for (int k = 0; k < 12; ++k) c[k] = in[k];
    for (int k = 0; k < 3; ++k)
      if (c[3 + k] != c[9 + k])
        return fail(GBFFT_ERR_INVALID, "Setup is not compatible with in-place r2r transforms");
  } else if (nin == 3) {
    for (int k = 0; k < 3; ++k) {
      c[k] = in[k];
      c[3 + k] = 1;  // ifirst
      c[6 + k] = 1;  // ndismiss
      if (c[k] == 1) c[6 + k] = 0;  // DCT-I
      if (c[k] == 5) {              // DST-I
        c[3 + k] = 2;
        c[6 + k] = 2;
      }
      if (c[k] == 7) c[3 + k] = 2;  // DST-III
      c[9 + k] = c[3 + k];
    }
  } else {
    return fail(GBFFT_ERR_INVALID, "Invalid argument");
  }
  static const int inverse[9] = {0, 1, 3, 2, 4, 5, 7, 6, 8};
  for (int k = 0; k < 3; ++k) c[12 + k] = inverse[c[k]];
  return GBFFT_OK;
}

int setup_dtt_axis(DttAxis& a, int kind, int first, int ndismiss, int naxis, int prec) {
  a.kind = kind;
  a.off = first - 1;
  a.n = naxis - ndismiss;
  if (a.off < 0 || a.n < 1 || a.off + a.n > naxis || (kind == 1 && a.n < 2))
    return fail(GBFFT_ERR_INVALID, "r2r window outside the axis");
  a.M = kind == 1 ? 2 * (a.n - 1) : kind == 5 ? 2 * (a.n + 1) : 2 * a.n;
  std::string why;
  if (!factorize(a.M, a.plan, why)) return fail(GBFFT_ERR_UNSUPPORTED, "r2r extension: " + why);
  if (a.M > kMaxN || dtt_smem_bytes(prec, a.M, 1) > 200 * 1024)
    return fail(GBFFT_ERR_UNSUPPORTED, "r2r extension does not fit one shared-memory tile");
  int rc = upload_table(&a.tw, twiddles(a.M), prec);
  if (rc != GBFFT_OK) return rc;
  // the two-stage plan in FP32 only: in FP64 its 30-point butterflies take
  // 210 registers a thread and the 510-point pass ran slower than the
  // runtime-planned one
  const bool mixed = dtt_mixed_length(a.M) && prec == GBFFT_PREC_SINGLE;
  if (dtt_fast_length(a.M) || mixed) {
    std::vector<int> radices;
    if (mixed) {
      radices = {mixed_r0(a.M), a.M / mixed_r0(a.M)};
    } else {
      for (int s = 0; s < fast_nst(a.M, 16); ++s) radices.push_back(fast_radix(a.M, 16, s));
    }
    rc = upload_table(&a.twf, stage_twiddles(radices), prec);
    if (rc != GBFFT_OK) return rc;
  }
  std::vector<double> w = twiddles(4 * a.n);
  w.resize(2 * (size_t)a.n);
  rc = upload_table(&a.w4, w, prec);
  if (rc != GBFFT_OK) return rc;
  const long double pi = 3.141592653589793238462643383279502884L;
  a.c0x = (double)cosl(pi / (4.0L * a.n));
  a.c0y = (double)(-sinl(pi / (4.0L * a.n)));
  return GBFFT_OK;
}

}  // namespace

extern "C" {

int gbfft_dtt_create(int format, int nx, int ny, int nz, const int* skip, int prec, const int* dtt, int ndtt,
                     gbfft_dtt_t* out) {
  if (!out) return fail(GBFFT_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (format != GBFFT_PHYSICAL_IN_X && format != GBFFT_PHYSICAL_IN_Z)
    return fail(GBFFT_ERR_INVALID, "Invalid value for pencil");
  if (nx <= 0) return fail(GBFFT_ERR_INVALID, "Invalid value for nx");
  if (ny <= 0) return fail(GBFFT_ERR_INVALID, "Invalid value for ny");
  if (nz <= 0) return fail(GBFFT_ERR_INVALID, "Invalid value for nz");
  if (prec != GBFFT_PREC_SINGLE && prec != GBFFT_PREC_DOUBLE) return fail(GBFFT_ERR_INVALID, "bad precision");
  gbfft_dtt_t d = new gbfft_dtt_s;
  d->format = format;
  d->nx = nx;
  d->ny = ny;
  d->nz = nz;
  d->prec = prec;
  for (int k = 0; k < 3; ++k) d->skip[k] = skip ? (skip[k] != 0) : 0;
  int rc = dtt_config(dtt, ndtt, d->cfg);
  const int lens[3] = {nx, ny, nz};
  for (int dir = 0; dir < 2 && rc == GBFFT_OK; ++dir)
    for (int k = 0; k < 3 && rc == GBFFT_OK; ++k) {
      if (d->skip[k]) continue;
      const int kind = d->cfg[dir == 0 ? k : 12 + k];
      const int first = d->cfg[dir == 0 ? 3 + k : 9 + k];
      rc = setup_dtt_axis(d->ax[dir][k], kind, first, d->cfg[6 + k], lens[k], prec);
    }
  if (rc != GBFFT_OK) {
    const std::string msg = g_err;
    release_dtt(d);
    d->magic = 0;
    delete d;
    g_err = msg;
    return rc;
  }
  g_err.clear();
  *out = d;
  return GBFFT_OK;
}

int gbfft_dtt_destroy(gbfft_dtt_t d) {
  if (!d) return GBFFT_OK;
  if (!valid_dtt(d)) return fail(GBFFT_ERR_INVALID, "not an r2r engine");
  release_dtt(d);
  d->magic = 0;
  delete d;
  return GBFFT_OK;
}

int gbfft_dtt_get_config(gbfft_dtt_t d, int* cfg) {
  if (!valid_dtt(d) || !cfg) return fail(GBFFT_ERR_INVALID, "bad argument");
  for (int k = 0; k < 15; ++k) cfg[k] = d->cfg[k];
  return GBFFT_OK;
}

int gbfft_exec_r2r(gbfft_dtt_t d, void* d_in, void* d_out, int isign, void* stream) {
  if (!valid_dtt(d)) return fail(GBFFT_ERR_INVALID, "not an r2r engine");
  if (!d_in || !d_out) return fail(GBFFT_ERR_INVALID, "null array pointer");
  if (isign != GBFFT_FORWARD && isign != GBFFT_BACKWARD) return fail(GBFFT_ERR_INVALID, "Invalid value");
  const size_t bytes = (size_t)d->nx * d->ny * d->nz * d->prec;
  if (d_in != d_out && overlap(d_in, bytes, d_out, bytes))
    return fail(GBFFT_ERR_INVALID, "input and output partially overlap");
  if (!aligned(d_in, d->prec) || !aligned(d_out, d->prec))
    return fail(GBFFT_ERR_INVALID, "array not aligned to its element size");
  cudaStream_t st = (cudaStream_t)stream;
  const int dir = isign == GBFFT_FORWARD ? 0 : 1;
  const bool x_first = (d->format == GBFFT_PHYSICAL_IN_X) == (isign == GBFFT_FORWARD);
  const int order[3] = {x_first ? 0 : 2, 1, x_first ? 2 : 0};
  const long long nx = d->nx, ny = d->ny, nz = d->nz;
  for (int i = 0; i < 3; ++i) {
    const int k = order[i];
    // the first pass in place on the input, the second into the output
    // (the transposes at one rank), the third in place on the output
    void* src = i == 0 ? d_in : (i == 1 ? d_in : d_out);
    void* dst = i == 0 ? d_in : d_out;
    if (d->skip[k]) {
      if (src != dst) {
        cudaError_t err = launch_copy(src, dst, bytes, st);
        if (err != cudaSuccess) return cuda_fail(err, "copy launch");
      }
      continue;
    }
    const DttAxis& ax = d->ax[dir][k];
    DttArgs a;
    std::memset(&a, 0, sizeof(a));
    a.src = src;
    a.dst = dst;
    a.off = ax.off;
    a.n = ax.n;
    a.kind = ax.kind;
    a.M = ax.M;
    a.nst = ax.plan.nst;
    for (int s = 0; s < kMaxStages; ++s) a.radix[s] = s < ax.plan.nst ? ax.plan.radix[s] : 0;
    a.tw = ax.tw;
    a.twf = ax.twf;
    a.w4 = ax.w4;
    a.c0x = ax.c0x;
    a.c0y = ax.c0y;
    const bool contiguous = k == 0;
    if (k == 0) {
      a.sn = 1;
      a.sl = nx;
      a.nlines = ny * nz;
      a.nv = 1;
      a.naxis = (int)nx;
    } else if (k == 1) {
      a.sn = nx;
      a.sl = nx * ny;
      a.nlines = nx;
      a.nv = (int)nz;
      a.naxis = (int)ny;
    } else {
      a.sn = nx * ny;
      a.sl = nx;
      a.nlines = nx;
      a.nv = (int)ny;
      a.naxis = (int)nz;
    }
    if (ax.twf && dtt_mixed_length(ax.M)) {
      // compile-time two-stage plan: R1 threads a line, at most 256 a CTA;
      // contiguous about 128, strided up to 16 neighbouring lines
      const int tplm = ax.M / mixed_r0(ax.M);
      int Lm = contiguous ? (tplm >= 128 ? 1 : 128 / tplm) : 16;
      while (Lm > 1 && Lm * tplm > 256) --Lm;
      while (Lm > 1 && (size_t)fast_smem_entries(ax.M, Lm) * 2 * d->prec > 100 * 1024) --Lm;
      if (a.nlines < Lm) Lm = (int)a.nlines;
      a.L = Lm;
      a.tpl = tplm;
      cudaError_t err = launch_dtt_pass(d->prec, contiguous, a, st);
      if (err != cudaSuccess) return cuda_fail(err, "r2r pass launch");
      continue;
    }
    if (ax.twf) {
      // compile-time 16-point plan: M / 16 threads a line; contiguous
      // 128-thread CTAs, strided up to 16 neighbouring lines
      const int tplf = ax.M / 16, maxt = fast_max_threads(16, d->prec);
      int Lf = contiguous ? (tplf >= 128 ? 1 : 128 / tplf) : 16;
      while (Lf > 1 && Lf * tplf > maxt) --Lf;
      while (Lf > 1 && (size_t)fast_smem_entries(ax.M, Lf) * 2 * d->prec > 100 * 1024) --Lf;
      if (a.nlines < Lf) Lf = (int)a.nlines;
      a.L = Lf;
      a.tpl = tplf;
      cudaError_t err = launch_dtt_pass(d->prec, contiguous, a, st);
      if (err != cudaSuccess) return cuda_fail(err, "r2r pass launch");
      continue;
    }
    // about 8 points of the extension a thread; contiguous: 128-thread CTAs,
    // strided: 16 neighbouring lines (64-byte row segments in FP32)
    int tpl = (ax.M + 7) / 8;
    if (tpl < 1) tpl = 1;
    int L;
    if (contiguous) {
      if (tpl > kMaxThreads) tpl = kMaxThreads;
      L = 128 / tpl;
      if (L < 1) L = 1;
    } else {
      L = 16;
      while (L * tpl > kMaxThreads && tpl > 16) tpl /= 2;
      while (L > 1 && L * tpl > kMaxThreads) L /= 2;
    }
    while (L > 1 && dtt_smem_bytes(d->prec, ax.M, L) > 100 * 1024) --L;
    if (a.nlines < L) L = (int)a.nlines;
    a.L = L;
    a.tpl = tpl;
    cudaError_t err = launch_dtt_pass(d->prec, contiguous, a, st);
    if (err != cudaSuccess) return cuda_fail(err, "r2r pass launch");
  }
  return GBFFT_OK;
}

}  // extern "C"
