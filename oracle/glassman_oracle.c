/*
 * Oracle (test infrastructure only): a CPU restatement of the 2DECOMP&FFT
 * "generic" FFT backend, used as the checker for the GPU path.  Nothing in
 * the product links or calls this file; only tests/, the smoke check and the
 * CPU-baseline leg of bench.py do.
 *
 * What is restated, with the reference lines each function follows:
 *   spcfft_*  / spcpft_*   src/glassman.f90:29-67 and :69-108 (Glassman general-N
 *                          FFT, smallest-factor-first, Horner evaluation, twiddle
 *                          recurrence OMEGA = DELTA*OMEGA, ANGLE constant
 *                          6.28318530717958 evaluated in the working precision).
 *   c2c_1m_{x,y,z}_*       src/fft_generic.f90:112-208 (line gather, spcfft, scatter)
 *   r2c_1m_{x,z}_*         src/fft_generic.f90:211-294 (real line packed as complex,
 *                          full complex FFT, keep the first n/2+1 outputs)
 *   c2r_1m_{x,z}_*         src/fft_generic.f90:297-384 (Hermitian fill
 *                          buf(i)=conj(buf(d+2-i)), inverse FFT, real part)
 *   fft3d_{c2c,r2c,c2r}_*  src/fft_common_3d.f90:9-296 for one rank (dims = 1x1),
 *                          where every transpose_* is the copy of
 *                          src/transpose_x_to_y.f90:41-50 and siblings.
 *
 * Both the double build (mytype = real64) and the single build
 * (mytype = real32) are instantiated: the suffix _d / _s selects them.
 *
 * Arrays are Fortran-ordered (i fastest): a(i,j,k) lives at i + n1*(j + n2*k).
 * Complex values are interleaved (re, im) pairs.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -fPIC -shared (see oracle/build.py).
 * -ffp-contract=off keeps every multiply and add separately rounded, as the
 * Fortran source states them, on both x86-64 and aarch64.
 *
 * Parity status: the reference cannot be compiled here (no Fortran compiler),
 * so this restatement is pinned against the reference's own known-answer
 * tests (round-trip thresholds of examples/fft_physical_{x,z}, the exact
 * transpose chain of examples/test2d) and cross-checked against pocketfft.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#define PHYSICAL_IN_X 1
#define PHYSICAL_IN_Z 3
#define FFT_FORWARD (-1)
#define FFT_BACKWARD 1

/* Work arrays of the 3D drivers come from a pool that persists across calls,
 * as the reference's decomp_pool_get buffers do (src/fft_common_3d.f90:209-230),
 * so that a timed round trip does not pay for fresh pages.  Slot 0: the
 * input-preserving copy (wk1), slot 1: wk2_r2c.  Not thread-safe: one host
 * thread calls the oracle at a time (OpenMP works inside the calls). */
static void* g_pool[2];
static size_t g_pool_bytes[2];

static void* pool_get(int slot, size_t bytes) {
  if (g_pool_bytes[slot] < bytes) {
    free(g_pool[slot]);
    g_pool[slot] = malloc(bytes);
    g_pool_bytes[slot] = g_pool[slot] ? bytes : 0;
  }
  return g_pool[slot];
}

int oracle_pool_release(void) {
  for (int i = 0; i < 2; ++i) {
    free(g_pool[i]);
    g_pool[i] = NULL;
    g_pool_bytes[i] = 0;
  }
  return 0;
}

/* Copy of whole arrays split over the OpenMP threads: at P ranks each rank
 * copies its own pencil, so the P-thread stand-in copies in parallel too. */
static void par_copy(void* dst, const void* src, size_t bytes) {
  if (dst == src) return;
  const char* s = (const char*)src;
  char* d = (char*)dst;
  if ((d < s + bytes) && (s < d + bytes)) {
    memmove(dst, src, bytes);
    return;
  }
  const size_t chunk = (size_t)1 << 20;
  long nch = (long)((bytes + chunk - 1) / chunk);
  _Pragma("omp parallel for schedule(static)")
  for (long c = 0; c < nch; ++c) {
    size_t o = (size_t)c * chunk;
    size_t len = bytes - o < chunk ? bytes - o : chunk;
    memcpy(d + o, s + o, len);
  }
}

#define DEFINE_ORACLE(T, SFX)                                                           \
  typedef struct { T re, im; } cplx_##SFX;                                              \
                                                                                        \
  static inline cplx_##SFX cmul_##SFX(cplx_##SFX a, cplx_##SFX b) {                     \
    cplx_##SFX r;                                                                       \
    r.re = a.re * b.re - a.im * b.im;                                                   \
    r.im = a.re * b.im + a.im * b.re;                                                   \
    return r;                                                                           \
  }                                                                                     \
                                                                                        \
  /* src/glassman.f90:69-108 (SPCPFT): UIN(B,C,A) -> UOUT(B,A,C) */                    \
  static void spcpft_##SFX(int A, int B, int C, const cplx_##SFX* uin,                  \
                           cplx_##SFX* uout, int isign) {                               \
    /* ANGLE = 6.28318530717958_mytype / REAL(A*C, mytype), stored in double */         \
    double angle = (double)((T)6.28318530717958 / (T)(A * C));                          \
    cplx_##SFX omega = {(T)1, (T)0};                                                    \
    cplx_##SFX delta;                                                                   \
    delta.re = (T)cos(angle);                                                           \
    delta.im = (isign == 1) ? (T)sin(angle) : (T)(-sin(angle));                         \
    for (int ic = 0; ic < C; ++ic) {                                                    \
      for (int ia = 0; ia < A; ++ia) {                                                  \
        for (int ib = 0; ib < B; ++ib) {                                                \
          cplx_##SFX sum = uin[ib + (size_t)B * (C - 1) + (size_t)B * C * ia];          \
          for (int jc = C - 2; jc >= 0; --jc) {                                         \
            cplx_##SFX u = uin[ib + (size_t)B * jc + (size_t)B * C * ia];               \
            cplx_##SFX p = cmul_##SFX(omega, sum);                                      \
            sum.re = u.re + p.re;                                                       \
            sum.im = u.im + p.im;                                                       \
          }                                                                             \
          uout[ib + (size_t)B * ia + (size_t)B * A * ic] = sum;                         \
        }                                                                               \
        omega = cmul_##SFX(delta, omega);                                               \
      }                                                                                 \
    }                                                                                   \
  }                                                                                     \
                                                                                        \
  /* src/glassman.f90:29-67 (SPCFFT): unnormalised DFT of U(N), any N */                \
  void spcfft_##SFX(cplx_##SFX* u, int n, int isign, cplx_##SFX* work) {                \
    int a = 1, b = n, c = 1, inu = 1;                                                   \
    while (b > 1) {                                                                     \
      a = c * a;                                                                        \
      c = 2;                                                                            \
      while (b % c != 0) ++c;                                                           \
      b = b / c;                                                                        \
      if (inu) spcpft_##SFX(a, b, c, u, work, isign);                                   \
      else spcpft_##SFX(a, b, c, work, u, isign);                                       \
      inu = !inu;                                                                       \
    }                                                                                   \
    if (!inu) memcpy(u, work, sizeof(cplx_##SFX) * (size_t)n);                          \
  }                                                                                     \
                                                                                        \
  /* 1D entry for tests: n complex values, in place */                                  \
  int oracle_fft1d_##SFX(void* data, int n, int isign) {                                \
    cplx_##SFX* w = (cplx_##SFX*)malloc(sizeof(cplx_##SFX) * (size_t)n);                \
    if (!w) return 1;                                                                   \
    spcfft_##SFX((cplx_##SFX*)data, n, isign, w);                                       \
    free(w);                                                                            \
    return 0;                                                                           \
  }                                                                                     \
                                                                                        \
  /* Line walker shared by every *_1m_* routine: a line of length n starts at   */     \
  /* element offset `base` and advances by `step` elements.                     */     \
  /* src/fft_generic.f90:112-142 (x), :145-175 (y), :178-208 (z)                */     \
  static void c2c_lines_##SFX(cplx_##SFX* a, int n1, int n2, int n3, int axis,          \
                              int isign, long max_lines) {                              \
    int n = axis == 0 ? n1 : (axis == 1 ? n2 : n3);                                     \
    int nu = axis == 0 ? n2 : n1;                                                       \
    int nv = axis == 2 ? n2 : n3;                                                       \
    size_t step = axis == 0 ? 1 : (axis == 1 ? (size_t)n1 : (size_t)n1 * n2);          \
    long nlines = (long)nu * nv;                                                        \
    if (max_lines >= 0 && max_lines < nlines) nlines = max_lines;                       \
    _Pragma("omp parallel")                                                             \
    {                                                                                   \
      cplx_##SFX* buf = (cplx_##SFX*)malloc(sizeof(cplx_##SFX) * (size_t)n);            \
      cplx_##SFX* scr = (cplx_##SFX*)malloc(sizeof(cplx_##SFX) * (size_t)n);            \
      _Pragma("omp for schedule(static)")                                               \
      for (long l = 0; l < nlines; ++l) {                                               \
        int u = (int)(l % nu), v = (int)(l / nu);                                       \
        size_t base;                                                                    \
        if (axis == 0) base = (size_t)n1 * (u + (size_t)n2 * v);                        \
        else if (axis == 1) base = u + (size_t)n1 * n2 * v;                             \
        else base = u + (size_t)n1 * v;                                                 \
        for (int i = 0; i < n; ++i) buf[i] = a[base + step * i];                        \
        spcfft_##SFX(buf, n, isign, scr);                                               \
        for (int i = 0; i < n; ++i) a[base + step * i] = buf[i];                        \
      }                                                                                 \
      free(buf);                                                                        \
      free(scr);                                                                        \
    }                                                                                   \
  }                                                                                     \
                                                                                        \
  /* r2c along axis 0 (x) or 2 (z): src/fft_generic.f90:211-251, :254-294.      */     \
  /* in: real (n1,n2,n3); out: complex with the axis length d = n/2+1.          */     \
  static void r2c_lines_##SFX(const T* in, cplx_##SFX* out, int n1, int n2, int n3,     \
                              int axis, long max_lines) {                               \
    int n = axis == 0 ? n1 : n3;                                                        \
    int d = n / 2 + 1;                                                                  \
    int o1 = axis == 0 ? d : n1, o2 = n2;                                               \
    int nu = axis == 0 ? n2 : n1, nv = axis == 0 ? n3 : n2;                             \
    long nlines = (long)nu * nv;                                                        \
    if (max_lines >= 0 && max_lines < nlines) nlines = max_lines;                       \
    _Pragma("omp parallel")                                                             \
    {                                                                                   \
      cplx_##SFX* buf = (cplx_##SFX*)malloc(sizeof(cplx_##SFX) * (size_t)n);            \
      cplx_##SFX* scr = (cplx_##SFX*)malloc(sizeof(cplx_##SFX) * (size_t)n);            \
      _Pragma("omp for schedule(static)")                                               \
      for (long l = 0; l < nlines; ++l) {                                               \
        int u = (int)(l % nu), v = (int)(l / nu);                                       \
        size_t ib, is, ob, os;                                                          \
        if (axis == 0) {                                                                \
          ib = (size_t)n1 * (u + (size_t)n2 * v); is = 1;                               \
          ob = (size_t)o1 * (u + (size_t)o2 * v); os = 1;                               \
        } else {                                                                        \
          ib = u + (size_t)n1 * v; is = (size_t)n1 * n2;                                \
          ob = u + (size_t)o1 * v; os = (size_t)o1 * o2;                                \
        }                                                                               \
        for (int i = 0; i < n; ++i) { buf[i].re = in[ib + is * i]; buf[i].im = (T)0; }  \
        spcfft_##SFX(buf, n, FFT_FORWARD, scr);                                         \
        for (int i = 0; i < d; ++i) out[ob + os * i] = buf[i];                          \
      }                                                                                 \
      free(buf);                                                                        \
      free(scr);                                                                        \
    }                                                                                   \
  }                                                                                     \
                                                                                        \
  /* c2r along axis 0 (x) or 2 (z): src/fft_generic.f90:297-344, :347-384.      */     \
  /* n1,n2,n3 are the REAL (output) sizes.                                      */     \
  static void c2r_lines_##SFX(const cplx_##SFX* in, T* out, int n1, int n2, int n3,     \
                              int axis, long max_lines) {                               \
    int n = axis == 0 ? n1 : n3;                                                        \
    int d = n / 2 + 1;                                                                  \
    int i1 = axis == 0 ? d : n1, i2 = n2;                                               \
    int nu = axis == 0 ? n2 : n1, nv = axis == 0 ? n3 : n2;                             \
    long nlines = (long)nu * nv;                                                        \
    if (max_lines >= 0 && max_lines < nlines) nlines = max_lines;                       \
    _Pragma("omp parallel")                                                             \
    {                                                                                   \
      cplx_##SFX* buf = (cplx_##SFX*)malloc(sizeof(cplx_##SFX) * (size_t)n);            \
      cplx_##SFX* scr = (cplx_##SFX*)malloc(sizeof(cplx_##SFX) * (size_t)n);            \
      _Pragma("omp for schedule(static)")                                               \
      for (long l = 0; l < nlines; ++l) {                                               \
        int u = (int)(l % nu), v = (int)(l / nu);                                       \
        size_t ib, is, ob, os;                                                          \
        if (axis == 0) {                                                                \
          ib = (size_t)i1 * (u + (size_t)i2 * v); is = 1;                               \
          ob = (size_t)n1 * (u + (size_t)n2 * v); os = 1;                               \
        } else {                                                                        \
          ib = u + (size_t)i1 * v; is = (size_t)i1 * i2;                                \
          ob = u + (size_t)n1 * v; os = (size_t)n1 * n2;                                \
        }                                                                               \
        for (int i = 0; i < d; ++i) buf[i] = in[ib + is * i];                           \
        /* Fortran: do i = d/2+2, d : buf(i) = conjg(buf(d+2-i)), d = n here */         \
        for (int i = n / 2 + 1; i < n; ++i) {                                           \
          buf[i].re = buf[n - i].re;                                                    \
          buf[i].im = -buf[n - i].im;                                                   \
        }                                                                               \
        spcfft_##SFX(buf, n, FFT_BACKWARD, scr);                                        \
        for (int i = 0; i < n; ++i) out[ob + os * i] = buf[i].re;                       \
      }                                                                                 \
      free(buf);                                                                        \
      free(scr);                                                                        \
    }                                                                                   \
  }                                                                                     \
                                                                                        \
  static void copy_##SFX(void* dst, const void* src, size_t bytes) {                    \
    par_copy(dst, src, bytes);                                                          \
  }                                                                                     \
                                                                                        \
  /* src/fft_common_3d.f90:9-116 at dims = (1,1).  `in` is modified when        */     \
  /* inplace != 0 (the reference's intent(INOUT)); skip[3] are the c2c skips.   */     \
  int oracle_fft3d_c2c_##SFX(void* in_, void* out_, int nx, int ny, int nz,             \
                             int format, int isign, int inplace, const int* skip) {     \
    cplx_##SFX* in = (cplx_##SFX*)in_;                                                  \
    cplx_##SFX* out = (cplx_##SFX*)out_;                                                \
    size_t bytes = sizeof(cplx_##SFX) * (size_t)nx * ny * nz;                           \
    int sx = skip ? skip[0] : 0, sy = skip ? skip[1] : 0, sz = skip ? skip[2] : 0;      \
    cplx_##SFX* wk = in;                                                                \
    int fwd_x = (format == PHYSICAL_IN_X && isign == FFT_FORWARD) ||                    \
                (format == PHYSICAL_IN_Z && isign == FFT_BACKWARD);                     \
    if (!inplace) {                                                                     \
      wk = (cplx_##SFX*)pool_get(0, bytes);                                             \
      if (!wk) return 1;                                                                \
      par_copy(wk, in, bytes);                                                          \
    }                                                                                   \
    if (fwd_x) {                                                                        \
      if (!sx) c2c_lines_##SFX(wk, nx, ny, nz, 0, isign, -1);                               \
      if (!sy) c2c_lines_##SFX(wk, nx, ny, nz, 1, isign, -1);                               \
      copy_##SFX(out, wk, bytes); /* transpose_y_to_z */                               \
      if (!sz) c2c_lines_##SFX(out, nx, ny, nz, 2, isign, -1);                              \
    } else {                                                                            \
      if (!sz) c2c_lines_##SFX(wk, nx, ny, nz, 2, isign, -1);                               \
      copy_##SFX(out, wk, bytes); /* transpose_z_to_y */                               \
      if (!sy) c2c_lines_##SFX(out, nx, ny, nz, 1, isign, -1);                              \
      if (!sx) c2c_lines_##SFX(out, nx, ny, nz, 0, isign, -1);                              \
    }                                                                                   \
    return 0;                                                                           \
  }                                                                                     \
                                                                                        \
  /* src/fft_common_3d.f90:121-189 at dims = (1,1): no normalisation.           */     \
  int oracle_fft3d_r2c_##SFX(const T* in, void* out_, int nx, int ny, int nz,           \
                             int format, const int* skip) {                             \
    cplx_##SFX* out = (cplx_##SFX*)out_;                                                \
    int sx = skip ? skip[0] : 0, sy = skip ? skip[1] : 0, sz = skip ? skip[2] : 0;      \
    if (format == PHYSICAL_IN_X) {                                                      \
      int d = nx / 2 + 1;                                                               \
      r2c_lines_##SFX(in, out, nx, ny, nz, 0, -1); /* wk13, then copies: same layout */     \
      if (!sy) c2c_lines_##SFX(out, d, ny, nz, 1, FFT_FORWARD, -1);                         \
      if (!sz) c2c_lines_##SFX(out, d, ny, nz, 2, FFT_FORWARD, -1);                         \
    } else if (format == PHYSICAL_IN_Z) {                                               \
      int d = nz / 2 + 1;                                                               \
      r2c_lines_##SFX(in, out, nx, ny, nz, 2, -1);                                          \
      if (!sy) c2c_lines_##SFX(out, nx, ny, d, 1, FFT_FORWARD, -1);                         \
      if (!sx) c2c_lines_##SFX(out, nx, ny, d, 0, FFT_FORWARD, -1);                         \
    } else {                                                                            \
      return 2;                                                                         \
    }                                                                                   \
    (void)sx; (void)sz;                                                                 \
    return 0;                                                                           \
  }                                                                                     \
                                                                                        \
  /* src/fft_common_3d.f90:194-296 at dims = (1,1).  in_ is the spectral array; */     \
  /* it is modified when inplace != 0.                                           */    \
  int oracle_fft3d_c2r_##SFX(void* in_, T* out, int nx, int ny, int nz, int format,     \
                             int inplace, const int* skip) {                            \
    cplx_##SFX* in = (cplx_##SFX*)in_;                                                  \
    int sx = skip ? skip[0] : 0, sy = skip ? skip[1] : 0, sz = skip ? skip[2] : 0;      \
    int s1 = format == PHYSICAL_IN_X ? nx / 2 + 1 : nx;                                 \
    int s3 = format == PHYSICAL_IN_Z ? nz / 2 + 1 : nz;                                 \
    size_t bytes = sizeof(cplx_##SFX) * (size_t)s1 * ny * s3;                           \
    cplx_##SFX* wk = in;                                                                \
    cplx_##SFX* wk2;                                                                    \
    if (format != PHYSICAL_IN_X && format != PHYSICAL_IN_Z) return 2;                   \
    wk2 = (cplx_##SFX*)pool_get(1, bytes);                                              \
    if (!wk2) return 1;                                                                 \
    if (!inplace) {                                                                     \
      wk = (cplx_##SFX*)pool_get(0, bytes);                                             \
      if (!wk) return 1;                                                                \
      par_copy(wk, in, bytes);                                                          \
    }                                                                                   \
    if (format == PHYSICAL_IN_X) {                                                      \
      if (!sz) c2c_lines_##SFX(wk, s1, ny, s3, 2, FFT_BACKWARD, -1);                        \
      par_copy(wk2, wk, bytes); /* transpose_z_to_y */                                 \
      if (!sy) c2c_lines_##SFX(wk2, s1, ny, s3, 1, FFT_BACKWARD, -1);                       \
      c2r_lines_##SFX(wk2, out, nx, ny, nz, 0, -1);                                         \
    } else {                                                                            \
      if (!sx) c2c_lines_##SFX(wk, s1, ny, s3, 0, FFT_BACKWARD, -1);                        \
      if (!sy) c2c_lines_##SFX(wk, s1, ny, s3, 1, FFT_BACKWARD, -1);                        \
      par_copy(wk2, wk, bytes); /* transpose_y_to_z into wk13 */                       \
      c2r_lines_##SFX(wk2, out, nx, ny, nz, 2, -1);                                         \
    }                                                                                   \
    return 0;                                                                           \
  }

#define DEFINE_SAMPLE(T, SFX)                                                           \
  /* Run one line pass of the generic backend over its first max_lines lines  */       \
  /* (loop order of src/fft_generic.f90), for bounded CPU timing samples.     */       \
  /* kind 0: c2c along axis on `a` (complex n1 x n2 x n3), isign forward;     */       \
  /* kind 1: r2c along axis from real `a` into complex `b`;                   */       \
  /* kind 2: c2r along axis from complex `a` into real `b`.                   */       \
  /* For kinds 1 and 2, n1..n3 are the real sizes.                            */       \
  int oracle_sample_##SFX(int kind, int axis, void* a, void* b, int n1, int n2, int n3,  \
                          long max_lines) {                                            \
    if (kind == 0) c2c_lines_##SFX((cplx_##SFX*)a, n1, n2, n3, axis, FFT_FORWARD,      \
                                   max_lines);                                         \
    else if (kind == 1) r2c_lines_##SFX((const T*)a, (cplx_##SFX*)b, n1, n2, n3, axis, \
                                        max_lines);                                    \
    else if (kind == 2) c2r_lines_##SFX((const cplx_##SFX*)a, (T*)b, n1, n2, n3, axis, \
                                        max_lines);                                    \
    else return 2;                                                                     \
    return 0;                                                                          \
  }

DEFINE_ORACLE(double, d)
DEFINE_ORACLE(float, s)
DEFINE_SAMPLE(double, d)
DEFINE_SAMPLE(float, s)

/* transpose_{x_to_y,y_to_z,z_to_y,y_to_x} at one rank: dst = src
 * (src/transpose_x_to_y.f90:41-50, src/transpose_y_to_z.f90:40-49,
 *  src/transpose_z_to_y.f90:41-47, src/transpose_y_to_x.f90:41). */
int oracle_transpose_copy(void* dst, const void* src, size_t bytes) {
  memmove(dst, src, bytes);
  return 0;
}

#ifdef _OPENMP
#include <omp.h>
#endif
/* Thread count for the line loops (the reference runs one MPI rank per core;
 * here the same line loops are shared by OpenMP threads). */
int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}
