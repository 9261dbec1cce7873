// Mirror of the 2DECOMP&FFT FFT module (src/fft_common.f90) and of the
// one-rank decomposition it sits on (src/decomp_2d_init_fin.f90,
// src/decomp_2d.f90), over the engines of gbfft.h.  The reference keeps its
// state in module variables (fft_engines(:), n_grid, the ph/sp/format
// pointers re-bound by engine%use_it); the same state lives here in one
// host-side table.  Single host thread per process, as in the reference's
// MPI-only model.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "decomp_2d_fft.h"
#include "gbfft_internal.h"

namespace {

struct Grid {
  gbfft_engine_t eng = nullptr;
  gbfft_dtt_t dtt = nullptr;  // opt_DTT given: the r2r transforms of the grid
  bool initialised = false;
  int format = 0, nx = 0, ny = 0, nz = 0, inplace = 0;
};

struct State {
  bool decomp_init = false;
  int nx = 0, ny = 0, nz = 0;  // nx_global, ny_global, nz_global
  int prec = GBFFT_PREC_DOUBLE;
  int default_inplace = 0;
  std::vector<Grid> grids;  // fft_engines(1:n_grid)
  int current = -1;         // index of the grid the module pointers follow
  cudaStream_t stream = nullptr;
} g;

int err(int code, const std::string& m) { return gbfft::set_error(code, m.c_str()); }

void destroy_grid(Grid& gr) {
  if (gr.eng) gbfft_engine_destroy(gr.eng);
  if (gr.dtt) gbfft_dtt_destroy(gr.dtt);
  gr = Grid();
}

const Grid* cur() {
  if (g.current < 0 || g.current >= (int)g.grids.size()) return nullptr;
  const Grid& gr = g.grids[g.current];
  return gr.initialised ? &gr : nullptr;
}

int transpose(const void* src, void* dst, int is_complex, int kind) {
  if (!g.decomp_init) return err(GBFFT_ERR_STATE, "decomp_2d_init must be called first");
  return gbfft_transpose(kind, is_complex, g.prec, src, dst, g.nx, g.ny, g.nz, g.stream);
}

}  // namespace

extern "C" {

int d2d_decomp_2d_init(int nx, int ny, int nz, int p_row, int p_col, int prec) {
  if (g.decomp_init) return err(GBFFT_ERR_STATE, "decomp_2d_init called twice");
  if (nx <= 0 || ny <= 0 || nz <= 0) return err(GBFFT_ERR_INVALID, "Invalid global size");
  if (p_row < 0 || p_col < 0) return err(GBFFT_ERR_INVALID, "Invalid 2D processor grid");
  if ((p_row > 1) || (p_col > 1))
    return err(GBFFT_ERR_UNSUPPORTED,
               "Invalid 2D processor grid - nproc /= p_row*p_col: this backend runs one rank");
  if (prec != GBFFT_PREC_SINGLE && prec != GBFFT_PREC_DOUBLE)
    return err(GBFFT_ERR_INVALID, "Invalid value for precision (4 or 8)");
  g.decomp_init = true;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.prec = prec;
  return GBFFT_OK;
}

int d2d_decomp_2d_finalize(void) {
  if (!g.grids.empty()) d2d_fft_finalize();
  g.decomp_init = false;
  g.nx = g.ny = g.nz = 0;
  return GBFFT_OK;
}

int d2d_get_decomp_main(int xst[3], int xen[3], int xsz[3], int yst[3], int yen[3], int ysz[3],
                        int zst[3], int zen[3], int zsz[3]) {
  if (!g.decomp_init) return err(GBFFT_ERR_STATE, "decomp_2d_init must be called first");
  // one rank: partition (src/decomp_2d.f90:1016-1064) gives the whole grid
  const int n[3] = {g.nx, g.ny, g.nz};
  int* st[3] = {xst, yst, zst};
  int* en[3] = {xen, yen, zen};
  int* sz[3] = {xsz, ysz, zsz};
  for (int p = 0; p < 3; ++p)
    for (int d = 0; d < 3; ++d) {
      if (st[p]) st[p][d] = 1;
      if (en[p]) en[p][d] = n[d];
      if (sz[p]) sz[p][d] = n[d];
    }
  return GBFFT_OK;
}

int d2d_transpose_x_to_y(const void* s, void* d, int c) { return transpose(s, d, c, GBFFT_X_TO_Y); }
int d2d_transpose_y_to_z(const void* s, void* d, int c) { return transpose(s, d, c, GBFFT_Y_TO_Z); }
int d2d_transpose_z_to_y(const void* s, void* d, int c) { return transpose(s, d, c, GBFFT_Z_TO_Y); }
int d2d_transpose_y_to_x(const void* s, void* d, int c) { return transpose(s, d, c, GBFFT_Y_TO_X); }

int d2d_fft_set_default_inplace(int inplace) {
  g.default_inplace = inplace ? 1 : 0;
  return GBFFT_OK;
}

// src/fft_common.f90:381-413
int d2d_fft_set_ngrid(int ngrid) {
  if (ngrid < 1) return err(GBFFT_ERR_INVALID, "Invalid value for n_grid");
  if ((int)g.grids.size() > ngrid) {
    for (size_t i = ngrid; i < g.grids.size(); ++i) destroy_grid(g.grids[i]);
    if (g.current >= ngrid) g.current = -1;
  }
  g.grids.resize(ngrid);
  return GBFFT_OK;
}

int d2d_fft_get_ngrid(void) { return (int)g.grids.size(); }

// src/fft_common.f90:66-242 (the four init overloads and engine%init)
int d2d_fft_init(int pencil, int nx, int ny, int nz, int igrid, int opt_inplace,
                 int opt_inplace_r2c, int opt_inplace_c2r, const int* opt_skip) {
  return d2d_fft_init_dtt(pencil, nx, ny, nz, igrid, opt_inplace, opt_inplace_r2c, opt_inplace_c2r, opt_skip,
                          nullptr, 0);
}

// decomp_2d_fft_engine_init with opt_DTT (src/fft_fftw3_f03.f90:230-331):
// the engine of the grid plus, when opt_dtt is given, its r2r transforms
int d2d_fft_init_dtt(int pencil, int nx, int ny, int nz, int igrid, int opt_inplace, int opt_inplace_r2c,
                     int opt_inplace_c2r, const int* opt_skip, const int* opt_dtt, int n_dtt) {
  if (!g.decomp_init) return err(GBFFT_ERR_STATE, "decomp_2d_init must be called first");
  if (nx == 0 && ny == 0 && nz == 0 && igrid == 0) {  // fft_init_noarg / fft_init_arg
    nx = g.nx;
    ny = g.ny;
    nz = g.nz;
  }
  if (igrid == 0) {  // fft_init_one_grid
    int rc = d2d_fft_set_ngrid(1);
    if (rc) return rc;
    igrid = 1;
  }
  if (igrid < 1 || igrid > (int)g.grids.size()) return err(GBFFT_ERR_INVALID, "Invalid value for igrid");
  Grid& gr = g.grids[igrid - 1];
  if (gr.initialised) return err(GBFFT_ERR_STATE, "FFT engine should only be initialised once");
  if (nx <= 0) return err(GBFFT_ERR_INVALID, "Invalid value for nx");
  if (ny <= 0) return err(GBFFT_ERR_INVALID, "Invalid value for ny");
  if (nz <= 0) return err(GBFFT_ERR_INVALID, "Invalid value for nz");
  const int inplace = opt_inplace < 0 ? g.default_inplace : (opt_inplace ? 1 : 0);
  if (opt_inplace_r2c >= 0) return err(GBFFT_ERR_UNSUPPORTED, "In-place r2c transform is not yet available");
  if (opt_inplace_c2r >= 0) return err(GBFFT_ERR_UNSUPPORTED, "In-place c2r transform is not yet available");
  if (pencil != GBFFT_PHYSICAL_IN_X && pencil != GBFFT_PHYSICAL_IN_Z)
    return err(GBFFT_ERR_INVALID, "Invalid value for pencil");
  gbfft_engine_t eng = nullptr;
  int rc = gbfft_engine_create(pencil, nx, ny, nz, inplace, opt_skip, g.prec, GBFFT_FORM_PLAIN, &eng);
  if (rc) return rc;
  gbfft_dtt_t dtt = nullptr;
  if (opt_dtt) {
    rc = gbfft_dtt_create(pencil, nx, ny, nz, opt_skip, g.prec, opt_dtt, n_dtt, &dtt);
    if (rc) {
      gbfft_engine_destroy(eng);
      return rc;
    }
  }
  gr.eng = eng;
  gr.dtt = dtt;
  gr.initialised = true;
  gr.format = pencil;
  gr.nx = nx;
  gr.ny = ny;
  gr.nz = nz;
  gr.inplace = inplace;
  g.current = igrid - 1;  // engine%use_it() at the end of engine%init
  return GBFFT_OK;
}

// src/fft_common.f90:418-443, :446-479
int d2d_fft_use_grid(int igrid) {
  if (igrid == 0) {
    if (g.grids.empty()) return err(GBFFT_ERR_STATE, "The FFT module was not initialised");
    igrid = 1;
  }
  if (igrid < 1 || igrid > (int)g.grids.size()) return err(GBFFT_ERR_INVALID, "Invalid value for igrid");
  if (!g.grids[igrid - 1].initialised) return err(GBFFT_ERR_STATE, "FFT engine is not ready");
  g.current = igrid - 1;
  return GBFFT_OK;
}

int d2d_fft_get_engine(int igrid, gbfft_engine_t* engine) {
  if (!engine) return err(GBFFT_ERR_INVALID, "null output pointer");
  if (igrid == 0) {
    if (g.grids.empty()) return err(GBFFT_ERR_STATE, "The FFT module was not initialised");
    igrid = 1;
  }
  if (igrid < 1 || igrid > (int)g.grids.size()) return err(GBFFT_ERR_INVALID, "Invalid value for igrid");
  *engine = g.grids[igrid - 1].eng;
  return GBFFT_OK;
}

int d2d_fft_3d_c2c(void* in, void* out, int isign) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "FFT library must be initialised first");
  return gbfft_exec_c2c(gr->eng, in, out, isign, g.stream);
}

int d2d_fft_3d_r2c(const void* in_r, void* out_c) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "FFT library must be initialised first");
  return gbfft_exec_r2c(gr->eng, in_r, out_c, g.stream);
}

int d2d_fft_3d_c2r(void* in_c, void* out_r) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "FFT library must be initialised first");
  return gbfft_exec_c2r(gr->eng, in_c, out_r, g.stream);
}

// decomp_2d_dtt_3d_r2r (src/fft_fftw3_f03.f90:1959-2023) on the current grid
int d2d_dtt_3d_r2r(void* in, void* out, int isign) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "FFT library must be initialised first");
  if (!gr->dtt) return err(GBFFT_ERR_STATE, "No DTT for the current engine");
  return gbfft_exec_r2r(gr->dtt, in, out, isign, g.stream);
}

// decomp_2d_fft_get_dtt_input (src/fft_fftw3_f03.f90:629-643): the forward
// kinds 1..8 of the current grid's r2r transforms
int d2d_fft_get_dtt_input(int kinds[3]) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "Invalid operation");
  if (!gr->dtt) return err(GBFFT_ERR_STATE, "No DTT for the current engine");
  int cfg[15];
  int rc = gbfft_dtt_get_config(gr->dtt, cfg);
  if (rc) return rc;
  for (int k = 0; k < 3; ++k) kinds[k] = cfg[k];
  return GBFFT_OK;
}

int d2d_fft_finalize(void) {
  for (Grid& gr : g.grids) destroy_grid(gr);
  g.grids.clear();
  g.current = -1;
  return GBFFT_OK;
}

int d2d_fft_get_size(int istart[3], int iend[3], int isize[3]) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "FFT library must be initialised first");
  int ph[3], sp[3];
  int rc = gbfft_engine_get_sizes(gr->eng, ph, sp);
  if (rc) return rc;
  for (int d = 0; d < 3; ++d) {
    if (istart) istart[d] = 1;
    if (iend) iend[d] = sp[d];
    if (isize) isize[d] = sp[d];
  }
  return GBFFT_OK;
}

int d2d_fft_get_ph_size(int xsz[3]) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "FFT library must be initialised first");
  return gbfft_engine_get_sizes(gr->eng, xsz, nullptr);
}

int d2d_fft_get_sp_size(int xsz[3]) {
  const Grid* gr = cur();
  if (!gr) return err(GBFFT_ERR_STATE, "FFT library must be initialised first");
  return gbfft_engine_get_sizes(gr->eng, nullptr, xsz);
}

int d2d_fft_get_format(void) {
  const Grid* gr = cur();
  return gr ? gr->format : 0;
}
int d2d_fft_get_inplace(void) {
  const Grid* gr = cur();
  return gr ? gr->inplace : 0;
}
int d2d_fft_get_inplace_r2c(void) { return 0; }
int d2d_fft_get_inplace_c2r(void) { return 0; }
int d2d_fft_backend(void) { return GBFFT_D2D_FFT_BACKEND; }

int d2d_set_stream(void* stream) {
  g.stream = (cudaStream_t)stream;
  return GBFFT_OK;
}

int d2d_fft_log(char* buf, int len) {
  if (!buf || len <= 0) return err(GBFFT_ERR_INVALID, "bad buffer");
  const Grid* gr = cur();
  std::string s = "===== FFT engine: gb300 (sm_103a Stockham, one rank) =====\n";
  if (gr) {
    int ph[3], sp[3];
    gbfft_engine_get_sizes(gr->eng, ph, sp);
    char line[256];
    std::snprintf(line, sizeof line,
                  "Physical space data in %s pencil\n ph: %d x %d x %d  sp: %d x %d x %d\n"
                  "Precision: %s\nOVERWRITE: %s (c2c input preserved; c2r input %s)\n",
                  gr->format == GBFFT_PHYSICAL_IN_X ? "X" : "Z", ph[0], ph[1], ph[2], sp[0],
                  sp[1], sp[2], g.prec == GBFFT_PREC_DOUBLE ? "double" : "single",
                  gr->inplace ? "yes" : "no", gr->inplace ? "destroyed" : "preserved");
    s += line;
  } else {
    s += "not initialised\n";
  }
  std::strncpy(buf, s.c_str(), (size_t)len - 1);
  buf[len - 1] = 0;
  return GBFFT_OK;
}

}  // extern "C"
