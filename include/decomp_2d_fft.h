/*
 * decomp_2d_fft.h -- C-linkage mirror of the 2DECOMP&FFT FFT module API
 * (module decomp_2d_fft, src/fft_common.f90) and of the one-rank pieces of
 * module decomp_2d it depends on, implemented over the GB300 backend of
 * gbfft.h.  Names, argument meaning and error checks follow the reference;
 * where the reference calls decomp_2d_abort (src/decomp_2d_mpi.f90:166-190)
 * these functions return a nonzero status with the same message, readable
 * through gbfft_last_error_string().
 *
 * Only p_row = p_col = 1 (one rank, one GPU) is supported: every pencil of a
 * field then has the shape (nx, ny, nz) and starts at (1, 1, 1).
 * Logical arguments are ints (0 = .false.).  "Optional" arguments take -1
 * (scalars) or NULL (arrays) for "not present".
 */
#ifndef DECOMP_2D_FFT_H
#define DECOMP_2D_FFT_H

#include "gbfft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* decomp_2d_init(nx, ny, nz, p_row, p_col) (src/decomp_2d_init_fin.f90:15-184)
 * at one rank.  p_row/p_col 0 means "choose" (= 1 here).  prec is the
 * reference's build-time mytype: GBFFT_PREC_SINGLE or GBFFT_PREC_DOUBLE. */
int d2d_decomp_2d_init(int nx, int ny, int nz, int p_row, int p_col, int prec);
/* decomp_2d_finalize: also finalizes the FFT module if still initialised. */
int d2d_decomp_2d_finalize(void);
/* decomp_info of decomp_main: xst/xen/xsz, yst/..., zst/... (1-based). */
int d2d_get_decomp_main(int xst[3], int xen[3], int xsz[3], int yst[3], int yen[3],
                        int ysz[3], int zst[3], int zen[3], int zsz[3]);

/* transpose_x_to_y / y_to_z / z_to_y / y_to_x of a decomp_main-shaped field
 * (src/decomp_2d.f90:140-222 generic names; one-rank bodies
 * src/transpose_x_to_y.f90:41-50 and siblings).  is_complex selects
 * complex(mytype); the call is ordered on the module stream. */
int d2d_transpose_x_to_y(const void* src, void* dst, int is_complex);
int d2d_transpose_y_to_z(const void* src, void* dst, int is_complex);
int d2d_transpose_z_to_y(const void* src, void* dst, int is_complex);
int d2d_transpose_y_to_x(const void* src, void* dst, int is_complex);

/* The OVERWRITE build flag (DECOMP_2D_FFT_INPLACE,
 * src/decomp_2d_constants.f90:125-129) as a runtime default for
 * opt_inplace = -1. */
int d2d_fft_set_default_inplace(int inplace);

/* decomp_2d_fft_init, all four overloads (src/fft_common.f90:42-47):
 *   nx = ny = nz = 0 and igrid = 0    -> fft_init_arg(pencil[, skip]) on the
 *                                        decomp_main sizes
 *   igrid = 0                         -> fft_init_one_grid (one grid)
 *   igrid >= 1                        -> fft_init_multiple_grids
 * opt_inplace: -1 = default, 0/1 = given.  opt_inplace_r2c / opt_inplace_c2r:
 * -1 = absent; any other value is rejected as in src/fft_common.f90:177-182.
 * opt_skip: NULL or three flags (opt_skip_XYZ_c2c). */
int d2d_fft_init(int pencil, int nx, int ny, int nz, int igrid, int opt_inplace,
                 int opt_inplace_r2c, int opt_inplace_c2r, const int* opt_skip);
/* decomp_2d_fft_init with opt_DTT (src/fft_fftw3_f03.f90:230-331, the FFTW
 * backend's r2r option): as d2d_fft_init, plus the grid's real-to-real
 * transforms when opt_dtt is not NULL (3 kinds or the 12-int form of
 * gbfft_dtt_create; n_dtt its length). */
int d2d_fft_init_dtt(int pencil, int nx, int ny, int nz, int igrid, int opt_inplace, int opt_inplace_r2c,
                     int opt_inplace_c2r, const int* opt_skip, const int* opt_dtt, int n_dtt);
/* decomp_2d_dtt_3d_r2r(in, out, isign) on the current grid
 * (src/fft_fftw3_f03.f90:1959-2023); "No DTT for the current engine" when
 * the grid was initialised without opt_DTT. */
int d2d_dtt_3d_r2r(void* in, void* out, int isign);
/* decomp_2d_fft_get_dtt_input (src/fft_fftw3_f03.f90:629-643). */
int d2d_fft_get_dtt_input(int kinds[3]);
/* decomp_2d_fft_set_ngrid / get_ngrid / use_grid (src/fft_common.f90:381-443);
 * igrid = 0 means "absent" for use_grid. */
int d2d_fft_set_ngrid(int ngrid);
int d2d_fft_get_ngrid(void);
int d2d_fft_use_grid(int igrid);
/* decomp_2d_fft_get_engine (src/fft_common.f90:485-514): the grid's engine. */
int d2d_fft_get_engine(int igrid, gbfft_engine_t* engine);
/* decomp_2d_fft_3d generic interface (src/fft_common.f90:49-53) on the
 * current grid, device arrays, ordered on the module stream. */
int d2d_fft_3d_c2c(void* in, void* out, int isign);
int d2d_fft_3d_r2c(const void* in_r, void* out_c);
int d2d_fft_3d_c2r(void* in_c, void* out_r);
/* decomp_2d_fft_finalize (src/fft_common.f90:247-282). */
int d2d_fft_finalize(void);
/* decomp_2d_fft_get_size (src/fft_common.f90:311-327): the spectral array's
 * start/end/size (1-based) in the pencil the forward transform ends in. */
int d2d_fft_get_size(int istart[3], int iend[3], int isize[3]);
/* decomp_2d_fft_get_ph / get_sp sizes: xsz of ph and of sp. */
int d2d_fft_get_ph_size(int xsz[3]);
int d2d_fft_get_sp_size(int xsz[3]);
/* decomp_2d_fft_get_format / get_inplace / get_inplace_r2c / get_inplace_c2r */
int d2d_fft_get_format(void);
int d2d_fft_get_inplace(void);
int d2d_fft_get_inplace_r2c(void);
int d2d_fft_get_inplace_c2r(void);
/* D2D_FFT_BACKEND of this module (GBFFT_D2D_FFT_BACKEND). */
int d2d_fft_backend(void);
/* Stream the module's transforms and transposes are enqueued on (NULL =
 * legacy default stream).  The reference's GPU path runs on the default
 * stream; this is the hook for callers that own a stream. */
int d2d_set_stream(void* stream);
/* decomp_2d_fft_log (src/fft_log.f90:16-69): writes the setup summary of the
 * current grid into buf (NUL-terminated, at most len bytes). */
int d2d_fft_log(char* buf, int len);

#ifdef __cplusplus
}
#endif

#endif /* DECOMP_2D_FFT_H */
