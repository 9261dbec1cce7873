/*
 * gbfft.h -- C ABI of the GB300 (sm_103a) 3D FFT backend for 2DECOMP&FFT at
 * one rank (p_row = p_col = 1).
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status (GBFFT_OK = 0).  On failure the message is available
 * from gbfft_last_error_string() (thread-local).  Device pointers are CUDA
 * device addresses; `stream` is a cudaStream_t (NULL = legacy default stream).
 * Calls are stream-ordered: they enqueue work and return without waiting,
 * exactly like the cuFFT exec calls they replace.
 *
 * Array layout: a 3D array (n1, n2, n3) is stored with the first index
 * fastest (Fortran order), as every 2DECOMP pencil is.  Complex values are
 * interleaved (re, im).  Arrays must be aligned to their element size
 * (sizeof(real) for real arrays, 2 * sizeof(real) for complex ones).  At one rank the X-, Y- and Z-pencil of a field share
 * the same shape and the same layout.
 */
#ifndef GBFFT_H
#define GBFFT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GBFFT_OK 0
#define GBFFT_ERR_INVALID 1     /* bad argument (size, format, pointer)      */
#define GBFFT_ERR_ALLOC 2       /* device allocation failed                  */
#define GBFFT_ERR_CUDA 3        /* a CUDA runtime call failed                */
#define GBFFT_ERR_UNSUPPORTED 4 /* valid request this backend cannot run     */
#define GBFFT_ERR_STATE 5       /* wrong call order (use before init, ...)   */
#define GBFFT_ERR_TIMEOUT 6     /* a bounded device wait gave up             */
#define GBFFT_ERR_BOUNDS 7      /* bounds-checked build: an access outside an
                                   array was caught (and skipped)            */

/* ---- constants, same values as src/decomp_2d_constants.f90 ----------- */
#define GBFFT_PHYSICAL_IN_X 1 /* decomp_2d_constants.f90:92 PHYSICAL_IN_X */
#define GBFFT_PHYSICAL_IN_Z 3 /* decomp_2d_constants.f90:93 PHYSICAL_IN_Z */
#define GBFFT_FORWARD (-1)    /* decomp_2d_constants.f90:86 DECOMP_2D_FFT_FORWARD */
#define GBFFT_BACKWARD 1      /* decomp_2d_constants.f90:87 DECOMP_2D_FFT_BACKWARD */
#define GBFFT_D2D_FFT_BACKEND 5 /* new id beside D2D_FFT_BACKEND_CUFFT = 4 (:81) */

/* precision of an engine: mytype of the reference build (DOUBLE_PREC or not) */
#define GBFFT_PREC_SINGLE 4
#define GBFFT_PREC_DOUBLE 8

/* arithmetic form of the axis passes */
#define GBFFT_FORM_PLAIN 0 /* CUDA-core FP32 / FP64 butterflies              */
#define GBFFT_FORM_SPLIT 1 /* radix-16 stages as split-FP16 tensor-core DFTs
                              (FP32 data; axes of 256, 512, 1024 points; other
                              axes run the plain kernels) */
#define GBFFT_FORM_SPLIT_TC 2 /* as GBFFT_FORM_SPLIT, with strided 1024-point
                                 c2c passes as two 32-point split-FP16 DFT
                                 products on the 5th-generation tensor cores
                                 (tcgen05, accumulators in tensor memory) */

/* transpose kinds (src/decomp_2d.f90:140-222 generic transpose_* names) */
#define GBFFT_X_TO_Y 0
#define GBFFT_Y_TO_Z 1
#define GBFFT_Z_TO_Y 2
#define GBFFT_Y_TO_X 3

typedef struct gbfft_engine_s* gbfft_engine_t;

/* Create one FFT grid.  Replaces decomp_2d_fft_engine_init + init_fft_engine
 * of the cuFFT backend (src/fft_common.f90:141-242, src/fft_cufft.f90:263-431):
 * validates sizes and format with the same rules, builds the per-axis plans
 * and twiddle tables, and allocates the work area.
 *   format  GBFFT_PHYSICAL_IN_X or GBFFT_PHYSICAL_IN_Z
 *   inplace nonzero = OVERWRITE: c2c/c2r may destroy their input
 *   skip    NULL or three flags: skip the x / y / z c2c transforms
 *           (opt_skip_XYZ_c2c; r2c/c2r along the real axis cannot be skipped
 *           and only warns, as src/fft_generic.f90:221-222 does)
 *   prec    GBFFT_PREC_SINGLE or GBFFT_PREC_DOUBLE
 *   form    GBFFT_FORM_PLAIN, GBFFT_FORM_SPLIT or GBFFT_FORM_SPLIT_TC (both split
 *           forms need PREC_SINGLE) */
int gbfft_engine_create(int format, int nx, int ny, int nz, int inplace,
                        const int* skip, int prec, int form,
                        gbfft_engine_t* engine);

/* Free plans, tables and work area (src/fft_cufft.f90:436-470,
 * finalize_fft_engine). */
int gbfft_engine_destroy(gbfft_engine_t engine);

/* Sizes of the physical (ph) and spectral (sp) arrays, (n1, n2, n3) each:
 * decomp_2d_fft_get_size / ph%xsz / sp%xsz at one rank
 * (src/fft_common.f90:204-216, :311-327). */
int gbfft_engine_get_sizes(gbfft_engine_t engine, int ph[3], int sp[3]);

/* Bytes of device work area the engine holds (0 when none is needed): the
 * c2r / padded-layout work area, plus, when an axis is longer than one
 * shared-memory tile (more than 8192 points, or an FP64 line whose two
 * buffers exceed the tile), two grid-sized complex buffers for that axis's
 * stage-by-stage passes. */
int gbfft_engine_work_bytes(gbfft_engine_t engine, size_t* bytes);

/* 3D r2c, forward, unnormalised: fft_3d_r2c (src/fft_common_3d.f90:121-189,
 * GPU src/fft_cufft.f90:795-934).  d_in real ph-shaped, d_out complex
 * sp-shaped.  d_in is not modified.  d_in and d_out must not overlap. */
int gbfft_exec_r2c(gbfft_engine_t engine, const void* d_in, void* d_out,
                   void* stream);

/* 3D c2r, backward, unnormalised: fft_3d_c2r (src/fft_common_3d.f90:194-296,
 * GPU src/fft_cufft.f90:939-1170).  d_in complex sp-shaped is preserved
 * unless the engine is inplace. */
int gbfft_exec_c2r(gbfft_engine_t engine, void* d_in, void* d_out,
                   void* stream);

/* 3D c2c: fft_3d_c2c (src/fft_common_3d.f90:9-116, GPU src/fft_cufft.f90:676-790).
 * isign = GBFFT_FORWARD or GBFFT_BACKWARD.  d_in == d_out is allowed. */
int gbfft_exec_c2c(gbfft_engine_t engine, void* d_in, void* d_out, int isign,
                   void* stream);

/* transpose_x_to_y / y_to_z / z_to_y / y_to_x at one rank: an identity-layout
 * copy of n1*n2*n3 elements (src/transpose_x_to_y.f90:41-50,
 * src/transpose_y_to_z.f90:40-49, src/transpose_z_to_y.f90:41-47,
 * src/transpose_y_to_x.f90:41).  is_complex selects complex(mytype). */
int gbfft_transpose(int kind, int is_complex, int prec, const void* d_src,
                    void* d_dst, int n1, int n2, int n3, void* stream);

/* ---- multi-rank pencil transposes (p_row x p_col ranks) ----------------
 * The pieces of transpose_x_to_y / y_to_z / z_to_y / y_to_x on a
 * p_row x p_col rank grid that run on each rank's GPU.  A transpose packs
 * the local pencil into one send buffer of per-peer blocks
 * (gbfft_transpose_pack), exchanges the buffers with the caller's
 * communication library -- MPI_ALLTOALLV or NCCL grouped send/receive on the
 * column communicator for x <-> y, the row communicator for y <-> z, as the
 * reference does (src/transpose_x_to_y.f90:96-129,
 * src/transpose_y_to_z.f90:94-156) -- and unpacks the received buffer into
 * the destination pencil (gbfft_transpose_unpack).  Ranks are numbered
 * row-major on the grid (rank = coord1 * p_col + coord2), as the
 * reference's Cartesian topology (src/decomp_2d_init_fin.f90:95-122). */
#define GBFFT_MAX_PEERS 1024 /* ranks of one row or column communicator */

/* Sub-block of each pencil owned by a rank (1-based, inclusive ends):
 * decomp_info_init's partition of the grid (src/decomp_2d.f90:411-416,
 * partition :1016-1064), X pencil (x local, y over p_row, z over p_col),
 * Y pencil (x over p_row, y local, z over p_col), Z pencil (x over p_row,
 * y over p_col, z local). */
typedef struct {
  int xst[3], xen[3], xsz[3];
  int yst[3], yen[3], ysz[3];
  int zst[3], zen[3], zsz[3];
  int coord[2]; /* (coord1, coord2) on the rank grid */
} gbfft_pencil_info_t;
/* Errors as the reference's: "Invalid 2D processor grid. Make sure that
 * min(nx,ny) >= p_row and min(ny,nz) >= p_col" (src/decomp_2d.f90:399-405). */
int gbfft_decomp_info(int nx, int ny, int nz, int p_row, int p_col, int rank, gbfft_pencil_info_t* info);
/* distribute (src/decomp_2d.f90:1070-1105): n points over nproc ranks,
 * 1-based starts, ends and sizes (nproc entries each). */
int gbfft_decomp_distribute(int n, int nproc, int* st, int* en, int* sz);
/* The exchange of one transpose kind (GBFFT_X_TO_Y ...) seen from `rank`:
 * per peer of its communicator (*npeers = p_row for x <-> y, p_col for
 * y <-> z, in communicator rank order), the block widths along the split
 * dimension of the send side and of the receive side (the dist arrays of
 * get_dist, src/decomp_2d.f90:1112-1133), and the ALLTOALLV send / receive
 * counts and 0-based displacements in elements (prepare_buffer,
 * :1138-1206).  Arrays of GBFFT_MAX_PEERS entries are always large enough. */
int gbfft_decomp_counts(int nx, int ny, int nz, int p_row, int p_col, int rank, int kind, int* send_dist,
                        int* send_cnts, int* send_disp, int* recv_dist, int* recv_cnts, int* recv_disp,
                        int* npeers);
/* mem_split_* of a transpose kind as one kernel: the local (n1, n2, n3)
 * source pencil (real or complex, single or double precision) split along
 * the kind's send dimension (x for X_TO_Y, y for Y_TO_Z and Y_TO_X, z for
 * Z_TO_Y) into npeers blocks of widths dist[m], block m written in Fortran
 * order at element displacement disp[m] of d_send
 * (src/transpose_x_to_y.f90:266-323, src/transpose_y_to_z.f90:370-428,
 * src/transpose_z_to_y.f90:370-427, src/transpose_y_to_x.f90:266-323).
 * dist and disp are host arrays; the copy is bit-exact and stream-ordered.
 * send_elems is the send buffer's size in elements: a block that would reach
 * past it is rejected (GBFFT_ERR_INVALID) before anything is launched. */
int gbfft_transpose_pack(int kind, int is_complex, int prec, const void* d_src, int n1, int n2, int n3,
                         int npeers, const int* dist, const int* disp, void* d_send, size_t send_elems,
                         void* stream);
/* mem_merge_* of a transpose kind as one kernel: the received blocks of
 * d_recv (widths dist[m] along the kind's receive dimension -- y for X_TO_Y
 * and Z_TO_Y, z for Y_TO_Z, x for Y_TO_X -- at displacements disp[m]) into
 * the local (n1, n2, n3) destination pencil (src/transpose_x_to_y.f90:384-441,
 * src/transpose_y_to_z.f90:490-548, src/transpose_z_to_y.f90:488-545,
 * src/transpose_y_to_x.f90:384-441).  recv_elems: d_recv's size in
 * elements, checked as for the pack. */
int gbfft_transpose_unpack(int kind, int is_complex, int prec, const void* d_recv, int n1, int n2, int n3,
                           int npeers, const int* dist, const int* disp, size_t recv_elems, void* d_dst,
                           void* stream);

/* ---- halo-cell update (src/halo.f90, src/halo_common.f90) -------------
 * The device data movement of update_halo: a copy of the box of
 * box[0] x box[1] x box[2] elements at 0-based offset src_off of the
 * Fortran-ordered array d_src (extents src_dims) to dst_off of d_dst
 * (extents dst_dims) -- the pencil into the interior of its halo-extended
 * array (src/halo_common.f90:20-75), and the slabs of `level` planes a rank
 * sends to and receives from its neighbours, packed into and unpacked from
 * contiguous buffers (halo_exchange_{x,y,z}_body.f90; the exchange itself
 * is the caller's point-to-point messaging, as MPI_IRECV / MPI_ISSEND
 * there).  Bit-exact, stream-ordered; a box outside either array is
 * rejected (GBFFT_ERR_INVALID) before anything is launched. */
int gbfft_box_copy(int is_complex, int prec, const void* d_src, const int* src_dims, const int* src_off,
                   void* d_dst, const int* dst_dims, const int* dst_off, const int* box, void* stream);

/* Device memory for pencil arrays: replaces alloc_x/alloc_y/alloc_z of the
 * device build (src/alloc_dev.f90:10-135).  gbfft_malloc returns 256-byte
 * aligned memory. */
int gbfft_malloc(void** d_ptr, size_t bytes);
int gbfft_free(void* d_ptr);

/* Message of the last failing call on this host thread ("" if none). */
const char* gbfft_last_error_string(void);

/* Number of warnings raised so far ("r2c / c2r transform can not be
 * skipped", src/fft_generic.f90:221-222), for callers that check them. */
int gbfft_warning_count(void);

/* ---- batched uneven grids (the multiple-grids use of
 *      src/fft_common.f90:381-479) ------------------------------------- */
typedef struct gbfft_batch_s* gbfft_batch_t;

/* A batch is a list of (engine, real array, spectral array) items.  Forward
 * runs every item's r2c (real -> spectral), backward every item's c2r
 * (spectral -> real, the real array is overwritten).
 *   gbfft_batch_forward / _backward   per-grid loop: each grid's passes as
 *                                     their own launches, grid after grid;
 *   gbfft_batch_run(mask)             mask 1 forward, 2 backward, 3 both:
 *                                     in ONE persistent launch when the batch
 *                                     is persistent-capable (FP32 engines,
 *                                     every line length in 32, 48, 64, 96,
 *                                     128, 192, 256), else the per-grid loop.
 * gbfft_batch_set_persistent(0) forces the per-grid loop.  The persistent
 * launch uploads its pass descriptors on first use (synchronously). */
int gbfft_batch_create(gbfft_batch_t* batch);
int gbfft_batch_add(gbfft_batch_t batch, gbfft_engine_t engine,
                    const void* d_real, void* d_spec);
int gbfft_batch_forward(gbfft_batch_t batch, void* stream);
int gbfft_batch_backward(gbfft_batch_t batch, void* stream);
int gbfft_batch_set_persistent(gbfft_batch_t batch, int enable);
int gbfft_batch_run(gbfft_batch_t batch, int mask, void* stream);
/* persistent = 1 when gbfft_batch_run uses the one-launch path. */
int gbfft_batch_info(gbfft_batch_t batch, int* persistent, int* launches_per_run);
/* Status of the last persistent run (waits for the device): GBFFT_ERR_TIMEOUT
 * if one of its bounded inter-tile waits gave up. */
int gbfft_batch_status(gbfft_batch_t batch);
/* Capture gbfft_batch_run(batch, 3) (forward then backward, persistent or
 * per-grid loop as set) in one CUDA graph; gbfft_batch_graph_launch enqueues
 * a replay on `stream`.  Capture needs a non-default stream. */
int gbfft_batch_graph_build(gbfft_batch_t batch, void* stream);
int gbfft_batch_graph_launch(gbfft_batch_t batch, void* stream);
int gbfft_batch_destroy(gbfft_batch_t batch);

/* ---- per-pass device timing, for benchmarks ---------------------------
 * While enabled, every axis pass an engine enqueues is bracketed by two CUDA
 * events recorded on the pass's stream.  gbfft_engine_profile_read resolves
 * them (it waits for the events) and returns, for pass kind `kind`
 * (GBFFT_PASS_*), the number of launches, their summed device time in ms and
 * the summed algorithmic bytes (one read and one write of the array). */
#define GBFFT_PASS_R2C 0
#define GBFFT_PASS_C2R 1
#define GBFFT_PASS_C2C_X 2
#define GBFFT_PASS_C2C_Y 3
#define GBFFT_PASS_C2C_Z 4
#define GBFFT_PASS_XY 5   /* x and y passes fused per z-plane (one kernel) */
#define GBFFT_PASS_KINDS 6
int gbfft_engine_set_profiling(gbfft_engine_t engine, int enable);

/* Tile shape of one pass kind (GBFFT_PASS_*): lines per CTA.  0 restores the
 * built-in choice.  Used by the autotuner; rejected when the CTA would exceed
 * the kernel's thread or shared-memory limit. */
int gbfft_engine_set_tile(gbfft_engine_t engine, int kind, int lines_per_cta);

/* Cluster launch of one pass kind (GBFFT_PASS_*) on its power-of-two
 * one-shot kernel: ctas 2, 4 or 8 launches neighbouring CTAs (neighbouring
 * lines) as thread-block clusters, which the GPU co-schedules, and sync = 1
 * starts every CTA with a cluster barrier, so that the row segments that
 * the CTAs of a cluster read from the same rows of a strided axis arrive at
 * DRAM together.  0 (default) launches plain CTAs.  gbfft_engine_get_cluster
 * fills GBFFT_PASS_KINDS ints each. */
int gbfft_engine_set_cluster(gbfft_engine_t engine, int kind, int ctas, int sync);
int gbfft_engine_get_cluster(gbfft_engine_t engine, int* ctas, int* sync);

/* Row layout of the passes.  pad = 1: the work area's rows of complex values
 * (sp[0] of them) start on 64-byte boundaries, and every pass of an r2c or
 * c2r but the last writes there, so that the strided passes store whole
 * 32-byte sectors (rows of nx/2+1 values are mostly misaligned otherwise);
 * pad = 2: the same for c2r only, r2c working in its output; pad = 0
 * (default): the arrays' own rows.  Engines created with inplace have no
 * work area and ignore it.  flat = 1 (default): a z pass whose output rows
 * are unpadded and do not start on 32-byte sectors (or hold a number of
 * values that is not a multiple of 16) takes the lines of each (x, y) plane
 * flat, so that its row segments are as aligned as the plane.  Both are
 * tuning choices (keys pad= and flat= of the tuning cache); the work area
 * is sized for padded rows whatever the setting. */
int gbfft_engine_set_layout(gbfft_engine_t engine, int pad, int flat);
int gbfft_engine_get_layout(gbfft_engine_t engine, int* pad, int* flat);

/* Host-only description of the axis passes an engine with these arguments
 * would run (no device memory, no GPU needed): which = 0 r2c, 1 c2r, 2 c2c
 * forward, 3 c2c backward; pad / flat as gbfft_engine_set_layout, -1 for
 * the engine's own choice (tuning cache or default).  Fills up to
 * max_passes entries and sets *n_passes to the number of passes (0 for a
 * c2c with every axis skipped, which is a copy).  Strides are in elements of
 * each side's type (real on the real side of r2c / c2r); a pass's lines are
 * u < nlines (complex lines; real lines u < real_lines for r2c / c2r) and,
 * on strided axes, v < nv, starting at u * s_l (contiguous), u + v * s_l
 * (strided) or, when row_w > 0, (u / row_w) * s_r + u % row_w; point n of a
 * line sits at + n * s_n.  src / dst: 0 the input array, 1 the output
 * array, 2 the engine's work area.  The x/y fusion is not described. */
typedef struct {
  int kind;       /* 0 c2c, 1 r2c, 2 c2r */
  int contiguous; /* 1: lines along x */
  int n;          /* points a line (real points for r2c / c2r) */
  int row_w;
  long long nlines, real_lines, nv;
  long long s_src_n, s_src_l, s_src_r, s_dst_n, s_dst_l, s_dst_r;
  int src, dst;
} gbfft_pass_desc_t;
int gbfft_plan_describe(int format, int nx, int ny, int nz, int inplace, const int* skip, int prec, int pad,
                        int flat, int which, gbfft_pass_desc_t* out, int max_passes, int* n_passes);

/* Bulk-tensor-copy staging of the y passes: 1 (default) runs every FP32 c2c
 * y pass of 1024 points whose rows and planes lie multiples of 16 bytes
 * apart (the padded work area, rows of an even number of values) as one
 * persistent kernel per pass, one CTA per SM, whose tiles arrive in shared
 * memory by cp.async.bulk.tensor copies two tiles ahead of the one being
 * transformed and leave it the same way; 0 runs the one-shot kernel.
 * A pass whose bounded wait for its copies gives up sets the status that
 * gbfft_engine_status reports.  Tuning-cache key tma=0/1. */
int gbfft_engine_set_tma(gbfft_engine_t engine, int enable);
int gbfft_engine_get_tma(gbfft_engine_t engine, int* enable);

/* Pass fusion: 1 (default) lets the engine run the x and y passes of each
 * z-plane in one kernel where a fused kernel exists for the lengths; 0 runs
 * one kernel per axis. */
int gbfft_engine_set_fusion(gbfft_engine_t engine, int enable);

/* ---- autotuning ---------------------------------------------------------
 * Engines apply a tuning cache at creation: a text file (default
 * tune_cache.txt in the package directory, or $GBFFT_TUNE_CACHE; "" = none)
 * with lines "prec format nx ny nz key=value ...": per pass kind the lines
 * per CTA (r2c c2r c2c_x c2c_y c2c_z xy_fused) and the cluster launch
 * (cl_<pass> = CTAs a cluster, cls_<pass> = 1 for the start barrier),
 * fuse=0/1, pad= / flat= (gbfft_engine_set_layout), tma=0/1
 * (gbfft_engine_set_tma), and e_x / e_y / e_z, the points per thread of the
 * x / y / z plan (as gbfft_engine_set_plan).  The tuner
 * (2decomp-fft_gb300/tune.py) measures the choices and writes the file. */
int gbfft_tune_cache_path(const char* path); /* NULL = default, "" = none */
/* Re-plan axis 0, 1 or 2: 512 or 1024 points with 16 or 32 points per
 * thread (radix 16, 16, ... or two radix-32 stages; a contiguous line of 32
 * points a thread is one warp); 243, 270, 360, 384 or 400 points with the
 * balanced plan (points = 9, 30, 30, 24, 20: 9 9 3, 15 6 3, 10 6 6, 8 8 6,
 * 20 20) or points = 2 for the two-stage plan n = R0 R1.  Resets the tile
 * shapes.  Waits for the device. */
int gbfft_engine_set_plan(gbfft_engine_t engine, int axis, int points);
/* Current fusion switch, lines per CTA per pass kind (GBFFT_PASS_KINDS
 * ints, 0 = built-in) and points per thread per axis (3 ints, 0 = the axis
 * has no compile-time plan). */
int gbfft_engine_get_tuning(gbfft_engine_t engine, int* fuse, int* tiles, int* points);

/* Status of the engine's most recent fused x/y pass: waits for the device,
 * returns GBFFT_ERR_TIMEOUT if one of its bounded inter-CTA waits gave up
 * (the result of that transform is then invalid), GBFFT_OK otherwise.  The
 * fused pass keeps per-engine counters, so one engine must not run two
 * transforms at the same time on different streams. */
int gbfft_engine_status(gbfft_engine_t engine);
int gbfft_engine_profile_read(gbfft_engine_t engine, int kind, long long* launches,
                              double* ms, double* bytes);

/* ---- allocation-free c2r ---------------------------------------------
 * No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory (code running under another runtime's memory
 * pool, inside a callback, or after reserving all device memory up front).
 * It does what gbfft_exec_c2r does for a non-OVERWRITE engine without skip
 * flags (input preserved, unnormalised), but takes the grid description
 * instead of an engine and allocates nothing: its twiddle tables and its
 * work area live in one static device array of GBFFT_NOALLOC_SCRATCH_BYTES
 * that every GPU loading this library holds until the process exits.
 *   - Sizes whose tables + spectral-sized work area exceed the array are
 *     rejected with GBFFT_ERR_INVALID.
 *   - All calls share the array: calls whose GPU work overlaps (other
 *     streams, other host threads) race and corrupt each other.
 *   - The first call on a device (with it current) looks up the array's
 *     device address; make that first call before any stream capture.
 *   - The runtime loads device code lazily by default, so that first call is
 *     most likely also when the device reserves the array: make it before
 *     reserving all device memory or entering a region that may not
 *     allocate, or run with CUDA_MODULE_LOADING=EAGER.
 *   - The cached address belongs to the primary context: cudaDeviceReset
 *     between calls is not supported.
 *   - Arrays must be aligned to their elements, as for gbfft_exec_c2r; a
 *     misaligned pointer is rejected before any launch. */
#define GBFFT_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int gbfft_exec_c2r_noalloc(int format, int nx, int ny, int nz, int prec,
                           const void* d_in, void* d_out, void* stream);

/* Failure detection self-test (no counterpart in the reference): run the
 * bounded wait the inter-CTA kernels use, on a device counter holding
 * counter_value, waiting for `need` with at most poll_limit polls (<= 2^26).
 * *timed_out = 1 when the wait gave up (counter_value < need), 0 otherwise.
 * The kernel ends either way; nothing is left waiting on the GPU. */
int gbfft_selftest_bounded_wait(int counter_value, int need, long long poll_limit, int* timed_out);

/* ---- debugging aids (no counterpart in the reference) ------------------
 * gbfft_debug_fail_alloc(n): the (n+1)-th device allocation the library
 * makes from now on (n = 0: the next one) fails as if the device were out of
 * memory, once; -1 disarms.  Tests drive every allocation of engine, batch
 * and work-area creation into failure this way and check that each call
 * returns GBFFT_ERR_ALLOC and frees what it had allocated.
 * gbfft_set_nvtx(1) names every transform ("fft_r2c", "fft_c2r", "fft_c2c":
 * the reference's profiler regions, src/fft_common_3d.f90:22,114) and every
 * axis pass with an NVTX range, for timeline profilers; off by default,
 * GBFFT_NVTX=1 in the environment turns it on at load.
 * gbfft_debug_bounds_build() = 1 in a library built with -DGB_DEBUG_BOUNDS
 * (2decomp-fft_gb300/build.py --variant debug): there every global access of
 * the axis-pass kernels is checked against its array's extent, and one
 * outside it is skipped and reported by gbfft_engine_status as
 * GBFFT_ERR_BOUNDS instead of reaching memory. */
int gbfft_debug_fail_alloc(long long nth);
/* Device allocations the library holds right now (engines, batches, work
 * areas, gbfft_malloc), for leak checks. */
long long gbfft_debug_live_allocations(void);
int gbfft_set_nvtx(int enable);
int gbfft_debug_bounds_build(void);

/* Library version and kernel-launch counter (every kernel this library has
 * enqueued since load), for benchmarks that report launches. */
int gbfft_version(int* major, int* minor);
long long gbfft_launch_count(void);
/* Of those, the strided passes run by the bulk-tensor-copy kernel
 * (gbfft_engine_set_tma). */
long long gbfft_tma_pass_count(void);
/* Number of tcgen05 split-precision passes launched so far, process-wide
 * (GBFFT_FORM_SPLIT_TC engines); no counterpart in the reference. */
long long gbfft_tc_pass_count(void);

/* ---- real-to-real transforms (DCT / DST) ----------------------------------
 * decomp_2d_dtt_3d_r2r and the opt_DTT configuration of decomp_2d_fft_init
 * (src/fft_fftw3_f03.f90:341-471 configuration, 1555-1656 the 1D passes,
 * 1959-2023 the 3D driver; the reference runs them as FFTW r2r plans in its
 * FFTW backend only).  Kinds per axis, FFTW's unnormalised definitions: */
#define GBFFT_DCT1 1 /* REDFT00 */
#define GBFFT_DCT2 2 /* REDFT10 */
#define GBFFT_DCT3 3 /* REDFT01 */
#define GBFFT_DCT4 4 /* REDFT11 */
#define GBFFT_DST1 5 /* RODFT00 */
#define GBFFT_DST2 6 /* RODFT10 */
#define GBFFT_DST3 7 /* RODFT01 */
#define GBFFT_DST4 8 /* RODFT11 */
typedef struct gbfft_dtt_s* gbfft_dtt_t;
/* dtt: 3 kinds (x, y, z; the reference's default windows) or 12 ints: kinds,
 * ifirst (1-based first point of the window), ndismiss (points left out),
 * ofirst (must equal ifirst) per axis.  A window of n = n_axis - ndismiss
 * points starting at ifirst is transformed; the other points pass through.
 * skip: NULL or three flags (the c2c skip flags skip r2r passes too).
 * Errors as the reference's: "Invalid argument", "Setup is not compatible
 * with in-place r2r transforms". */
int gbfft_dtt_create(int format, int nx, int ny, int nz, const int* skip, int prec, const int* dtt, int ndtt,
                     gbfft_dtt_t* dtt_out);
int gbfft_dtt_destroy(gbfft_dtt_t dtt);
/* The 15-int configuration: forward kinds, ifirst, ndismiss, ofirst,
 * backward kinds (inverse of DCT-II is DCT-III, of DST-II DST-III, the others
 * their own), kinds numbered 1..8. */
int gbfft_dtt_get_config(gbfft_dtt_t dtt, int* cfg15);
/* decomp_2d_dtt_3d_r2r(in, out, isign): x, y, z for PHYSICAL_IN_X forward
 * and PHYSICAL_IN_Z backward, z, y, x otherwise.  The first pass works in
 * place on d_in (as the reference's), the result is in d_out (d_in == d_out
 * allowed).  Unnormalised: a round trip multiplies by the product over the
 * axes of 2(n-1) (DCT-I), 2(n+1) (DST-I) or 2n (the others), n the window
 * length. */
int gbfft_exec_r2r(gbfft_dtt_t dtt, void* d_in, void* d_out, int isign, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBFFT_H */
