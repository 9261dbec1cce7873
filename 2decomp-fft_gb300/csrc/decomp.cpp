// 2D pencil decomposition of an (nx, ny, nz) grid over a p_row x p_col
// rank grid: the host-side integer work of decomp_info_init
// (src/decomp_2d.f90:382-490) that multi-rank transposes need -- which
// rank owns which sub-block of each pencil, and the counts and
// displacements of the all-to-all exchanges between pencils.
//
// The rank grid is the reference's Cartesian topology: dims = (p_row,
// p_col), ranks numbered row-major (rank = coord1 * p_col + coord2, as
// MPI_CART_CREATE without reordering, src/decomp_2d_init_fin.f90:95-114);
// x <-> y exchanges run among the p_row ranks of one column (fixed coord2,
// DECOMP_2D_COMM_COL), y <-> z exchanges among the p_col ranks of one row
// (fixed coord1, DECOMP_2D_COMM_ROW).
#include <string>
#include <vector>

#include "gbfft.h"
#include "gbfft_internal.h"

namespace {

int fail(int code, const char* msg) { return gbfft::set_error(code, msg); }

// distribute (src/decomp_2d.f90:1070-1105): n points over p ranks, the
// first p - n % p ranks get n / p points, the rest one more; 1-based starts
// and ends.
void distribute(int n, int p, int* st, int* en, int* sz) {
  const int size1 = n / p, nu = n - size1 * p, nl = p - nu;
  for (int i = 0; i < p; ++i) {
    const int s = i < nl ? size1 : size1 + 1;
    st[i] = i == 0 ? 1 : en[i - 1] + 1;
    sz[i] = s;
    en[i] = st[i] + s - 1;
  }
}

// partition (src/decomp_2d.f90:1016-1064): pdim[i] = 1 local, 2 across
// p_row (coord1), 3 across p_col (coord2).
void partition(const int n[3], const int pdim[3], int p_row, int p_col, const int coord[2], int st[3], int en[3],
               int sz[3]) {
  for (int i = 0; i < 3; ++i) {
    if (pdim[i] == 1) {
      st[i] = 1;
      en[i] = n[i];
      sz[i] = n[i];
      continue;
    }
    const int p = pdim[i] == 2 ? p_row : p_col, c = pdim[i] == 2 ? coord[0] : coord[1];
    std::vector<int> s(p), e(p), z(p);
    distribute(n[i], p, s.data(), e.data(), z.data());
    st[i] = s[c];
    en[i] = e[c];
    sz[i] = z[c];
  }
}

int check(int nx, int ny, int nz, int p_row, int p_col, int rank) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return fail(GBFFT_ERR_INVALID, "Invalid value for nx, ny or nz");
  if (p_row <= 0 || p_col <= 0) return fail(GBFFT_ERR_INVALID, "Invalid 2D processor grid");
  if (rank < 0 || rank >= p_row * p_col) return fail(GBFFT_ERR_INVALID, "Invalid rank for the 2D processor grid");
  // src/decomp_2d.f90:399-405
  if (nx < p_row || ny < p_row || ny < p_col || nz < p_col)
    return fail(GBFFT_ERR_INVALID,
                "Invalid 2D processor grid. Make sure that min(nx,ny) >= p_row and min(ny,nz) >= p_col");
  return GBFFT_OK;
}

}  // namespace

extern "C" int gbfft_decomp_distribute(int n, int nproc, int* st, int* en, int* sz) {
  if (n <= 0 || nproc <= 0 || !st || !en || !sz) return fail(GBFFT_ERR_INVALID, "bad argument");
  distribute(n, nproc, st, en, sz);
  return GBFFT_OK;
}

extern "C" int gbfft_decomp_info(int nx, int ny, int nz, int p_row, int p_col, int rank, gbfft_pencil_info_t* info) {
  int rc = check(nx, ny, nz, p_row, p_col, rank);
  if (rc != GBFFT_OK) return rc;
  if (!info) return fail(GBFFT_ERR_INVALID, "bad argument");
  const int n[3] = {nx, ny, nz};
  info->coord[0] = rank / p_col;
  info->coord[1] = rank % p_col;
  // X pencil (1, 2, 3), Y pencil (2, 1, 3), Z pencil (2, 3, 1):
  // src/decomp_2d.f90:411-416
  const int px[3] = {1, 2, 3}, py[3] = {2, 1, 3}, pz[3] = {2, 3, 1};
  partition(n, px, p_row, p_col, info->coord, info->xst, info->xen, info->xsz);
  partition(n, py, p_row, p_col, info->coord, info->yst, info->yen, info->ysz);
  partition(n, pz, p_row, p_col, info->coord, info->zst, info->zen, info->zsz);
  return GBFFT_OK;
}

// prepare_buffer (src/decomp_2d.f90:1138-1206): per peer of the exchange,
// the send and receive counts and displacements (0-based, elements) of the
// ALLTOALLV, and the block widths along the split dimensions (the dist
// arrays, get_dist :1112-1133).
extern "C" int gbfft_decomp_counts(int nx, int ny, int nz, int p_row, int p_col, int rank, int kind,
                                   int* send_dist, int* send_cnts, int* send_disp, int* recv_dist,
                                   int* recv_cnts, int* recv_disp, int* npeers) {
  gbfft_pencil_info_t in;
  int rc = gbfft_decomp_info(nx, ny, nz, p_row, p_col, rank, &in);
  if (rc != GBFFT_OK) return rc;
  if (kind < GBFFT_X_TO_Y || kind > GBFFT_Y_TO_X) return fail(GBFFT_ERR_INVALID, "bad transpose kind");
  if (!send_dist || !send_cnts || !send_disp || !recv_dist || !recv_cnts || !recv_disp || !npeers)
    return fail(GBFFT_ERR_INVALID, "bad argument");
  const bool col = kind == GBFFT_X_TO_Y || kind == GBFFT_Y_TO_X;  // COMM_COL: p_row peers
  const int p = col ? p_row : p_col;
  std::vector<int> st(p), en(p), d1(p), d2(p);
  // x1dist / y1dist over p_row, y2dist / z2dist over p_col
  distribute(col ? nx : ny, p, st.data(), en.data(), d1.data());  // x1dist or y2dist
  distribute(col ? ny : nz, p, st.data(), en.data(), d2.data());  // y1dist or z2dist
  std::vector<int> c_a(p), c_b(p);
  for (int i = 0; i < p; ++i) {
    if (col) {
      c_a[i] = d1[i] * in.xsz[1] * in.xsz[2];  // x1cnts
      c_b[i] = in.ysz[0] * d2[i] * in.ysz[2];  // y1cnts
    } else {
      c_a[i] = in.ysz[0] * d1[i] * in.ysz[2];  // y2cnts
      c_b[i] = in.zsz[0] * in.zsz[1] * d2[i];  // z2cnts
    }
  }
  // x -> y and y -> z send the first set, receive the second; the reverse
  // transposes swap them
  const bool fwd = kind == GBFFT_X_TO_Y || kind == GBFFT_Y_TO_Z;
  const std::vector<int>& sd = fwd ? d1 : d2;
  const std::vector<int>& rd = fwd ? d2 : d1;
  const std::vector<int>& sc = fwd ? c_a : c_b;
  const std::vector<int>& rc_ = fwd ? c_b : c_a;
  int so = 0, ro = 0;
  for (int i = 0; i < p; ++i) {
    send_dist[i] = sd[i];
    recv_dist[i] = rd[i];
    send_cnts[i] = sc[i];
    recv_cnts[i] = rc_[i];
    send_disp[i] = so;
    recv_disp[i] = ro;
    so += sc[i];
    ro += rc_[i];
  }
  *npeers = p;
  return GBFFT_OK;
}
