// Drop-ins for the reference's Cython distance / variogram / gather kernels
// (cyth/interpmthds.pyx:123-248). These materialise full matrices and are
// the boundary-compatible path; the batched kernels of spi_factor.cu and
// spi_cells.cu fuse the same arithmetic and never write these matrices.
//
// All three are HBM-write bound: one thread per output element, consecutive
// threads on consecutive columns (coalesced stores), grid-stride loops with
// the grid sized to the SM count.
#include "spi_common.cuh"

namespace spi {

__global__ void k_fill_dists(const double* __restrict__ x1s, const double* __restrict__ y1s,
                             int64_t n1, const double* __restrict__ x2s,
                             const double* __restrict__ y2s, int64_t n2,
                             double* __restrict__ out) {
  int64_t total = n1 * n2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / n2, j = e - i * n2;
    out[e] = dist_f64(x1s[i], y1s[i], x2s[j], y2s[j]);
  }
}

// fill_vg_var_arr: with diag the lower triangle is the mirror of the upper
// one, which is what evaluating at dists[g, h] == dists[h, g] gives; the
// mirror is taken explicitly so that a non-symmetric input behaves as in
// the reference.
__global__ void k_fill_vg(const double* __restrict__ dists, int64_t rows, int64_t cols,
                          double* __restrict__ out, int covar, int diag, spi_vg_t vg,
                          double min_vg_val) {
  int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t h = e / cols, g = e - h * cols;
    int64_t src = (diag && g < h) ? (g * cols + h) : e;
    if (diag && g < h && (g >= rows || h >= cols)) {
      // mirror source outside a non-square matrix: the reference reads
      // in_vars[g, h], which was zero-initialised and never filled.
      out[e] = 0.0;
      continue;
    }
    out[e] = vg_fill_f64(vg, dists[src], covar, min_vg_val);
  }
}

__global__ void k_copy_at_idxs(const double* __restrict__ arr, int64_t arr_cols,
                               const int64_t* __restrict__ ri, int64_t nr,
                               const int64_t* __restrict__ ci, int64_t nc,
                               double* __restrict__ sub, int64_t sub_cols) {
  int64_t total = nr * nc;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / nc, j = e - i * nc;
    sub[i * sub_cols + j] = arr[ri[i] * arr_cols + ci[j]];
  }
}

static int grid_for(int64_t total, int threads) {
  static int n_sm = 0;
  if (n_sm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (n_sm <= 0) n_sm = 1;
  }
  int64_t want = (total + threads - 1) / threads;
  int64_t cap = (int64_t)n_sm * 8;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

}  // namespace spi

using namespace spi;

extern "C" int spi_fill_dists_2d_mat(const double* x1s, const double* y1s, int64_t n1,
                                     const double* x2s, const double* y2s, int64_t n2,
                                     double* dists, spi_stream_t stream) {
  if (n1 < 0 || n2 < 0) return SPI_ERR_ARG;
  if (n1 == 0 || n2 == 0) return SPI_OK;
  if (!x1s || !y1s || !x2s || !y2s || !dists) return SPI_ERR_ARG;
  k_fill_dists<<<grid_for(n1 * n2, 256), 256, 0, (cudaStream_t)stream>>>(x1s, y1s, n1, x2s,
                                                                         y2s, n2, dists);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_fill_vg_var_arr(const double* dists, int64_t rows, int64_t cols,
                                   double* out, int32_t covar_flag, int32_t diag_mat_flag,
                                   const spi_vg_t* vg, double min_vg_val,
                                   spi_stream_t stream) {
  if (rows < 0 || cols < 0 || !vg) return SPI_ERR_ARG;
  if (vg->n_comp < 1 || vg->n_comp > SPI_MAX_VG_COMP) return SPI_ERR_VG;
  for (int c = 0; c < vg->n_comp; ++c)
    if (vg->code[c] < SPI_VG_RNG || vg->code[c] > SPI_VG_HOL) return SPI_ERR_VG;
  if (rows == 0 || cols == 0) return SPI_OK;
  if (!dists || !out) return SPI_ERR_ARG;
  k_fill_vg<<<grid_for(rows * cols, 256), 256, 0, (cudaStream_t)stream>>>(
      dists, rows, cols, out, covar_flag ? 1 : 0, diag_mat_flag ? 1 : 0, *vg, min_vg_val);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_copy_2d_arr_at_idxs(const double* arr, int64_t arr_rows, int64_t arr_cols,
                                       const int64_t* row_idxs, int64_t n_rows,
                                       const int64_t* col_idxs, int64_t n_cols,
                                       double* subset, int64_t subset_cols,
                                       spi_stream_t stream) {
  if (n_rows < 0 || n_cols < 0 || arr_rows < 0 || arr_cols < 0) return SPI_ERR_ARG;
  if (subset_cols < n_cols) return SPI_ERR_ARG;
  if (n_rows == 0 || n_cols == 0) return SPI_OK;
  if (!arr || !row_idxs || !col_idxs || !subset) return SPI_ERR_ARG;
  (void)arr_rows;  // indices are validated by the host mirror before the call
  k_copy_at_idxs<<<grid_for(n_rows * n_cols, 256), 256, 0, (cudaStream_t)stream>>>(
      arr, arr_cols, row_idxs, n_rows, col_idxs, n_cols, subset, subset_cols);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
