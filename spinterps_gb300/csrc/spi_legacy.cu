// The single-neighbourhood kriging classes of cyth/interpmthds.pyx:251-765
// (OrdinaryKriging, SimpleKriging, ExternalDriftKriging(_MD) and the two
// indicator classes): one station set, one variogram, a list of output
// points, every intermediate array materialised as the classes expose it.
//
// Their semantics differ from the step engine's fill_vg_var_arr matrices:
// - the station semivariogram matrix sums the components for i != j and is
//   0 on the diagonal, and a point's right-hand side is 0 at distance 0, so
//   a nugget is a discontinuity at h = 0 (the step engine takes the sill);
// - no min_vg_val cut, no sum check, no nearest-station fallback;
// - SimpleKriging's matrix is -gamma with a zero diagonal: __init__ fills it
//   with the total sill before krige() has summed it (still 0.0), and
//   krige() subtracts gamma off the diagonal (lines 397-399, 413, 432-442); its
//   right-hand side is total sill - gamma (total sill at distance 0).
//
// Kernels: k_leg_system (one CTA: distances, the matrix, its Gauss-Jordan
// inverse in place of numpy.linalg.pinv); k_leg_rhs (every point's
// right-hand side, grid-stride); k_leg_lambda (lambda = P r for every
// point: an FP64 tiled contraction R P' over shared-memory tiles);
// k_leg_finish (a warp per point: estimate, variance, indicator).
#include "spi_common.cuh"
#include "spi_gj.cuh"

namespace spi {

constexpr int LT = 512;        // threads of the system CTA
constexpr int LG_T = 64;       // lambda tile (points and matrix rows)
constexpr int LG_K = 16;       // lambda tile depth

__device__ __forceinline__ double leg_gamma(const spi_vg_t& vg, double d) {
  double t = 0.0;
  for (int c = 0; c < vg.n_comp; ++c) t = __dadd_rn(t, vg_eval_f64(vg.code[c], d, vg.range[c], vg.sill[c]));
  return t;
}

__device__ __forceinline__ double leg_cov(const spi_vg_t& vg, double covar, double d) {
  double t = covar;
  for (int c = 0; c < vg.n_comp; ++c) t = __dsub_rn(t, vg_eval_f64(vg.code[c], d, vg.range[c], vg.sill[c]));
  return t;
}

__device__ __forceinline__ double leg_total_sill(const spi_vg_t& vg) {
  double t = 0.0;
  for (int c = 0; c < vg.n_comp; ++c) t = __dadd_rn(t, vg.sill[c]);
  return t;
}

// Distances, the kriging matrix and its inverse of one station set.
__global__ __launch_bounds__(LT) void k_leg_system(int sk, const double* __restrict__ xi,
                                                   const double* __restrict__ yi, int n,
                                                   const double* __restrict__ si, int n_drift,
                                                   spi_vg_t vg, double* __restrict__ dists,
                                                   double* __restrict__ lhs,
                                                   double* __restrict__ inv,
                                                   int32_t* __restrict__ status,
                                                   double* __restrict__ cond) {
  const int tid = threadIdx.x;
  const int a = sk ? 0 : 1 + n_drift;
  const int m = n + a;
  for (int64_t e = tid; e < (int64_t)m * m; e += LT) {
    const int i = (int)(e / m), j = (int)(e - (int64_t)i * m);
    double val;
    if (i < n && j < n) {
      double d = 0.0;
      val = 0.0;
      if (i != j) {
        const int lo = min(i, j), hi = max(i, j);
        d = dist_f64(xi[lo], yi[lo], xi[hi], yi[hi]);
        const double g = leg_gamma(vg, d);
        // SK: 0.0 - g_0 - g_1 ... == -(g_0 + g_1 + ...) exactly
        val = sk ? -g : g;
      }
      dists[(int64_t)i * n + j] = d;
    } else if (i >= n && j >= n) {
      val = 0.0;
    } else {
      const int st = (i < n) ? i : j;
      const int k = (i < n) ? (j - n) : (i - n);
      val = (k == 0) ? 1.0 : si[(int64_t)(k - 1) * n + st];
    }
    lhs[e] = val;
    inv[e] = val;
  }
  __syncthreads();
  extern __shared__ double lsm[];
  double* f = lsm;
  double* prow = lsm + m;
  int* piv = reinterpret_cast<int*>(lsm + 2 * m);
  const int fail = gj_invert<LT>(inv, m, f, prow, piv);
  // ||lhs||_F ||inv||_F >= cond_2: where it stays under 1 / (m eps), pinv's
  // cut-off removes no singular value and pinv is this inverse
  __shared__ double red[2][LT / 32];
  double sa = 0.0, sb = 0.0;
  if (!fail)
    for (int64_t e = tid; e < (int64_t)m * m; e += LT) {
      sa = fma(lhs[e], lhs[e], sa);
      sb = fma(inv[e], inv[e], sb);
    }
  for (int o = 16; o > 0; o >>= 1) {
    sa += __shfl_xor_sync(0xffffffffu, sa, o);
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = sa;
    red[1][tid >> 5] = sb;
  }
  __syncthreads();
  if (tid == 0) {
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < LT / 32; ++w) {
      ta += red[0][w];
      tb += red[1][w];
    }
    status[0] = fail;
    if (cond) cond[0] = fail ? __longlong_as_double(0x7ff0000000000000LL) : sqrt(ta) * sqrt(tb);
  }
}

// rhss[k, :] of every point k.
__global__ void k_leg_rhs(int sk, const double* __restrict__ xi, const double* __restrict__ yi,
                          int n, const double* __restrict__ xk, const double* __restrict__ yk,
                          const double* __restrict__ skd, int64_t n_out, int n_drift,
                          spi_vg_t vg, double* __restrict__ rhss) {
  const int a = sk ? 0 : 1 + n_drift;
  const int m = n + a;
  const double covar = leg_total_sill(vg);
  const int64_t total = n_out * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = e / m;
    const int j = (int)(e - k * m);
    double v;
    if (j < n) {
      const double d = dist_f64(xi[j], yi[j], xk[k], yk[k]);
      if (d == 0.0)
        v = sk ? covar : 0.0;
      else
        v = sk ? leg_cov(vg, covar, d) : leg_gamma(vg, d);
    } else if (j == n) {
      v = 1.0;
    } else {
      v = skd[(int64_t)(j - n - 1) * n_out + k];
    }
    rhss[e] = v;
  }
}

// lambda_full[k, i] = sum_j rhss[k, j] inv[i, j]; entries i < n go to
// lambdas[k, i], the rest to mus[i - n, k]. Block: LG_T points x LG_T
// rows, 256 threads with 4 x 4 outputs each.
__global__ __launch_bounds__(256) void k_leg_lambda(const double* __restrict__ rhss,
                                                    const double* __restrict__ inv, int64_t n_out,
                                                    int n, int m, double* __restrict__ lambdas,
                                                    double* __restrict__ mus) {
  __shared__ double rs[LG_K][LG_T + 1];
  __shared__ double ps[LG_K][LG_T + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t k0 = (int64_t)blockIdx.x * LG_T;
  const int i0 = blockIdx.y * LG_T;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;
  for (int j0 = 0; j0 < m; j0 += LG_K) {
#pragma unroll
    for (int q = 0; q < (LG_T * LG_K) / 256; ++q) {
      const int e = tid + q * 256;
      const int row = e / LG_K, col = e % LG_K;
      const int64_t kk = k0 + row;
      const int ii = i0 + row, jj = j0 + col;
      rs[col][row] = (kk < n_out && jj < m) ? rhss[kk * m + jj] : 0.0;
      ps[col][row] = (ii < m && jj < m) ? inv[(int64_t)ii * m + jj] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int jj = 0; jj < LG_K; ++jj) {
      double rv[4], pv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) rv[r] = rs[jj][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) pv[c] = ps[jj][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fma(rv[r], pv[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int64_t k = k0 + ty * 4 + r;
    if (k >= n_out) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + tx * 4 + c;
      if (i < n)
        lambdas[k * n + i] = acc[r][c];
      else if (i < m)
        mus[(int64_t)(i - n) * n_out + k] = acc[r][c];
    }
  }
}

// A warp per point: zk = lambda'z; OK: est = max(0, lambda'r + mu);
// SK: est = max(0, total sill - lambda'c); with ixi (the indicator
// classes' ikrige): ik = max(0, lambda'ixi), est = max(0, ik (1 - ik)).
__global__ void k_leg_finish(int sk, const double* __restrict__ zi,
                             const double* __restrict__ ixi, int n, int64_t n_out, int m,
                             spi_vg_t vg, const double* __restrict__ rhss,
                             const double* __restrict__ lambdas, const double* __restrict__ mus,
                             double* __restrict__ zk, double* __restrict__ est,
                             double* __restrict__ ik) {
  const int lane = threadIdx.x & 31;
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (k >= n_out) return;
  const double* lam = lambdas + k * n;
  const double* r = rhss + k * m;
  double tz = 0.0, tr = 0.0, ti = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double l = lam[i];
    tz = fma(l, zi[i], tz);
    tr = fma(l, r[i], tr);
    if (ixi) ti = fma(l, ixi[i], ti);
  }
  for (int o = 16; o > 0; o >>= 1) {
    tz += __shfl_xor_sync(0xffffffffu, tz, o);
    tr += __shfl_xor_sync(0xffffffffu, tr, o);
    ti += __shfl_xor_sync(0xffffffffu, ti, o);
  }
  if (lane == 0) {
    zk[k] = tz;
    if (ixi) {
      const double p = fmax(0.0, ti);
      ik[k] = p;
      if (est) est[k] = fmax(0.0, p * (1.0 - p));
    } else if (est) {
      est[k] = sk ? fmax(0.0, leg_total_sill(vg) - tr) : fmax(0.0, tr + mus[k]);
    }
  }
}

}  // namespace spi

static int leg_check(int32_t kind, const double* xi, const double* yi, int32_t n,
                     const double* si, int32_t n_drift, const spi_vg_t* vg) {
  if (kind != SPI_KIND_OK && kind != SPI_KIND_SK && kind != SPI_KIND_EDK) return SPI_ERR_ARG;
  if (!xi || !yi || !vg || n < 1 || n_drift < 0) return SPI_ERR_ARG;
  if (vg->n_comp < 1 || vg->n_comp > SPI_MAX_VG_COMP) return SPI_ERR_VG;
  if (kind == SPI_KIND_EDK && (n_drift < 1 || !si)) return SPI_ERR_ARG;
  if (kind != SPI_KIND_EDK && n_drift != 0) return SPI_ERR_ARG;
  return SPI_OK;
}

extern "C" int spi_legacy_system(int32_t kind, const double* xi, const double* yi, int32_t n,
                                 const double* si, int32_t n_drift, const spi_vg_t* vg,
                                 double* in_dists, double* lhs, double* lhs_inv,
                                 int32_t* status, double* cond, spi_stream_t stream) {
  int rc = leg_check(kind, xi, yi, n, si, n_drift, vg);
  if (rc) return rc;
  if (!in_dists || !lhs || !lhs_inv || !status) return SPI_ERR_ARG;
  const int sk = kind == SPI_KIND_SK;
  const int64_t m = (int64_t)n + (sk ? 0 : 1 + n_drift);
  const size_t smem = (size_t)m * (2 * sizeof(double) + sizeof(int));
  if (smem > 200 * 1024) return SPI_ERR_TOO_LARGE;
  if (!spi::smem_opt_in(spi::k_leg_system, smem)) return SPI_ERR_CUDA;
  spi::k_leg_system<<<1, spi::LT, smem, (cudaStream_t)stream>>>(sk, xi, yi, n, si, n_drift, *vg,
                                                                in_dists, lhs, lhs_inv, status,
                                                                cond);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_legacy_points(int32_t kind, const double* xi, const double* yi,
                                 const double* zi, const double* ixi, int32_t n,
                                 const double* xk, const double* yk, const double* sk_drift,
                                 int64_t n_out, int32_t n_drift, const spi_vg_t* vg,
                                 const double* lhs_inv, double* rhss, double* lambdas,
                                 double* mus, double* zk, double* est, double* ik,
                                 spi_stream_t stream) {
  int rc = leg_check(kind, xi, yi, n, sk_drift, n_drift, vg);
  if (rc) return rc;
  if (n_out < 0) return SPI_ERR_ARG;
  if (n_out == 0) return SPI_OK;
  const int sk = kind == SPI_KIND_SK;
  const int a = sk ? 0 : 1 + n_drift;
  if (!zi || !xk || !yk || !lhs_inv || !rhss || !lambdas || !zk) return SPI_ERR_ARG;
  if (a > 0 && !mus) return SPI_ERR_ARG;
  if (ixi && !ik) return SPI_ERR_ARG;
  const int m = n + a;
  if ((n_out + spi::LG_T - 1) / spi::LG_T > 0x7fffffff || (n_out * 32 + 255) / 256 > 0x7fffffff)
    return SPI_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  spi::k_leg_rhs<<<152 * 16, 256, 0, st>>>(sk, xi, yi, n, xk, yk, sk_drift, n_out, n_drift, *vg,
                                          rhss);
  SPI_LAUNCH_CHECK();
  dim3 grid((unsigned)((n_out + spi::LG_T - 1) / spi::LG_T),
            (unsigned)((m + spi::LG_T - 1) / spi::LG_T));
  spi::k_leg_lambda<<<grid, 256, 0, st>>>(rhss, lhs_inv, n_out, n, m, lambdas, mus);
  SPI_LAUNCH_CHECK();
  spi::k_leg_finish<<<(unsigned)((n_out * 32 + 255) / 256), 256, 0, st>>>(
      sk, zi, ixi, n, n_out, m, *vg, rhss, lambdas, mus, zk, est, ik);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
