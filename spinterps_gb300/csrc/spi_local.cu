// Interpolation from each cell's own neighbours: the neighbour methods
// 'nrst' / 'pie' of the step engine (interp/steps.py:584-606, 673-833).
// There, each group of cells with the same neighbour list is one call of
// _get_interp (interp/steps.py:245-401) with those stations alone; here one
// warp takes one (cell, step) and does what that call does for it:
// - one neighbour: its value (variance NaN);
// - NNB: the nearest neighbour's value (first on ties);
// - IDW: the mean of the neighbours where no value reaches
//   min_value_to_interp_thresh, else weights (d / max d)^-p over them (NaN
//   on a neighbour), as orc_idw_group / fill_wts_and_sum;
// - OK / SK / EDK: the mean (variance 0) where no value reaches the
//   threshold or the variogram is nugget-only; else the reference's saddle
//   matrix of the neighbours ([[Gamma, 1, S], [1', 0, 0], [S', 0, 0]],
//   SK: the covariances; fill_vg_var_arr entries with the min_vg_val cut)
//   solved with its right-hand side by Gauss-Jordan with partial pivoting
//   in shared memory (lanes over rows and columns), which is pinv's
//   solution for a nonsingular matrix; an exactly singular one gives the
//   nearest neighbour's value and marks the step as a problem step (the
//   reference's pinv failure branch). The sum check isclose(sum(lambda), 1)
//   falls back to the nearest neighbour (variance 0); the OK variance is
//   lambda'r + lambda_n (interp/steps.py:403-435).
// Estimates are clipped to the cut-offs (interp/steps.py:466-476).
// FP64 throughout: the systems have at most 64 stations.
#include "spi_common.cuh"

namespace spi {

constexpr int LOC_KMAX = SPI_LOCAL_MAX_NEBS;  // neighbours per cell

struct LocalArgs {
  spi_domain_t dom;
  int32_t kind;          // SPI_KIND_OK / SK / EDK, or 3 IDW, 4 NNB
  int32_t k;             // neighbour slots per cell
  const int32_t* nebs;   // [n_cells, k] station indices, -1 = empty slot
  int32_t n_steps;
  const int32_t* steps;  // data rows
  const int32_t* out_row;
  const double* data;    // [rows, ld] station values
  int64_t ld;
  const spi_vg_t* vg;    // [n_steps] (kriging)
  const int32_t* nug;    // [n_steps] nugget-only variogram (kriging)
  double min_var_thr;
  double idw_exp;
  int32_t want_var;
  int32_t m_max;         // saddle size bound (shared memory per warp)
  spi_out_t out;
  int32_t* prblm;        // [n_steps]
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename OutT>
__global__ void k_local(LocalArgs A) {
  extern __shared__ double lsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int ldm = A.m_max + 1;
  double* M = lsm + (int64_t)wib * A.m_max * ldm;  // this warp's [m][m + 1]
  const int64_t C = A.dom.n_cells;
  const int64_t ntask = C * A.n_steps;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  OutT* est_out = reinterpret_cast<OutT*>(A.out.est);
  OutT* var_out = reinterpret_cast<OutT*>(A.out.var);
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  const int krig = A.kind <= SPI_KIND_EDK;
  const int sk = A.kind == SPI_KIND_SK;
  const int nd = A.kind == SPI_KIND_EDK ? A.dom.n_drift : 0;
  const int a = krig ? (sk ? 0 : 1 + nd) : 0;

  for (int64_t t = w0; t < ntask; t += nw) {
    const int q = (int)(t / C);
    const int64_t cell = t - (int64_t)q * C;
    const int64_t row = A.out_row[q];
    const double* z = A.data + (int64_t)A.steps[q] * A.ld;
    const double cx = A.dom.cell_x[cell], cy = A.dom.cell_y[cell];
    const int32_t* nb = A.nebs + cell * A.k;
    // this lane's neighbours (slots lane, lane + 32)
    int s0 = -1, s1 = -1;
    if (lane < A.k) s0 = nb[lane];
    if (lane + 32 < A.k) s1 = nb[lane + 32];
    const int n = __popc(__ballot_sync(0xffffffffu, s0 >= 0)) +
                  __popc(__ballot_sync(0xffffffffu, s1 >= 0));
    const double z0 = s0 >= 0 ? z[s0] : 0.0, z1 = s1 >= 0 ? z[s1] : 0.0;
    // distances to the cell, and the nearest neighbour (first on ties)
    const double d0 = s0 >= 0 ? dist_f64(cx, cy, A.dom.stn_x[s0], A.dom.stn_y[s0]) : INFINITY;
    const double d1 = s1 >= 0 ? dist_f64(cx, cy, A.dom.stn_x[s1], A.dom.stn_y[s1]) : INFINITY;
    double bd = d0;
    int bi = lane;
    if (d1 < bd) {
      bd = d1;
      bi = lane + 32;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double od = __shfl_xor_sync(0xffffffffu, bd, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (od < bd || (od == bd && oi < bi)) {
        bd = od;
        bi = oi;
      }
    }
    const double znear = __shfl_sync(0xffffffffu, bi < 32 ? z0 : z1, bi & 31);
    const bool flag = __any_sync(0xffffffffu, (s0 >= 0 && z0 >= A.min_var_thr) ||
                                                  (s1 >= 0 && z1 >= A.min_var_thr));
    // the reference's mean of the neighbours' values
    const double mean = warp_sum((s0 >= 0 ? z0 : 0.0) + (s1 >= 0 ? z1 : 0.0)) / n;
    double est, var = nan;
    if (n == 1) {
      est = znear;
    } else if (A.kind == 4) {
      est = znear;
    } else if (A.kind == 3) {
      if (!flag) {
        est = mean;
      } else {
        double dmax = fmax(s0 >= 0 ? d0 : -INFINITY, s1 >= 0 ? d1 : -INFINITY);
        for (int o = 16; o > 0; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        auto wt = [&](double d) {
          const double r = dmax > 0.0 ? d / dmax : d;
          return (A.idw_exp == 2.0) ? 1.0 / (r * r)
                                    : (A.idw_exp == 1.0 ? 1.0 / r : 1.0 / pow(r, A.idw_exp));
        };
        const double w0 = s0 >= 0 ? wt(d0) : 0.0, w1 = s1 >= 0 ? wt(d1) : 0.0;
        const double ws = warp_sum(w0 + w1);
        const double wz = warp_sum((s0 >= 0 ? w0 * z0 : 0.0) + (s1 >= 0 ? w1 * z1 : 0.0));
        est = wz / ws;
      }
    } else if (!flag || A.nug[q]) {
      est = mean;
      var = 0.0;
    } else {
      // the saddle matrix and the right-hand side, augmented: M [m][m + 1]
      const spi_vg_t vg = A.vg[q];
      const int m = n + a;
      for (int e = lane; e < m * (m + 1); e += 32) {
        const int i = e / (m + 1), j = e - i * (m + 1);
        double v;
        if (j == m) {  // right-hand side
          if (i < n) {
            const int si = nb[i];
            v = vg_fill_f64(vg, dist_f64(cx, cy, A.dom.stn_x[si], A.dom.stn_y[si]), sk,
                            A.dom.min_vg_val);
          } else {
            v = (i == n) ? 1.0 : A.dom.cell_drift[(int64_t)(i - n - 1) * C + cell];
          }
        } else if (i < n && j < n) {
          const int lo = nb[min(i, j)], hi = nb[max(i, j)];
          v = vg_fill_f64(vg, dist_f64(A.dom.stn_x[lo], A.dom.stn_y[lo], A.dom.stn_x[hi],
                                       A.dom.stn_y[hi]),
                          sk, A.dom.min_vg_val);
        } else if (i >= n && j >= n) {
          v = 0.0;
        } else {
          const int st = nb[i < n ? i : j], kk = (i < n) ? (j - n) : (i - n);
          v = (kk == 0) ? 1.0 : A.dom.stn_drift[(int64_t)st * A.dom.n_drift + (kk - 1)];
        }
        M[i * ldm + j] = v;
      }
      __syncwarp();
      // Gauss-Jordan with partial pivoting (first row of maximum |pivot|)
      bool singular = false;
      for (int c = 0; c < m && !singular; ++c) {
        double best = -1.0;
        int bp = 0x7fffffff;
        for (int r = c + lane; r < m; r += 32) {
          const double x = fabs(M[r * ldm + c]);
          if (x > best || isnan(x)) {
            best = isnan(x) ? INFINITY : x;
            bp = r;
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const double ob = __shfl_xor_sync(0xffffffffu, best, o);
          const int op = __shfl_xor_sync(0xffffffffu, bp, o);
          if (ob > best || (ob == best && op < bp)) {
            best = ob;
            bp = op;
          }
        }
        if (!(best > 0.0) || isinf(best)) {
          singular = true;
          break;
        }
        if (bp != c)
          for (int j = c + lane; j <= m; j += 32) {
            const double tmp = M[c * ldm + j];
            M[c * ldm + j] = M[bp * ldm + j];
            M[bp * ldm + j] = tmp;
          }
        __syncwarp();
        const double piv = M[c * ldm + c];
        __syncwarp();
        for (int j = c + lane; j <= m; j += 32) M[c * ldm + j] /= piv;
        __syncwarp();
        for (int r = lane; r < m; r += 32) {
          if (r == c) continue;
          const double f = M[r * ldm + c];
          if (f != 0.0)
            for (int j = c; j <= m; ++j) M[r * ldm + j] -= f * M[c * ldm + j];
        }
        __syncwarp();
      }
      if (singular) {
        est = znear;
        var = 0.0;
        if (lane == 0) atomicOr(A.prblm + q, 1);
      } else {
        // lambda = M[:, m]; sum check over the stations' weights
        double sl = 0.0, ez = 0.0, lr = 0.0;
        for (int i = lane; i < m; i += 32) {
          const double l = M[i * ldm + m];
          if (i < n) {
            sl += l;
            ez += l * z[nb[i]];
          }
        }
        sl = warp_sum(sl);
        ez = warp_sum(ez);
        if (!isclose_one(sl)) {
          est = znear;
          var = 0.0;
        } else {
          est = ez;
          if (A.want_var && A.kind == SPI_KIND_OK) {
            // lambda'r + lambda_n, r rebuilt (M's column m now holds lambda)
            for (int i = lane; i < m; i += 32) {
              double r;
              if (i < n) {
                const int si = nb[i];
                r = vg_fill_f64(vg, dist_f64(cx, cy, A.dom.stn_x[si], A.dom.stn_y[si]), 0,
                                A.dom.min_vg_val);
              } else {
                r = 1.0;
              }
              lr += M[i * ldm + m] * r;
            }
            lr = warp_sum(lr);
            var = lr + M[n * ldm + m];
          }
        }
      }
      __syncwarp();
    }
    if (lane == 0) {
      est_out[row * C + cell] = cast_out<OutT>(clip_est(est, A.out));
      if (var_out && A.kind == SPI_KIND_OK) var_out[row * C + cell] = cast_out<OutT>(var);
    }
  }
}

}  // namespace spi

extern "C" int spi_local_cells(const spi_domain_t* dom, int32_t kind, int32_t k,
                               const int32_t* nebs, int32_t n_steps, const int32_t* steps,
                               const int32_t* out_row, const double* data, int64_t ld,
                               const spi_vg_t* vg, const int32_t* nug, double min_var_thr,
                               double idw_exp, int32_t want_var, const spi_out_t* out,
                               int32_t* prblm, spi_stream_t stream) {
  if (!dom || !out || kind < 0 || kind > 4 || k < 1 || n_steps < 0) return SPI_ERR_ARG;
  if (k > spi::LOC_KMAX) return SPI_ERR_TOO_LARGE;
  if (n_steps == 0 || dom->n_cells == 0) return SPI_OK;
  if (!nebs || !steps || !out_row || !data || !out->est || !dom->cell_x || !dom->cell_y ||
      !dom->stn_x || !dom->stn_y)
    return SPI_ERR_ARG;
  const bool krig = kind <= SPI_KIND_EDK;
  if (krig && (!vg || !nug || !prblm)) return SPI_ERR_ARG;
  if (kind == SPI_KIND_EDK && dom->n_drift > 0 && (!dom->stn_drift || !dom->cell_drift))
    return SPI_ERR_ARG;
  const int a = krig ? (kind == SPI_KIND_SK ? 0 : 1 + (kind == SPI_KIND_EDK ? dom->n_drift : 0))
                     : 0;
  const int m_max = krig ? k + a : 1;
  const size_t per_warp = (size_t)m_max * (m_max + 1) * sizeof(double);
  int warps = (int)((160 * 1024) / per_warp);
  warps = warps < 1 ? 1 : (warps > 8 ? 8 : warps);
  const size_t smem = krig ? per_warp * warps : 0;
  spi::LocalArgs A;
  A.dom = *dom;
  A.kind = kind;
  A.k = k;
  A.nebs = nebs;
  A.n_steps = n_steps;
  A.steps = steps;
  A.out_row = out_row;
  A.data = data;
  A.ld = ld;
  A.vg = vg;
  A.nug = nug;
  A.min_var_thr = min_var_thr;
  A.idw_exp = idw_exp;
  A.want_var = want_var;
  A.m_max = m_max;
  A.out = *out;
  A.prblm = prblm;
  const int64_t ntask = dom->n_cells * (int64_t)n_steps;
  int64_t blocks = (ntask + warps - 1) / warps;
  if (blocks > 152 * 64) blocks = 152 * 64;
  cudaStream_t st = (cudaStream_t)stream;
  if (out->out_f64) {
    if (!spi::smem_opt_in(spi::k_local<double>, smem)) return SPI_ERR_CUDA;
    spi::k_local<double><<<(unsigned)blocks, 32 * warps, smem, st>>>(A);
  } else {
    if (!spi::smem_opt_in(spi::k_local<float>, smem)) return SPI_ERR_CUDA;
    spi::k_local<float><<<(unsigned)blocks, 32 * warps, smem, st>>>(A);
  }
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
