// Kriging from each cell's own neighbours, one system per neighbour group:
// the reference's neighbour methods 'nrst' / 'pie' (interp/steps.py:584-606,
// 673-833) call _get_interp (interp/steps.py:245-401) once per group of
// cells with identical neighbour lists; for every step it inverts the
// group's matrix once (np.linalg.pinv, interp/steps.py:351-352) and then
// forms lmds = inv @ rhs per cell (_fill_krig_idw_dst_data,
// interp/steps.py:403-435). Here likewise:
// - k_grp_factor: one warp per (group, step) builds the group's saddle
//   matrix ([[Gamma, 1, S], [1', 0, 0], [S', 0, 0]], SK: the covariances)
//   in shared memory and inverts it in place by Gauss-Jordan with partial
//   pivoting (row interchanges, undone as column interchanges at the end).
//   Groups whose inverse is suspect (||M||_F ||P||_F > 1e15, or a zero
//   pivot) go to spi_local_grp_pinv (csrc/spi_pinv.cu), which replaces the
//   inverse by numpy.linalg.pinv's truncated inverse by the rule of the
//   global engine's route-1 check, or marks the (group, step) singular.
//   Steps where no neighbour value reaches the threshold, or with a
//   nugget-only variogram, or groups of one station need no system.
// - k_grp_apply: one thread per (cell, step), cells in group order so that
//   a warp's threads read the same inverse: the right-hand side (the
//   variogram to each neighbour, 1, the cell's drifts), lambda = inv @ rhs,
//   the sum check isclose(sum(lambda[:n]), 1) with its nearest-neighbour
//   fallback, the estimate lambda[:n]' z and the OK variance
//   sum(lambda * rhs) + lambda[n], in the reference's order of operations;
//   the mean (variance 0) where no value reaches the threshold or the
//   variogram is nugget-only; a single neighbour's value (variance NaN);
//   the nearest neighbour (variance 0) and a problem step where the group's
//   system is singular.
// FP64 throughout. Steps are processed in chunks that fit the caller's
// scratch.
#include "spi_common.cuh"
#include "spi_saddle.cuh"

namespace spi {

// Gauss-Jordan suspects handed to the pinv check (csrc/spi_pinv.cu).
int local_grp_pinv(const spi_domain_t& dom, int kind, int k, const int32_t* grp_nebs,
                   int32_t n_grps, int32_t q0, int32_t nq, const spi_vg_t* vg, double* inv,
                   int32_t ld, int32_t* status, double* pinv_scratch, int32_t* prblm,
                   cudaStream_t st);

namespace {

constexpr int GF_WARPS_MAX = 8;   // warps per CTA of k_grp_factor
constexpr int GA_T = 128;         // threads per CTA of k_grp_apply
constexpr double kCondSuspect = 1e15;

enum : int32_t { GRP_OK = 0, GRP_SINGULAR = 1, GRP_NONE = 2, GRP_SUSPECT = 3, GRP_ZERO_PIV = 4 };

struct GrpArgs {
  spi_domain_t dom;
  int32_t kind;
  int32_t k;
  const int32_t* grp_nebs;  // [n_grps, k]
  int32_t n_grps;
  const int32_t* cell_grp;  // [n_cells]
  const int32_t* order;     // [n_cells] or null
  const int32_t* steps;
  const int32_t* out_row;
  const double* data;
  int64_t ld;
  const spi_vg_t* vg;
  const int32_t* nug;
  double min_var_thr;
  int32_t want_var;
  int32_t m_max;
  spi_out_t out;
  int32_t* prblm;
};

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Neighbour slots in use (the valid ones come first).
__device__ __forceinline__ int group_size(const int32_t* nb, int k) {
  int n = 0;
  while (n < k && nb[n] >= 0) ++n;
  return n;
}

__global__ void k_grp_factor(GrpArgs A, int32_t q0, int32_t nq, double* __restrict__ inv,
                             int32_t* __restrict__ status) {
  extern __shared__ double gsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int mm = A.m_max;
  double* M = gsm + (int64_t)wib * (mm * mm + mm);  // [mm][mm], then the column f
  double* f = M + mm * mm;
  const int sk = A.kind == SPI_KIND_SK;
  const int a = extra_rows(A.kind, A.dom.n_drift);
  const int64_t G = A.n_grps;
  const int64_t ntask = G * nq;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = w0; t < ntask; t += nw) {
    const int ql = (int)(t / G);
    const int64_t g = t - (int64_t)ql * G;
    const int q = q0 + ql;
    const int32_t* nb = A.grp_nebs + g * A.k;
    const int n = group_size(nb, A.k);
    const double* z = A.data + (int64_t)A.steps[q] * A.ld;
    bool flag = false;
    for (int i = lane; i < n; i += 32) flag |= z[nb[i]] >= A.min_var_thr;
    flag = __any_sync(0xffffffffu, flag);
    if (n <= 1 || !flag || A.nug[q]) {
      if (lane == 0) status[t] = GRP_NONE;
      continue;
    }
    const spi_vg_t vg = A.vg[q];
    const int m = n + a;
    double fm = 0.0;
    for (int e = lane; e < m * m; e += 32) {
      const int i = e / m, j = e - i * m;
      const double x = saddle_entry(A.dom, vg, nb, n, sk, i, j);
      M[i * mm + j] = x;
      fm += x * x;
    }
    fm = warp_sum_d(fm);
    __syncwarp();
    // in-place Gauss-Jordan inversion; piv[c] kept in lane c % 32's
    // register slot c / 32
    int piv0 = 0, piv1 = 0, piv2 = 0;
    bool zero_piv = false;
    for (int c = 0; c < m; ++c) {
      double best = -1.0;
      int bp = 0x7fffffff;
      for (int r = c + lane; r < m; r += 32) {
        const double x = fabs(M[r * mm + c]);
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
        zero_piv = true;
        break;
      }
      if (lane == (c & 31)) {
        if (c < 32) piv0 = bp;
        else if (c < 64) piv1 = bp;
        else piv2 = bp;
      }
      if (bp != c)
        for (int j = lane; j < m; j += 32) {
          const double tmp = M[c * mm + j];
          M[c * mm + j] = M[bp * mm + j];
          M[bp * mm + j] = tmp;
        }
      __syncwarp();
      const double d = M[c * mm + c];
      __syncwarp();
      for (int j = lane; j < m; j += 32) M[c * mm + j] = (j == c ? 1.0 : M[c * mm + j]) / d;
      for (int i = lane; i < m; i += 32) f[i] = M[i * mm + c];
      __syncwarp();
      for (int j = lane; j < m; j += 32) {
        const double rc = M[c * mm + j];
        for (int i = 0; i < m; ++i) {
          if (i == c) continue;
          const double fi = f[i];
          if (fi != 0.0) M[i * mm + j] = (j == c ? 0.0 : M[i * mm + j]) - fi * rc;
        }
      }
      __syncwarp();
    }
    if (zero_piv) {
      if (lane == 0) status[t] = GRP_ZERO_PIV;
      __syncwarp();
      continue;
    }
    // undo the row interchanges as column interchanges, last first
    for (int c = m - 1; c >= 0; --c) {
      const int src = c & 31;
      const int p = __shfl_sync(0xffffffffu, c < 32 ? piv0 : (c < 64 ? piv1 : piv2), src);
      if (p != c)
        for (int i = lane; i < m; i += 32) {
          const double tmp = M[i * mm + c];
          M[i * mm + c] = M[i * mm + p];
          M[i * mm + p] = tmp;
        }
      __syncwarp();
    }
    double* P = inv + t * (int64_t)mm * mm;
    double fp = 0.0;
    for (int e = lane; e < m * m; e += 32) {
      const int i = e / m, j = e - i * m;
      const double x = M[i * mm + j];
      P[i * mm + j] = x;
      fp += x * x;
    }
    fp = warp_sum_d(fp);
    if (lane == 0) status[t] = (sqrt(fm) * sqrt(fp) <= kCondSuspect) ? GRP_OK : GRP_SUSPECT;
    __syncwarp();
  }
}

template <typename OutT>
__global__ __launch_bounds__(GA_T) void k_grp_apply(GrpArgs A, int32_t q0, int32_t nq,
                                                    const double* __restrict__ inv,
                                                    const int32_t* __restrict__ status) {
  extern __shared__ double bsm[];  // [m_max][GA_T]: each thread's right-hand side
  double* b = bsm + threadIdx.x;
  const int64_t C = A.dom.n_cells;
  const int64_t G = A.n_grps;
  const int mm = A.m_max;
  const int sk = A.kind == SPI_KIND_SK;
  const int nd = A.kind == SPI_KIND_EDK ? A.dom.n_drift : 0;
  const int a = extra_rows(A.kind, A.dom.n_drift);
  const bool var_ok = A.want_var && A.kind == SPI_KIND_OK && A.out.var;
  OutT* est_out = reinterpret_cast<OutT*>(A.out.est);
  OutT* var_out = reinterpret_cast<OutT*>(A.out.var);
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  const int64_t ntask = C * nq;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ntask;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int ql = (int)(t / C);
    const int64_t i = t - (int64_t)ql * C;
    const int64_t cell = A.order ? A.order[i] : i;
    const int64_t g = A.cell_grp[cell];
    const int q = q0 + ql;
    const int64_t row = A.out_row[q];
    const double* z = A.data + (int64_t)A.steps[q] * A.ld;
    const int32_t* nb = A.grp_nebs + g * A.k;
    const int n = group_size(nb, A.k);
    const double cx = A.dom.cell_x[cell], cy = A.dom.cell_y[cell];
    // distances (kept in b until the right-hand side replaces them), the
    // nearest neighbour (first on ties), the threshold flag and the mean
    double bd = INFINITY, znear = 0.0, zsum = 0.0;
    bool flag = false;
    for (int j = 0; j < n; ++j) {
      const int s = nb[j];
      const double d = dist_f64(cx, cy, A.dom.stn_x[s], A.dom.stn_y[s]);
      const double zj = z[s];
      b[(int64_t)j * GA_T] = d;
      if (d < bd) {
        bd = d;
        znear = zj;
      }
      flag |= zj >= A.min_var_thr;
      zsum += zj;
    }
    double est, var = nan;
    if (n == 1) {
      est = z[nb[0]];
    } else if (!flag || A.nug[q]) {
      est = zsum / n;
      var = 0.0;
    } else if (status[(int64_t)ql * G + g] != GRP_OK) {
      est = znear;
      var = 0.0;
    } else {
      const spi_vg_t vg = A.vg[q];
      const int m = n + a;
      for (int j = 0; j < n; ++j)
        b[(int64_t)j * GA_T] = vg_fill_f64(vg, b[(int64_t)j * GA_T], sk, A.dom.min_vg_val);
      if (a > 0) b[(int64_t)n * GA_T] = 1.0;
      for (int e = 0; e < nd; ++e)
        b[(int64_t)(n + 1 + e) * GA_T] = A.dom.cell_drift[(int64_t)e * C + cell];
      const double* P = inv + ((int64_t)ql * G + g) * mm * mm;
      double sl = 0.0, ez = 0.0, lr = 0.0, ln = 0.0;
      for (int r = 0; r < m; ++r) {
        const double* pr = P + (int64_t)r * mm;
        double l = 0.0;
        for (int j = 0; j < m; ++j) l = fma(pr[j], b[(int64_t)j * GA_T], l);
        if (r < n) {
          sl += l;
          ez = fma(l, z[nb[r]], ez);
        }
        lr = fma(l, b[(int64_t)r * GA_T], lr);
        if (r == n) ln = l;
      }
      if (!isclose_one(sl)) {
        est = znear;
        var = 0.0;
      } else {
        est = ez;
        var = lr + ln;
      }
    }
    est_out[row * C + cell] = cast_out<OutT>(clip_est(est, A.out));
    if (var_ok) var_out[row * C + cell] = cast_out<OutT>(var);
  }
}

}  // namespace
}  // namespace spi

extern "C" int64_t spi_local_groups_scratch_bytes(int32_t kind, int32_t k, int32_t n_drift,
                                                  int32_t n_grps, int32_t n_steps) {
  if (kind < 0 || kind > SPI_KIND_EDK || k < 1 || n_grps < 0 || n_steps < 0 || n_drift < 0)
    return -1;
  const int64_t mm = k + spi::extra_rows(kind, n_drift);
  return SPI_LOCAL_GRP_PINV_BYTES(mm) + (int64_t)n_grps * n_steps * SPI_LOCAL_GRP_BYTES(mm);
}

extern "C" int spi_local_groups(const spi_domain_t* dom, int32_t kind, int32_t k,
                                const int32_t* grp_nebs, int32_t n_grps,
                                const int32_t* cell_grp, const int32_t* cell_order,
                                int32_t n_steps, const int32_t* steps, const int32_t* out_row,
                                const double* data, int64_t ld, const spi_vg_t* vg,
                                const int32_t* nug, double min_var_thr, int32_t want_var,
                                const spi_out_t* out, void* scratch, int64_t scratch_bytes,
                                int32_t* prblm, spi_stream_t stream) {
  if (!dom || !out || kind < 0 || kind > SPI_KIND_EDK || k < 1 || n_steps < 0 || n_grps < 0)
    return SPI_ERR_ARG;
  if (k > SPI_LOCAL_MAX_NEBS) return SPI_ERR_TOO_LARGE;
  if (n_steps == 0 || dom->n_cells == 0) return SPI_OK;
  if (n_grps == 0 || !grp_nebs || !cell_grp || !steps || !out_row || !data || !vg || !nug ||
      !prblm || !scratch || !out->est || !dom->cell_x || !dom->cell_y || !dom->stn_x ||
      !dom->stn_y)
    return SPI_ERR_ARG;
  if (kind == SPI_KIND_EDK && dom->n_drift > 0 && (!dom->stn_drift || !dom->cell_drift))
    return SPI_ERR_ARG;
  if (reinterpret_cast<uintptr_t>(scratch) % 16 != 0) return SPI_ERR_ARG;
  const int a = spi::extra_rows(kind, dom->n_drift);
  const int mm = k + a;
  if (mm > SPI_LOCAL_MAX_NEBS + 8) return SPI_ERR_TOO_LARGE;
  const int64_t per = SPI_LOCAL_GRP_BYTES(mm);
  const int64_t fixed = SPI_LOCAL_GRP_PINV_BYTES(mm);
  const int64_t per_step = per * n_grps;
  if (scratch_bytes < fixed + per_step) return SPI_ERR_TOO_LARGE;
  const int64_t q_fit = (scratch_bytes - fixed) / per_step;
  const int32_t nq_max = (int32_t)(q_fit < n_steps ? q_fit : n_steps);
  double* pinv_ws = reinterpret_cast<double*>(scratch);
  double* inv = reinterpret_cast<double*>(reinterpret_cast<char*>(scratch) + fixed);
  int32_t* status = reinterpret_cast<int32_t*>(inv + (int64_t)nq_max * n_grps * mm * mm);

  spi::GrpArgs A;
  A.dom = *dom;
  A.kind = kind;
  A.k = k;
  A.grp_nebs = grp_nebs;
  A.n_grps = n_grps;
  A.cell_grp = cell_grp;
  A.order = cell_order;
  A.steps = steps;
  A.out_row = out_row;
  A.data = data;
  A.ld = ld;
  A.vg = vg;
  A.nug = nug;
  A.min_var_thr = min_var_thr;
  A.want_var = want_var;
  A.m_max = mm;
  A.out = *out;
  A.prblm = prblm;

  const size_t per_warp = ((size_t)mm * mm + mm) * sizeof(double);
  int warps = (int)((160 * 1024) / per_warp);
  warps = warps < 1 ? 1 : (warps > spi::GF_WARPS_MAX ? spi::GF_WARPS_MAX : warps);
  const size_t fsmem = per_warp * warps;
  const size_t asmem = (size_t)mm * spi::GA_T * sizeof(double);
  if (!spi::smem_opt_in(spi::k_grp_factor, fsmem)) return SPI_ERR_CUDA;
  if (out->out_f64) {
    if (!spi::smem_opt_in(spi::k_grp_apply<double>, asmem)) return SPI_ERR_CUDA;
  } else {
    if (!spi::smem_opt_in(spi::k_grp_apply<float>, asmem)) return SPI_ERR_CUDA;
  }
  cudaStream_t st = (cudaStream_t)stream;
  for (int32_t q0 = 0; q0 < n_steps; q0 += nq_max) {
    const int32_t nq = (n_steps - q0) < nq_max ? (n_steps - q0) : nq_max;
    const int64_t ftask = (int64_t)n_grps * nq;
    int64_t fblocks = (ftask + warps - 1) / warps;
    if (fblocks > 152 * 64) fblocks = 152 * 64;
    spi::k_grp_factor<<<(unsigned)fblocks, 32 * warps, fsmem, st>>>(A, q0, nq, inv, status);
    SPI_LAUNCH_CHECK();
    const int rc = spi::local_grp_pinv(*dom, kind, k, grp_nebs, n_grps, q0, nq, vg, inv, mm,
                                       status, pinv_ws, prblm, st);
    if (rc != SPI_OK) return rc;
    const int64_t atask = dom->n_cells * (int64_t)nq;
    int64_t ablocks = (atask + spi::GA_T - 1) / spi::GA_T;
    if (ablocks > 152 * 32) ablocks = 152 * 32;
    if (out->out_f64)
      spi::k_grp_apply<double><<<(unsigned)ablocks, spi::GA_T, asmem, st>>>(A, q0, nq, inv,
                                                                            status);
    else
      spi::k_grp_apply<float><<<(unsigned)ablocks, spi::GA_T, asmem, st>>>(A, q0, nq, inv,
                                                                          status);
    SPI_LAUNCH_CHECK();
  }
  return SPI_OK;
}
