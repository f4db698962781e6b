// The exact-inverse path's Gauss-Jordan inverse with the work of every
// elimination step spread over the whole GPU.
//
// k_gj (spi_factor.cu) inverts each system in one CTA: a pivot step there
// is a rank-1 update of the m x m matrix by 256 threads of one SM, and on
// the batched workload (m ~ 750, a few dozen systems) the one-SM-per-system
// layout left most of the GPU idle while the update streamed 9 MB per step
// through one SM. Here every step k of every system of the batch is two
// launches:
//   k_gjm_pivot  (one CTA per system): the pivot (first row of maximum
//                |A[i][k]|, i >= k), the row swap, the pivot row scaled by
//                1 / pivot (with 1 / pivot in place of the pivot), and the
//                column's multipliers saved;
//   k_gjm_update (CTAs over rows x systems): A[i][j] -= f[i] prow[j] for
//                every row i != k (column k: 0 - f[i] prow[k]).
// The arithmetic is that of gj_invert (spi_gj.cuh) operation for operation,
// so the inverse is the same to the last bit; only the work's layout
// differs. k_gjm_setup builds the saddle matrices and picks the systems,
// k_gjm_finish unscrambles the columns in reverse pivot order and sets the
// route as k_gj does (||M||_F ||P||_F against 1e15, the pinv check's
// candidates). No kernel waits on another CTA: the steps are ordered by
// their launches on the stream. Outside a stream capture the host reads
// the largest pending system's row count back after the set-up and
// launches only that many steps (a batch with no exact-inverse system
// launches none).
#include "spi_common.cuh"
#include "spi_saddle.cuh"

namespace spi {

namespace {

constexpr int GT = 256;
constexpr int GAM = SPI_MAX_DRIFT + 1;
constexpr int kPending = 5;  // route while the elimination runs
constexpr int kFailed = 6;   // a zero, infinite or NaN pivot was met

struct GjSys {
  int n, m;
  const int32_t* idx;
  double* A;
  double* f;    // [m] the step's multipliers
  double* piv;  // [m] pivot rows
  double* fm;   // ||M||_F^2
};

__device__ __forceinline__ GjSys gj_sys(const spi_domain_t& dom, const spi_systems_t& sys,
                                        const spi_krige_ws_t& ws, int s) {
  GjSys g;
  const int64_t off = sys.stn_off[s];
  g.n = (int)(sys.stn_off[s + 1] - off);
  g.m = g.n + extra_rows(sys.kind, dom.n_drift);
  g.idx = sys.stn_idx + off;
  g.A = ws.l_arena + sys.mat_off[s];
  double* sc = ws.gj_scratch + 1 + 2 * off + (int64_t)(2 * GAM + 1) * s;
  g.f = sc;
  g.piv = sc + g.m;
  g.fm = sc + 2 * g.m;
  return g;
}

__device__ double gjm_block_sum(double t, double* red) {
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = t;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < GT / 32; ++w) r += red[w];
  __syncthreads();
  return r;
}

// Route 0 for Cholesky systems under cond_max; the others get the saddle
// matrix in full storage and the pending route.
__global__ __launch_bounds__(GT) void k_gjm_setup(spi_domain_t dom, spi_systems_t sys,
                                                  spi_krige_ws_t ws, double cond_max) {
  const int s = blockIdx.y;
  const bool chol = ws.status[s] == 0 && ws.cond[s] <= cond_max;
  if (blockIdx.x == 0 && threadIdx.x == 0) ws.route[s] = chol ? 0 : kPending;
  if (chol) return;
  const GjSys g = gj_sys(dom, sys, ws, s);
  // the largest pending system's rows: the host launches that many steps
  if (blockIdx.x == 0 && threadIdx.x == 0)
    atomicMax(reinterpret_cast<int*>(ws.gj_scratch), g.m);
  const spi_vg_t vg = sys.vg[s];
  const int sk = sys.kind == SPI_KIND_SK;
  const int64_t mm = (int64_t)g.m * g.m;
  for (int64_t e = blockIdx.x * (int64_t)GT + threadIdx.x; e < mm;
       e += (int64_t)gridDim.x * GT) {
    const int i = (int)(e / g.m), j = (int)(e - (int64_t)i * g.m);
    g.A[e] = saddle_entry(dom, vg, g.idx, g.n, sk, i, j);
  }
}

// Step k: pivot, swap, scale, multipliers (and, at k = 0, ||M||_F^2).
__global__ __launch_bounds__(GT) void k_gjm_pivot(spi_domain_t dom, spi_systems_t sys,
                                                  spi_krige_ws_t ws, int k) {
  const int s = blockIdx.x;
  if (ws.route[s] != kPending) return;
  const GjSys g = gj_sys(dom, sys, ws, s);
  const int m = g.m;
  if (k >= m) return;
  __shared__ double rv[GT];
  __shared__ int ri[GT];
  __shared__ double red[GT / 32];
  __shared__ double dk;
  const int tid = threadIdx.x;
  double* A = g.A;
  if (k == 0) {
    double t = 0.0;
    for (int64_t e = tid; e < (int64_t)m * m; e += GT) t += A[e] * A[e];
    t = gjm_block_sum(t, red);
    if (tid == 0) *g.fm = t;
  }
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int i = k + tid; i < m; i += GT) {
    const double x = fabs(A[(int64_t)i * m + k]);
    if (x > best || (x == best && i < bi) || isnan(x)) {
      best = isnan(x) ? __longlong_as_double(0x7ff0000000000000LL) : x;
      bi = i;
    }
  }
  rv[tid] = best;
  ri[tid] = bi;
  __syncthreads();
  for (int o = GT / 2; o > 0; o >>= 1) {
    if (tid < o) {
      const double ob = rv[tid + o];
      const int oi = ri[tid + o];
      if (ob > rv[tid] || (ob == rv[tid] && oi < ri[tid])) {
        rv[tid] = ob;
        ri[tid] = oi;
      }
    }
    __syncthreads();
  }
  const int p = ri[0];
  if (!(rv[0] > 0.0) || isinf(rv[0])) {
    if (tid == 0) ws.route[s] = kFailed;
    return;
  }
  if (tid == 0) g.piv[k] = (double)p;
  if (p != k)
    for (int j = tid; j < m; j += GT) {
      const double t = A[(int64_t)k * m + j];
      A[(int64_t)k * m + j] = A[(int64_t)p * m + j];
      A[(int64_t)p * m + j] = t;
    }
  __syncthreads();
  if (tid == 0) dk = A[(int64_t)k * m + k];
  __syncthreads();
  const double dd = dk;
  for (int i = tid; i < m; i += GT) g.f[i] = (i == k) ? 0.0 : A[(int64_t)i * m + k];
  __syncthreads();
  for (int j = tid; j < m; j += GT) {
    double x = (j == k) ? 1.0 : A[(int64_t)k * m + j];
    A[(int64_t)k * m + j] = x / dd;
  }
}

// Step k: eliminate column k from every other row; blockIdx.x takes rows
// r = blockIdx.x, blockIdx.x + gridDim.x, ..., a warp per row, lanes over
// its columns.
__global__ __launch_bounds__(GT) void k_gjm_update(spi_domain_t dom, spi_systems_t sys,
                                                   spi_krige_ws_t ws, int k) {
  const int s = blockIdx.y;
  if (ws.route[s] != kPending) return;
  const GjSys g = gj_sys(dom, sys, ws, s);
  const int m = g.m;
  if (k >= m) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double* prow = g.A + (int64_t)k * m;
  for (int i = blockIdx.x * (GT / 32) + warp; i < m; i += gridDim.x * (GT / 32)) {
    if (i == k) continue;
    const double fi = g.f[i];
    double* row = g.A + (int64_t)i * m;
    for (int j = lane; j < m; j += 32) {
      const double base = (j == k) ? 0.0 : row[j];
      row[j] = base - fi * prow[j];
    }
  }
}

// Columns unscrambled in reverse pivot order, ||P||_F, the route.
__global__ __launch_bounds__(GT) void k_gjm_finish(spi_domain_t dom, spi_systems_t sys,
                                                   spi_krige_ws_t ws, int pinv_on) {
  const int s = blockIdx.x;
  const int rt = ws.route[s];
  if (rt != kPending && rt != kFailed) return;
  const GjSys g = gj_sys(dom, sys, ws, s);
  const int m = g.m;
  const int tid = threadIdx.x;
  __shared__ double red[GT / 32];
  const bool fail = rt == kFailed;
  double fp = 0.0;
  if (!fail) {
    for (int k = m - 1; k >= 0; --k) {
      const int p = (int)g.piv[k];
      if (p != k)
        for (int i = tid; i < m; i += GT) {
          const double t = g.A[(int64_t)i * m + k];
          g.A[(int64_t)i * m + k] = g.A[(int64_t)i * m + p];
          g.A[(int64_t)i * m + p] = t;
        }
      __syncthreads();
    }
    for (int64_t e = tid; e < (int64_t)m * m; e += GT) fp += g.A[e] * g.A[e];
  }
  fp = gjm_block_sum(fp, red);
  if (tid == 0) {
    const double cg = sqrt(*g.fm) * sqrt(fp);
    ws.cond[s] = fail ? __longlong_as_double(0x7ff0000000000000LL) : cg;
    // pinv (default rcond 1e-15) cuts nothing while cond_2 <= cg <= 1e15
    const bool suspect = fail || !(cg <= 1e15);
    if (pinv_on && m <= SPI_PINV_MAX_M && suspect)
      ws.route[s] = fail ? 4 : 3;
    else
      ws.route[s] = fail ? 2 : 1;
  }
}

}  // namespace

int launch_gj_multi(const spi_domain_t& dom, const spi_systems_t& sys, const spi_krige_ws_t& ws,
                    double cond_max, int pinv_on, cudaStream_t st) {
  if (sys.n_sys <= 0) return SPI_OK;
  const int max_m = sys.max_n + extra_rows(sys.kind, dom.n_drift);
  int gx = (int)(((int64_t)max_m * max_m + GT * 8 - 1) / (GT * 8));
  gx = gx < 1 ? 1 : (gx > 256 ? 256 : gx);
  if (cudaMemsetAsync(ws.gj_scratch, 0, sizeof(int), st) != cudaSuccess) return SPI_ERR_CUDA;
  k_gjm_setup<<<dim3(gx, sys.n_sys), GT, 0, st>>>(dom, sys, ws, cond_max);
  SPI_LAUNCH_CHECK();
  // Outside a stream capture the steps stop at the largest pending system
  // (none: no step at all), read back once per batch; a captured graph
  // keeps every step up to the batch's largest system (the kernels of a
  // system with fewer rows, or not pending, return at once).
  int steps = max_m;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return SPI_ERR_CUDA;
  if (cap == cudaStreamCaptureStatusNone) {
    int h = 0;
    if (cudaMemcpyAsync(&h, ws.gj_scratch, sizeof(int), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return SPI_ERR_CUDA;
    steps = h < max_m ? h : max_m;
  }
  // the update: about 8 rows per warp per step
  int ux = (max_m + (GT / 32) * 8 - 1) / ((GT / 32) * 8);
  ux = ux < 1 ? 1 : ux;
  for (int k = 0; k < steps; ++k) {
    k_gjm_pivot<<<sys.n_sys, GT, 0, st>>>(dom, sys, ws, k);
    k_gjm_update<<<dim3(ux, sys.n_sys), GT, 0, st>>>(dom, sys, ws, k);
  }
  SPI_LAUNCH_CHECK();
  k_gjm_finish<<<sys.n_sys, GT, 0, st>>>(dom, sys, ws, pinv_on);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

}  // namespace spi
