// numpy.linalg.pinv of the exact-inverse systems that pinv treats as
// singular (interp/steps.py:351-352): a parallel cyclic Jacobi
// eigen-decomposition of the symmetric saddle matrix in FP64.
//
// pinv(M) = V diag(1/s) U' keeps the singular values s > rcond s_max, with
// numpy's default rcond = 1e-15 (the reference passes none). For a
// symmetric M they are the |eigenvalues|, so with M = V L V' the same
// matrix is V diag(1/lambda) V' over |lambda| > 1e-15 max|lambda|. k_gj
// marks the candidates (route 3: its Gauss-Jordan inverse is valid but
// ||M||_F ||P||_F, a bound of the condition number, exceeds 1e15; route 4:
// Gauss-Jordan hit a zero pivot).
// Here each is diagonalised and
//   - when eigenvalues fall under the cut-off with none within a factor 30
//     of it on either side (a rank deficiency with a gap), pinv's answer is
//     stable under perturbation and the truncated pseudo-inverse replaces
//     the arena's inverse (route 1, pinv_used 1);
//   - when the cut-off falls inside a continuum of eigenvalues (rounding
//     noise decides what pinv drops), the Gauss-Jordan inverse stays
//     (route 1), or, after a zero pivot, the truncated pseudo-inverse is
//     taken anyway;
//   - when nothing falls under the cut-off the Gauss-Jordan inverse stays.
//
// Jacobi (Brent-Luk ordering): m - 1 rounds per sweep (m rounded up to
// even), each rotating m / 2 disjoint index pairs (p, q) at once: the 2 x 2
// rotations are computed from W, then applied to the pairs' rows, then to
// their columns (W <- J' W J) and to V's columns (V <- V J). Sweeps stop
// when the off-diagonal Frobenius norm reaches the rounding floor of the
// rotations (sqrt(8 m) eps ||M||_F, or no longer falls by 4x a sweep once
// under 1e-12 ||M||_F), after at most kSweeps. One CTA per scratch slot (SPI_PINV_SLOTS), each taking the
// candidates s = slot, slot + slots, ...; W and V live in the slot's
// scratch (global memory, L2-resident at m <= SPI_PINV_MAX_M = 256).
#include "spi_common.cuh"
#include "spi_saddle.cuh"

namespace spi {

namespace {

constexpr int PT = 256;        // threads per CTA
constexpr int kSweeps = 40;    // sweep limit
constexpr int GAP = 30;        // the cut-off's clear band, both sides
constexpr double kEps = 2.220446049250313e-16;
constexpr double kRcond = 1e-15;  // numpy.linalg.pinv's default cut-off

__device__ double cta_sum(double t, double* red) {
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = t;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < PT / 32; ++w) r += red[w];
  __syncthreads();
  return r;
}

__device__ double cta_max(double t, double* red) {
  for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = t;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < PT / 32; ++w) r = fmax(r, red[w]);
  __syncthreads();
  return r;
}

// The pair k of round r of the circle method over mm (even) indices.
__device__ __forceinline__ void round_pair(int r, int k, int mm, int& p, int& q) {
  if (k == 0) {
    p = r;
    q = mm - 1;
  } else {
    p = (r + k) % (mm - 1);
    q = (r - k + mm - 1) % (mm - 1);
  }
}

// Shared arrays of one CTA's Jacobi sweeps.
struct JacobiSmem {
  double red[PT / 32];
  double rc[SPI_PINV_MAX_M / 2], rs[SPI_PINV_MAX_M / 2];
  int rp[SPI_PINV_MAX_M / 2], rq[SPI_PINV_MAX_M / 2];
  double lam_inv[SPI_PINV_MAX_M];
};

// Diagonalises the symmetric W (m x m, row-major, global scratch) by
// cyclic Jacobi rotations, accumulating them in V (V = I on entry): on
// return W holds the eigenvalues on its diagonal, V the eigenvectors as
// columns. fm: ||W||_F^2. Whether the sweeps converged (the off-diagonal
// norm at its rounding floor) within kSweeps.
__device__ bool jacobi_sweeps(double* W, double* V, int m, double fm, JacobiSmem& sm) {
  const int tid = threadIdx.x;
  const int mm = m + (m & 1);
  double prev = __longlong_as_double(0x7ff0000000000000LL);
  for (int sweep = 0; sweep < kSweeps; ++sweep) {
    double off2 = 0.0;
    for (int e = tid; e < m * m; e += PT) {
      const int i = e / m, j = e - i * m;
      if (i != j) off2 += W[e] * W[e];
    }
    off2 = cta_sum(off2, sm.red);
    // converged: each off-diagonal entry at the rounding level of its
    // rotations (~eps times its row's diagonal), or stalled there
    if (off2 <= 8.0 * m * kEps * kEps * fm || (off2 <= 1e-24 * fm && off2 > 0.25 * prev))
      return true;
    prev = off2;
    for (int r = 0; r < mm - 1; ++r) {
      // the round's rotations
      if (tid < mm / 2) {
        int p, q;
        round_pair(r, tid, mm, p, q);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        double c = 1.0, sn = 0.0;
        if (q < m) {
          const double apq = W[p * m + q];
          if (apq != 0.0) {
            const double app = W[p * m + p], aqq = W[q * m + q];
            const double th = (aqq - app) / (2.0 * apq);
            double t;
            if (fabs(th) > 1e150)
              t = 0.5 / th;
            else
              t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            sn = t * c;
          }
        }
        sm.rp[tid] = p;
        sm.rq[tid] = q;
        sm.rc[tid] = c;
        sm.rs[tid] = sn;
      }
      __syncthreads();
      // rows p, q of W (W <- J' W)
      for (int e = tid; e < (mm / 2) * m; e += PT) {
        const int k = e / m, j = e - k * m;
        const int p = sm.rp[k], q = sm.rq[k];
        if (q >= m || sm.rs[k] == 0.0) continue;
        const double c = sm.rc[k], sn = sm.rs[k];
        const double wp = W[p * m + j], wq = W[q * m + j];
        W[p * m + j] = c * wp - sn * wq;
        W[q * m + j] = sn * wp + c * wq;
      }
      __syncthreads();
      // columns p, q of W and V (W <- W J, V <- V J)
      for (int e = tid; e < m * (mm / 2); e += PT) {
        const int i = e / (mm / 2), k = e - i * (mm / 2);
        const int p = sm.rp[k], q = sm.rq[k];
        if (q >= m || sm.rs[k] == 0.0) continue;
        const double c = sm.rc[k], sn = sm.rs[k];
        const double wp = W[i * m + p], wq = W[i * m + q];
        W[i * m + p] = c * wp - sn * wq;
        W[i * m + q] = sn * wp + c * wq;
        const double vp = V[i * m + p], vq = V[i * m + q];
        V[i * m + p] = c * vp - sn * vq;
        V[i * m + q] = sn * vp + c * vq;
      }
      __syncthreads();
    }
  }
  return false;
}

// P = V diag(lam_inv) V' (row-major m x m, row stride ld).
__device__ void pinv_assemble(const double* V, const double* lam_inv, int m, double* P,
                              int ld) {
  for (int e = threadIdx.x; e < m * m; e += PT) {
    const int i = e / m, j = e - i * m;
    const double* vi = V + i * m;
    const double* vj = V + j * m;
    double t = 0.0;
    for (int k = 0; k < m; ++k) t = fma(vi[k] * lam_inv[k], vj[k], t);
    P[(int64_t)i * ld + j] = t;
  }
}

__global__ __launch_bounds__(PT) void k_pinv(spi_domain_t dom, spi_systems_t sys,
                                             spi_krige_ws_t ws) {
  __shared__ JacobiSmem sm;
  const int tid = threadIdx.x;
  double* W = ws.pinv_scratch + (size_t)blockIdx.x * 2 * SPI_PINV_MAX_M * SPI_PINV_MAX_M;
  double* V = W + SPI_PINV_MAX_M * SPI_PINV_MAX_M;
  const int sk = sys.kind == SPI_KIND_SK;
  const int a = extra_rows(sys.kind, dom.n_drift);
  for (int s = blockIdx.x; s < sys.n_sys; s += gridDim.x) {
    const int rt = ws.route[s];
    if (rt != 3 && rt != 4) continue;
    const int64_t off = sys.stn_off[s];
    const int n = (int)(sys.stn_off[s + 1] - off);
    const int32_t* idx = sys.stn_idx + off;
    const int m = n + a;
    const spi_vg_t vg = sys.vg[s];
    // W = M (stride m), V = I
    double fm = 0.0;
    for (int e = tid; e < m * m; e += PT) {
      const int i = e / m, j = e - i * m;
      const double x = saddle_entry(dom, vg, idx, n, sk, i, j);
      W[e] = x;
      V[e] = (i == j) ? 1.0 : 0.0;
      fm += x * x;
    }
    fm = cta_sum(fm, sm.red);
    const bool conv = jacobi_sweeps(W, V, m, fm, sm);
    // the eigenvalues, pinv's cut-off and the band around it
    double mx = 0.0;
    for (int i = tid; i < m; i += PT) mx = fmax(mx, fabs(W[i * m + i]));
    mx = cta_max(mx, sm.red);
    const double cut = kRcond * mx;
    double dropped = 0.0, near = 0.0, kept_min = 1e308;
    for (int i = tid; i < m; i += PT) {
      const double l = W[i * m + i], al = fabs(l);
      sm.lam_inv[i] = (al > cut) ? 1.0 / l : 0.0;
      dropped += (al <= cut) ? 1.0 : 0.0;
      near += (al > cut / GAP && al < cut * GAP) ? 1.0 : 0.0;
      if (al > cut) kept_min = fmin(kept_min, al);
    }
    dropped = cta_sum(dropped, sm.red);
    near = cta_sum(near, sm.red);
    kept_min = -cta_max(-kept_min, sm.red);
    const bool gj_ok = rt == 3;
    const bool gapped = dropped > 0.0 && near == 0.0;
    const bool take = conv && (gapped || !gj_ok);
    // P = V diag(lam_inv) V' into the arena (row-major m x m, as the
    // Gauss-Jordan inverse)
    if (take) pinv_assemble(V, sm.lam_inv, m, ws.l_arena + sys.mat_off[s], m);
    __syncthreads();
    if (tid == 0) {
      ws.route[s] = (take || gj_ok) ? 1 : 2;
      if (take) ws.cond[s] = mx / kept_min;
      if (ws.pinv_used) ws.pinv_used[s] = take ? 1 : 0;
    }
    __syncthreads();
  }
}

// The pseudo-inverse of one explicit symmetric matrix (spi_sym_pinv):
// eigenvalues with |lambda| <= rtol max |lambda| are dropped.
__global__ __launch_bounds__(PT) void k_sym_pinv(const double* __restrict__ M, int m,
                                                 double rtol, double* __restrict__ P,
                                                 double* __restrict__ scratch,
                                                 int32_t* __restrict__ status) {
  __shared__ JacobiSmem sm;
  const int tid = threadIdx.x;
  double* W = scratch;
  double* V = scratch + (size_t)m * m;
  double fm = 0.0;
  for (int e = tid; e < m * m; e += PT) {
    const int i = e / m, j = e - i * m;
    // the symmetric part (the matrices passed are symmetric up to rounding)
    const double x = 0.5 * (M[e] + M[(int64_t)j * m + i]);
    W[e] = x;
    V[e] = (i == j) ? 1.0 : 0.0;
    fm += x * x;
  }
  fm = cta_sum(fm, sm.red);
  const bool conv = jacobi_sweeps(W, V, m, fm, sm);
  double mx = 0.0;
  for (int i = tid; i < m; i += PT) mx = fmax(mx, fabs(W[i * m + i]));
  mx = cta_max(mx, sm.red);
  const double cut = rtol * mx;
  double dropped = 0.0;
  for (int i = tid; i < m; i += PT) {
    const double l = W[i * m + i];
    sm.lam_inv[i] = (fabs(l) > cut) ? 1.0 / l : 0.0;
    dropped += (fabs(l) > cut) ? 0.0 : 1.0;
  }
  dropped = cta_sum(dropped, sm.red);
  pinv_assemble(V, sm.lam_inv, m, P, m);
  if (tid == 0) *status = conv ? (int32_t)dropped : -1;
}

// The neighbour groups' suspects (csrc/spi_local_grp.cu): status 3 (a
// Gauss-Jordan inverse with ||M||_F ||P||_F > 1e15) or 4 (a zero pivot) of
// the (group, step) tasks t = ql * n_grps + g of steps q0 .. q0 + nq - 1.
// Each is diagonalised; eigenvalues up to GAP times pinv's cut-off
// (1e-15 max |lambda|) are taken for rounding noise, and the truncated
// pseudo-inverse without them replaces the inverse (row stride ld) where
// the Jacobi sweeps converged and either the smallest kept eigenvalue lies
// a further factor GAP above or Gauss-Jordan met a zero pivot; else the
// Gauss-Jordan inverse stays where it is valid, and otherwise the task is
// singular (status 1: the cells take their nearest neighbour and prblm[q]
// is set). In a neighbour group the dropped eigenvalues are mostly the
// rounding noise of co-located stations, whose rows are identical. Every CTA scans PT statuses at a time and works
// through the candidates among them.
__global__ __launch_bounds__(PT) void k_grp_pinv(spi_domain_t dom, int kind, int k,
                                                 const int32_t* __restrict__ grp_nebs,
                                                 int32_t n_grps, int32_t q0, int32_t nq,
                                                 const spi_vg_t* __restrict__ vg, double* inv,
                                                 int ld, int32_t* status, double* scratch,
                                                 int32_t* prblm) {
  __shared__ JacobiSmem sm;
  __shared__ int cand[PT];
  __shared__ int n_cand;
  const int tid = threadIdx.x;
  double* W = scratch + (size_t)blockIdx.x * 2 * ld * ld;
  double* V = W + (size_t)ld * ld;
  const int sk = kind == SPI_KIND_SK;
  const int a = extra_rows(kind, dom.n_drift);
  const int64_t G = n_grps;
  const int64_t ntask = G * nq;
  for (int64_t base = (int64_t)blockIdx.x * PT; base < ntask; base += (int64_t)gridDim.x * PT) {
    if (tid == 0) n_cand = 0;
    __syncthreads();
    {
      const int64_t t = base + tid;
      const int32_t s = t < ntask ? status[t] : 0;
      if (s == 3 || s == 4) cand[atomicAdd(&n_cand, 1)] = tid;
    }
    __syncthreads();
    const int nc = n_cand;
    for (int c = 0; c < nc; ++c) {
      const int64_t t = base + cand[c];
      const int gj_ok = status[t] == 3;
      const int ql = (int)(t / G);
      const int64_t g = t - (int64_t)ql * G;
      const int q = q0 + ql;
      const int32_t* nb = grp_nebs + g * k;
      int n = 0;
      while (n < k && nb[n] >= 0) ++n;
      const int m = n + a;
      const spi_vg_t v = vg[q];
      double fm = 0.0;
      for (int e = tid; e < m * m; e += PT) {
        const int i = e / m, j = e - i * m;
        const double x = saddle_entry(dom, v, nb, n, sk, i, j);
        W[e] = x;
        V[e] = (i == j) ? 1.0 : 0.0;
        fm += x * x;
      }
      fm = cta_sum(fm, sm.red);
      const bool conv = jacobi_sweeps(W, V, m, fm, sm);
      double mx = 0.0;
      for (int i = tid; i < m; i += PT) mx = fmax(mx, fabs(W[i * m + i]));
      mx = cta_max(mx, sm.red);
      // An exact rank deficiency (co-located stations) leaves eigenvalues
      // at the sweeps' rounding level, a few eps ||M|| and so up to about
      // pinv's cut-off itself, where numpy's SVD puts them far below it:
      // eigenvalues up to GAP times the cut-off count as that noise and
      // are dropped, and the truncation is clear when the smallest kept
      // eigenvalue lies a further factor GAP above.
      const double cut = kRcond * mx * GAP;
      double kept_min = 1e308;
      for (int i = tid; i < m; i += PT) {
        const double l = W[i * m + i], al = fabs(l);
        sm.lam_inv[i] = (al > cut) ? 1.0 / l : 0.0;
        if (al > cut) kept_min = fmin(kept_min, al);
      }
      kept_min = -cta_max(-kept_min, sm.red);
      const bool clear = kept_min > cut * GAP;
      const bool take = conv && (clear || !gj_ok);
      if (take) pinv_assemble(V, sm.lam_inv, m, inv + t * (int64_t)ld * ld, ld);
      __syncthreads();
      if (tid == 0) {
        const bool ok = take || gj_ok;
        status[t] = ok ? 0 : 1;
        if (!ok) atomicOr(prblm + q, 1);
      }
      __syncthreads();
    }
    __syncthreads();  // every thread has read n_cand before it is reset
  }
}

}  // namespace

int local_grp_pinv(const spi_domain_t& dom, int kind, int k, const int32_t* grp_nebs,
                   int32_t n_grps, int32_t q0, int32_t nq, const spi_vg_t* vg, double* inv,
                   int32_t ld, int32_t* status, double* pinv_scratch, int32_t* prblm,
                   cudaStream_t st) {
  const int64_t ntask = (int64_t)n_grps * nq;
  if (ntask <= 0) return SPI_OK;
  if (dom.n_drift < 0 || dom.n_drift > SPI_MAX_DRIFT) return SPI_ERR_TOO_LARGE;
  const int64_t blocks = (ntask + PT - 1) / PT;
  const int grid = blocks < SPI_LOCAL_GRP_PINV_SLOTS ? (int)blocks : SPI_LOCAL_GRP_PINV_SLOTS;
  k_grp_pinv<<<grid, PT, 0, st>>>(dom, kind, k, grp_nebs, n_grps, q0, nq, vg, inv, ld, status,
                                  pinv_scratch, prblm);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

int launch_pinv(const spi_domain_t& dom, const spi_systems_t& sys, const spi_krige_ws_t& ws,
                cudaStream_t st) {
  if (sys.n_sys <= 0) return SPI_OK;
  if (dom.n_drift < 0 || dom.n_drift > SPI_MAX_DRIFT) return SPI_ERR_TOO_LARGE;
  const int grid = sys.n_sys < SPI_PINV_SLOTS ? sys.n_sys : SPI_PINV_SLOTS;
  k_pinv<<<grid, PT, 0, st>>>(dom, sys, ws);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

}  // namespace spi

using namespace spi;

extern "C" int spi_sym_pinv(const double* M, int32_t m, double rtol, double* P, double* scratch,
                            int32_t* status, spi_stream_t stream) {
  if (!M || !P || !scratch || !status || m < 1) return SPI_ERR_ARG;
  if (m > SPI_PINV_MAX_M) return SPI_ERR_TOO_LARGE;
  if (!(rtol >= 0.0)) return SPI_ERR_ARG;
  k_sym_pinv<<<1, PT, 0, (cudaStream_t)stream>>>(M, m, rtol, P, scratch, status);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
