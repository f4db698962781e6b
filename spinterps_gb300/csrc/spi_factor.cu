// FP64 build + factorisation of every kriging system of a batch, and the
// per-step dual weights.
//
// Replaces, for all systems at once, what interp/steps.py:170-243 (LHS
// assembly from the precomputed cell/station variogram matrices) and
// interp/steps.py:350-352 (numpy.linalg.pinv of the LHS) do per group:
// the LHS is built straight from station coordinates (fused distance +
// variogram, never materialising the N x N matrix of every variogram), put
// in covariance form A = s*11' - Gamma, and factored A = L L' in FP64. The
// Lagrange / drift rows are handled by a Schur complement S = F'A^-1 F.
//
// GB300's FP64 pipe is narrow (about 2 DFMA per SM per clock), so these
// kernels are FP64-issue bound, not memory bound: one CTA per system, tiles
// staged in shared memory, and every operand read from L2 at most once per
// 32-wide block of FMAs.
#include "spi_common.cuh"
#include "spi_gj.cuh"
#include "spi_saddle.cuh"

namespace spi {

// The exact-inverse path's elimination over the whole GPU (spi_gj_multi.cu).
int launch_gj_multi(const spi_domain_t& dom, const spi_systems_t& sys, const spi_krige_ws_t& ws,
                    double cond_max, int pinv_on, cudaStream_t st);

// Resolves routes 3 / 4 left by k_gj (spi_pinv.cu).
int launch_pinv(const spi_domain_t& dom, const spi_systems_t& sys, const spi_krige_ws_t& ws,
                cudaStream_t st);

constexpr int NB = 32;        // panel width of the blocked factorisations
constexpr int FT = 256;       // threads per factor CTA
constexpr int GA = SPI_MAX_DRIFT + 1;

struct SysView {
  int64_t off;
  int n;
  const int32_t* idx;
  int64_t moff;
};

__device__ __forceinline__ SysView sys_view(const spi_systems_t& sys, int s) {
  SysView v;
  v.off = sys.stn_off[s];
  v.n = (int)(sys.stn_off[s + 1] - v.off);
  v.idx = sys.stn_idx + v.off;
  v.moff = sys.mat_off[s];
  return v;
}

// Sum of one value per thread over the block (all threads call it).
__device__ double block_sum(double t, double* red) {
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = t;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += red[w];
  __syncthreads();
  return r;
}

// A[i, j] for i >= j. The reference fills the upper triangle of the full
// station matrix from dists[lo, hi] and mirrors it (cyth/interpmthds.pyx:
// 196-226); with ascending station lists the entry (i, j), i > j, is the
// mirror of (j, i), whose distance is dist(stn[j], stn[i]).
// A variogram of nuggets alone. The reference's semivariogram is then the
// total sill at every distance, h = 0 included (cyth/interpmthds.pyx:38-84),
// so its saddle matrix [[c J, F], [F', 0]] has rank 2 a and numpy's pinv
// gives its minimum-norm solution: lambda = F (F'F)^-1 f with zero
// multipliers (OK: the mean of the values; EDK: the drifts' least-squares
// fit), and for SK (a zero covariance matrix) lambda = 0.
__device__ __forceinline__ bool nug_only(const spi_vg_t& vg) {
  for (int c = 0; c < vg.n_comp; ++c)
    if (vg.code[c] != SPI_VG_NUG) return false;
  return vg.n_comp > 0;
}

// The system matrix of the Cholesky path: the covariance form sh - Gamma
// (SK: the covariances). For a nugget-only variogram the covariance form
// is the zero matrix; the identity takes its place: the dual form then
// gives lambda = c - F nu with F'lambda = f, and with the covariances c = 0
// that is the minimum-norm solution above (SK: lambda = c = 0), whatever
// the matrix's size.
__global__ void k_build_sys(spi_domain_t dom, spi_systems_t sys, double* __restrict__ l_arena,
                            double* __restrict__ shift_out, int full) {
  const int s = blockIdx.y;
  SysView v = sys_view(sys, s);
  const spi_vg_t vg = sys.vg[s];
  const int sk = sys.kind == SPI_KIND_SK;
  const double sh = sk ? 0.0 : total_sill(vg);
  const bool nug = nug_only(vg);
  if (blockIdx.x == 0 && threadIdx.x == 0) shift_out[s] = sh;
  double* A = l_arena + v.moff;
  const int64_t nn = (int64_t)v.n * v.n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(e / v.n), j = (int)(e - (int64_t)i * v.n);
    if (j > i && !full) {
      A[e] = 0.0;
      continue;
    }
    if (nug) {
      A[e] = (i == j) ? 1.0 : 0.0;
      continue;
    }
    // (i, j) and its mirror from the same distance: dists[lo, hi]
    int si = v.idx[max(i, j)], sj = v.idx[min(i, j)];
    double d = dist_f64(dom.stn_x[sj], dom.stn_y[sj], dom.stn_x[si], dom.stn_y[si]);
    double g = vg_fill_f64(vg, d, sk, dom.min_vg_val);
    A[e] = sk ? g : __dsub_rn(sh, g);
  }
}

// Right-looking blocked Cholesky, in place on the lower triangle, in T
// (FP64; FP32 for the refinement path's factor). gate (optional): only
// systems with gate[s] == want are factored.
template <typename T>
__global__ __launch_bounds__(FT) void k_chol(spi_systems_t sys, T* __restrict__ l_arena,
                                            int32_t* __restrict__ status,
                                            const int32_t* __restrict__ gate, int want) {
  const int s = blockIdx.x;
  if (gate && gate[s] != want) return;
  SysView v = sys_view(sys, s);
  const int n = v.n;
  T* A = l_arena + v.moff;
  __shared__ T D[NB][NB + 1];
  __shared__ T Pi[64][NB + 1];
  __shared__ T Pj[64][NB + 1];
  __shared__ int fail;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) fail = 0;
  __syncthreads();
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int nb = min(NB, n - k0);
    for (int e = tid; e < NB * NB; e += FT) {
      int r = e / NB, c = e % NB;
      D[r][c] = (r < nb && c <= r) ? A[(int64_t)(k0 + r) * n + k0 + c] : 0.0;
    }
    __syncthreads();
    if (warp == 0) {
      for (int j = 0; j < nb; ++j) {
        T djj = D[j][j];
        if (!(djj > 0.0)) {  // not positive, or NaN
          if (lane == 0) fail = k0 + j + 1;
          break;
        }
        T ljj = sqrt(djj);
        __syncwarp();
        if (lane == j) D[j][j] = ljj;
        if (lane > j && lane < nb) D[lane][j] = D[lane][j] / ljj;
        __syncwarp();
        if (lane > j && lane < nb) {
          T lij = D[lane][j];
          for (int c = j + 1; c <= lane; ++c) D[lane][c] -= lij * D[c][j];
        }
        __syncwarp();
      }
    }
    __syncthreads();
    if (fail) break;
    for (int e = tid; e < nb * nb; e += FT) {
      int r = e / nb, c = e % nb;
      if (c <= r) A[(int64_t)(k0 + r) * n + k0 + c] = D[r][c];
    }
    // panel: rows below the diagonal block, A21 <- A21 L11^-T
    for (int r = k0 + nb + tid; r < n; r += FT) {
      T x[NB];
      T* row = A + (int64_t)r * n + k0;
#pragma unroll
      for (int j = 0; j < NB; ++j) x[j] = (j < nb) ? row[j] : 0.0;
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        if (j < nb) {
          T t = x[j];
#pragma unroll
          for (int c = 0; c < NB; ++c)
            if (c < j) t -= x[c] * D[j][c];
          x[j] = t / D[j][j];
        }
      }
#pragma unroll
      for (int j = 0; j < NB; ++j)
        if (j < nb) row[j] = x[j];
    }
    __syncthreads();
    // trailing update of the lower triangle: A22 -= L21 L21'
    const int r0 = k0 + nb;
    const int m = n - r0;
    if (m <= 0) continue;
    const int nt = (m + 63) / 64;
    for (int ti = 0; ti < nt; ++ti) {
      for (int tj = 0; tj <= ti; ++tj) {
        for (int e = tid; e < 64 * NB; e += FT) {
          int r = e / NB, c = e % NB;
          int gi = r0 + ti * 64 + r, gj = r0 + tj * 64 + r;
          Pi[r][c] = (gi < n && c < nb) ? A[(int64_t)gi * n + k0 + c] : 0.0;
          Pj[r][c] = (gj < n && c < nb) ? A[(int64_t)gj * n + k0 + c] : 0.0;
        }
        __syncthreads();
        const int rr = (tid / 16) * 4, cc = (tid % 16) * 4;
        T acc[4][4] = {};
#pragma unroll 4
        for (int c = 0; c < NB; ++c) {
          T a[4], b[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            a[q] = Pi[rr + q][c];
            b[q] = Pj[cc + q][c];
          }
#pragma unroll
          for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[p][q] += a[p] * b[q];
        }
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          int gi = r0 + ti * 64 + rr + p;
          if (gi >= n) continue;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int gj = r0 + tj * 64 + cc + q;
            if (gj <= gi) A[(int64_t)gi * n + gj] -= acc[p][q];
          }
        }
        __syncthreads();
      }
    }
  }
  __syncthreads();
  if (tid == 0) status[s] = fail;
}

// Linv = L^-1 by block rows: X_II = inv(L_II), X_IJ = -X_II sum_K L_IK X_KJ.
__global__ __launch_bounds__(FT) void k_trinv(spi_systems_t sys, const double* __restrict__ l_arena,
                                             double* __restrict__ x_arena,
                                             const int32_t* __restrict__ status,
                                             double* __restrict__ cond) {
  const int s = blockIdx.x;
  SysView v = sys_view(sys, s);
  const int n = v.n;
  const double* L = l_arena + v.moff;
  double* X = x_arena + v.moff;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (status[s] != 0) {
    if (tid == 0) cond[s] = __longlong_as_double(0x7ff0000000000000LL);
    return;
  }
  __shared__ double Ld[NB][NB + 1];
  __shared__ double Xd[NB][NB + 1];
  __shared__ double T[3][NB][NB + 1];
  __shared__ double red[FT / 32];
  double frob = 0.0;
  const int nblk = (n + NB - 1) / NB;
  for (int I = 0; I < nblk; ++I) {
    const int i0 = I * NB, nb = min(NB, n - i0);
    for (int e = tid; e < NB * NB; e += FT) {
      int r = e / NB, c = e % NB;
      Ld[r][c] = (r < nb && c <= r) ? L[(int64_t)(i0 + r) * n + i0 + c] : 0.0;
    }
    __syncthreads();
    if (warp == 0 && lane < nb) {
      const int j = lane;
      for (int i = 0; i < nb; ++i) {
        double val = 0.0;
        if (i >= j) {
          double t = (i == j) ? 1.0 : 0.0;
          for (int c = j; c < i; ++c) t -= Ld[i][c] * Xd[c][j];
          val = t / Ld[i][i];
        }
        Xd[i][j] = val;
      }
    }
    __syncthreads();
    for (int e = tid; e < nb * nb; e += FT) {
      int r = e / nb, c = e % nb;
      double xv = (c <= r) ? Xd[r][c] : 0.0;
      X[(int64_t)(i0 + r) * n + i0 + c] = xv;
      frob += xv * xv;
    }
    // off-diagonal blocks, 3 column blocks at a time
    for (int J0 = 0; J0 < I; J0 += 3) {
      const int nj = min(3, I - J0);
      for (int e = tid; e < nj * NB * NB; e += FT) {
        int jj = e / (NB * NB), rem = e % (NB * NB), r = rem / NB, c = rem % NB;
        double t = 0.0;
        if (r < nb) {
          const int J = J0 + jj;
          const double* lrow = L + (int64_t)(i0 + r) * n;
          for (int k = J * NB; k < i0; ++k) t += lrow[k] * X[(int64_t)k * n + J * NB + c];
        }
        T[jj][r][c] = t;
      }
      __syncthreads();
      for (int e = tid; e < nj * NB * NB; e += FT) {
        int jj = e / (NB * NB), rem = e % (NB * NB), r = rem / NB, c = rem % NB;
        if (r < nb) {
          double t = 0.0;
          for (int q = 0; q <= r; ++q) t += Xd[r][q] * T[jj][q][c];
          double xv = -t;
          X[(int64_t)(i0 + r) * n + (J0 + jj) * NB + c] = xv;
          frob += xv * xv;
        }
      }
      __syncthreads();
    }
    // zero the upper part of this block row (kept clean for contractions)
    for (int e = tid; e < nb * (n - i0 - nb); e += FT) {
      int r = e / (n - i0 - nb), c = e % (n - i0 - nb);
      X[(int64_t)(i0 + r) * n + i0 + nb + c] = 0.0;
    }
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) frob += __shfl_xor_sync(0xffffffffu, frob, o);
  if (lane == 0) red[warp] = frob;
  __syncthreads();
  if (tid == 0) {
    double f = 0.0;
    for (int w = 0; w < FT / 32; ++w) f += red[w];
    double a00 = L[0] * L[0];
    cond[s] = (double)n * a00 * f;
  }
}

// Exact-inverse path. Systems whose Cholesky failed, or whose condition
// estimate exceeds cond_max, get the reference's own saddle matrix
// [[Gamma, F], [F', 0]] (interp/steps.py:170-243; SK: the covariance
// matrix) inverted in place by Gauss-Jordan with partial pivoting (first
// row of maximum |pivot|), columns unscrambled in reverse pivot order.
// That is numpy.linalg.pinv (interp/steps.py:351) whenever pinv's
// singular-value cut-off (1e-15 s_max, numpy's default) removes nothing,
// which holds while ||M||_F ||P||_F <= 1e15; cond[s] receives that
// product. With
// pinv_on, systems of m <= SPI_PINV_MAX_M rows above it (or with a zero
// pivot) are left to k_pinv (route 3: inverse valid, 4: Gauss-Jordan
// failed). Dynamic shared memory: m pivot factors + m pivot indices.
__global__ __launch_bounds__(FT) void k_gj(spi_domain_t dom, spi_systems_t sys,
                                          double* __restrict__ l_arena,
                                          const int32_t* __restrict__ status,
                                          double* __restrict__ cond,
                                          int32_t* __restrict__ route, double cond_max,
                                          int pinv_on) {
  const int s = blockIdx.x;
  const int tid = threadIdx.x;
  if (status[s] == 0 && cond[s] <= cond_max) {
    if (tid == 0) route[s] = 0;
    return;
  }
  SysView v = sys_view(sys, s);
  const int n = v.n;
  const int sk = sys.kind == SPI_KIND_SK;
  const int a = extra_rows(sys.kind, dom.n_drift);
  const int m = n + a;
  const spi_vg_t vg = sys.vg[s];
  double* A = l_arena + v.moff;
  extern __shared__ double gsm[];
  double* f = gsm;                                   // [m]
  double* prow = gsm + m;                            // [m] the scaled pivot row
  int* piv = reinterpret_cast<int*>(gsm + 2 * m);    // [m]
  __shared__ double red[FT / 32];
  // saddle matrix, full storage, and its squared Frobenius norm
  double fm = 0.0;
  for (int64_t e = tid; e < (int64_t)m * m; e += FT) {
    const int i = (int)(e / m), j = (int)(e - (int64_t)i * m);
    const double val = saddle_entry(dom, vg, v.idx, n, sk, i, j);
    A[e] = val;
    fm += val * val;
  }
  fm = block_sum(fm, red);
  const int fail = gj_invert<FT>(A, m, f, prow, piv);
  double fp = 0.0;
  if (!fail)
    for (int64_t e = tid; e < (int64_t)m * m; e += FT) fp += A[e] * A[e];
  fp = block_sum(fp, red);
  if (tid == 0) {
    const double cg = sqrt(fm) * sqrt(fp);
    cond[s] = fail ? __longlong_as_double(0x7ff0000000000000LL) : cg;
    // pinv (default rcond 1e-15) cuts nothing while cond_2 <= cg <= 1e15
    const bool suspect = fail || !(cg <= 1e15);
    if (pinv_on && m <= SPI_PINV_MAX_M && suspect)
      route[s] = fail ? 4 : 3;
    else
      route[s] = fail ? 2 : 1;
  }
}

// y = X x (X lower, row-major n x n): warp per row, lanes along the row.
__device__ void matvec_lower(const double* __restrict__ X, int n, const double* __restrict__ x,
                             double* __restrict__ y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = warp; i < n; i += nw) {
    const double* row = X + (int64_t)i * n;
    double t = 0.0;
    for (int j = lane; j <= i; j += 32) t += row[j] * x[j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) y[i] = t;
  }
}

// y = X' q: thread per column, coalesced along rows.
__device__ void matvec_lower_t(const double* __restrict__ X, int n, const double* __restrict__ q,
                               double* __restrict__ y) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double t = 0.0;
    for (int i = j; i < n; ++i) t += X[(int64_t)i * n + j] * q[i];
    y[j] = t;
  }
}

__device__ double block_dot(const double* __restrict__ a, const double* __restrict__ b, int n,
                            double* red) {
  double t = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) t += a[i] * b[i];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = t;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += red[w];
  __syncthreads();
  return r;
}

// y = P[:, :n] x for the m x m row-major P (warp per row).
__device__ void matvec_rows(const double* __restrict__ P, int m, int n,
                            const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = warp; i < m; i += nw) {
    const double* row = P + (int64_t)i * m;
    double t = 0.0;
    for (int j = lane; j < n; j += 32) t += row[j] * x[j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) y[i] = t;
  }
}

// S^-1 of the small a x a Schur complement by Gauss-Jordan with partial
// pivoting (one thread), into Si and out [GA * GA], zero-padded.
__device__ void schur_inverse(const double (*S)[GA], int a, double (*Si)[GA],
                              double* __restrict__ out) {
  double M[GA][2 * GA];
  for (int i = 0; i < a; ++i)
    for (int j = 0; j < 2 * a; ++j) M[i][j] = (j < a) ? S[i][j] : (j - a == i ? 1.0 : 0.0);
  for (int c = 0; c < a; ++c) {
    int p = c;
    for (int r = c + 1; r < a; ++r)
      if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
    if (p != c)
      for (int j = 0; j < 2 * a; ++j) {
        double t = M[c][j];
        M[c][j] = M[p][j];
        M[p][j] = t;
      }
    double piv = M[c][c];
    for (int j = 0; j < 2 * a; ++j) M[c][j] /= piv;
    for (int r = 0; r < a; ++r)
      if (r != c) {
        double f = M[r][c];
        for (int j = 0; j < 2 * a; ++j) M[r][j] -= f * M[c][j];
      }
  }
  for (int i = 0; i < GA; ++i)
    for (int j = 0; j < GA; ++j) {
      double val = (i < a && j < a) ? M[i][a + j] : 0.0;
      Si[i][j] = val;
      out[i * GA + j] = val;
    }
}

// ---- triangular solves with the Cholesky factor (no inverse formed) ----
// Systems that need no OK variance never form Linv (n^3/3 FP64 per
// system); their dual vectors come from L by forward and backward
// substitution, nk <= KS right-hand sides at once, held in shared memory
// as Y[k * ldy + i]. L: row-major n x n, lower triangle (the upper one
// still holds the matrix and is never read).
constexpr int KS = 4;

// Y_k <- L^-1 Y_k. Blocks of 32 rows: the rows' dot products with the
// solved part (a warp per row, lanes along the row), then the 32 x 32
// diagonal block by one warp (a lane per row).
template <typename TL>
__device__ void trsv_lower_multi(const TL* __restrict__ L, int n, double* Y, int ldy,
                                 int nk) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i0 = 0; i0 < n; i0 += 32) {
    const int nb = min(32, n - i0);
    if (i0 > 0) {
      for (int r = warp; r < nb; r += FT / 32) {
        const TL* row = L + (int64_t)(i0 + r) * n;
        double acc[KS];
#pragma unroll
        for (int k = 0; k < KS; ++k) acc[k] = 0.0;
        for (int j = lane; j < i0; j += 32) {
          const double l = row[j];
#pragma unroll
          for (int k = 0; k < KS; ++k)
            if (k < nk) acc[k] = fma(l, Y[k * ldy + j], acc[k]);
        }
#pragma unroll
        for (int k = 0; k < KS; ++k)
          for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if (lane == 0)
          for (int k = 0; k < nk; ++k) Y[k * ldy + i0 + r] -= acc[k];
      }
      __syncthreads();
    }
    if (warp == 0) {
      double t[KS];
      const TL* Lb = L + (int64_t)(i0 + min(lane, nb - 1)) * n + i0;  // this lane's row
      // one reciprocal per row (divisions run on the 1/64-rate FP64 pipe)
      const double rd = 1.0 / (double)Lb[min(lane, nb - 1)];
#pragma unroll
      for (int k = 0; k < KS; ++k) t[k] = (lane < nb && k < nk) ? Y[k * ldy + i0 + lane] : 0.0;
      for (int c = 0; c < nb; ++c) {
        const double rcc = __shfl_sync(0xffffffffu, rd, c);
        const double lrc = (lane > c && lane < nb) ? (double)Lb[c] : 0.0;
#pragma unroll
        for (int k = 0; k < KS; ++k) {
          const double y = __shfl_sync(0xffffffffu, t[k], c) * rcc;
          if (lane == c) t[k] = y;
          else t[k] -= lrc * y;
        }
      }
      if (lane < nb)
        for (int k = 0; k < nk; ++k) Y[k * ldy + i0 + lane] = t[k];
    }
    __syncthreads();
  }
}

// Y_k <- L^-T Y_k. Blocks of 32 rows from the bottom: the diagonal block
// by one warp, then every earlier entry updated by the block's solved
// values (a thread per entry, reading the block's rows of L along them).
template <typename TL>
__device__ void trsv_lower_t_multi(const TL* __restrict__ L, int n, double* Y, int ldy,
                                   int nk) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = (n + 31) / 32;
  for (int I = nblk - 1; I >= 0; --I) {
    const int i0 = I * 32, nb = min(32, n - i0);
    if (warp == 0) {
      double t[KS];
      const double rd =
          1.0 / (double)L[(int64_t)(i0 + min(lane, nb - 1)) * n + i0 + min(lane, nb - 1)];
#pragma unroll
      for (int k = 0; k < KS; ++k) t[k] = (lane < nb && k < nk) ? Y[k * ldy + i0 + lane] : 0.0;
      for (int c = nb - 1; c >= 0; --c) {
        const TL* Lc = L + (int64_t)(i0 + c) * n + i0;  // row c of the block
        const double rcc = __shfl_sync(0xffffffffu, rd, c);
        const double lcr = (lane < c) ? (double)Lc[lane] : 0.0;
#pragma unroll
        for (int k = 0; k < KS; ++k) {
          const double y = __shfl_sync(0xffffffffu, t[k], c) * rcc;
          if (lane == c) t[k] = y;
          else t[k] -= lcr * y;
        }
      }
      if (lane < nb)
        for (int k = 0; k < nk; ++k) Y[k * ldy + i0 + lane] = t[k];
    }
    __syncthreads();
    for (int r = tid; r < i0; r += FT) {
      double acc[KS];
#pragma unroll
      for (int k = 0; k < KS; ++k) acc[k] = 0.0;
      for (int c = 0; c < nb; ++c) {
        const double l = L[(int64_t)(i0 + c) * n + r];
#pragma unroll
        for (int k = 0; k < KS; ++k)
          if (k < nk) acc[k] = fma(l, Y[k * ldy + i0 + c], acc[k]);
      }
      for (int k = 0; k < nk; ++k) Y[k * ldy + r] -= acc[k];
    }
    __syncthreads();
  }
}

// A^-1 applied to the kk vectors Y[k * n + i]: two triangular solves with
// the system's FP64 factor, or, where the system kept its FP32 factor
// (ws.ir[s] == 1), FP64 iterative refinement over it: x = L32^-T L32^-1 b,
// then, with the residual r = b - A x of the full FP64 matrix (kept in
// l_arena), x += L32^-T L32^-1 r until the componentwise backward error
// max_i |r_i| / (sum_j |A_ij| |x_j| + |b_i|) is under sqrt(n) eps (the
// FP64 solve's own level), at most SPI_IR_MAX_ITERS corrections. bval(k, i):
// entry i of right-hand side k (the Y held on entry); D: scratch of kk * n
// doubles. ws.ir_iters[s] records the corrections (their maximum over the
// calls); kIrFailed is or-ed in when they did not converge, and
// spi_krige_duals then refactors the system in FP64 and solves again.
constexpr int kIrFailed = 0x40000000;
template <typename BF>
__device__ void ainv_apply(const spi_krige_ws_t& ws, int s, int n, int64_t moff, double* Y,
                           double* D, int kk, BF bval) {
  if (!(ws.l32 && ws.ir && ws.ir[s] == 1)) {
    const double* L = ws.l_arena + moff;
    trsv_lower_multi(L, n, Y, n, kk);
    trsv_lower_t_multi(L, n, Y, n, kk);
    return;
  }
  const float* L = ws.l32 + moff;
  const double* A = ws.l_arena + moff;
  __shared__ double rmax[FT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double tol = sqrt((double)n) * 2.220446049250313e-16;
  trsv_lower_multi(L, n, Y, n, kk);
  trsv_lower_t_multi(L, n, Y, n, kk);
  int it = 0;
  bool conv = false;
  double prev = __longlong_as_double(0x7ff0000000000000LL);
  for (;; ++it) {
    // D = b - A x and the componentwise backward error, a warp per row
    double be = 0.0;
    __syncthreads();
    for (int i = warp; i < n; i += FT / 32) {
      const double* row = A + (int64_t)i * n;
      double t[KS], ta[KS];
#pragma unroll
      for (int k = 0; k < KS; ++k) t[k] = ta[k] = 0.0;
      for (int j = lane; j < n; j += 32) {
        const double a = row[j];
#pragma unroll
        for (int k = 0; k < KS; ++k)
          if (k < kk) {
            const double x = Y[k * n + j];
            t[k] = fma(a, x, t[k]);
            ta[k] = fma(fabs(a), fabs(x), ta[k]);
          }
      }
#pragma unroll
      for (int k = 0; k < KS; ++k)
        for (int o = 16; o > 0; o >>= 1) {
          t[k] += __shfl_xor_sync(0xffffffffu, t[k], o);
          ta[k] += __shfl_xor_sync(0xffffffffu, ta[k], o);
        }
      if (lane == 0)
        for (int k = 0; k < kk; ++k) {
          const double b = bval(k, i), r = b - t[k];
          D[k * n + i] = r;
          const double den = ta[k] + fabs(b);
          if (den > 0.0) be = fmax(be, fabs(r) / den);
          else if (r != 0.0) be = __longlong_as_double(0x7ff0000000000000LL);
        }
    }
    for (int o = 16; o > 0; o >>= 1) be = fmax(be, __shfl_xor_sync(0xffffffffu, be, o));
    __syncthreads();
    if (lane == 0) rmax[warp] = be;
    __syncthreads();
    be = 0.0;
    for (int w = 0; w < FT / 32; ++w) be = fmax(be, rmax[w]);
    if (be <= tol) {
      conv = true;
      break;
    }
    // a factor too far from A (cond x the FP32 rounding near 1 or above)
    // makes no progress: stop once a correction fails to halve the
    // backward error (a converging refinement shrinks it by orders of
    // magnitude per step)
    if (it == SPI_IR_MAX_ITERS || !(be < 0.5 * prev)) break;
    prev = be;
    trsv_lower_multi(L, n, D, n, kk);
    trsv_lower_t_multi(L, n, D, n, kk);
    for (int e = threadIdx.x; e < kk * n; e += FT) Y[e] += D[e];
  }
  __syncthreads();
  if (threadIdx.x == 0 && ws.ir_iters) {
    atomicMax(ws.ir_iters + s, it);
    if (!conv) atomicOr(ws.ir_iters + s, kIrFailed);
  }
}

// EDK systems whose drift rows are linearly dependent with the
// unbiasedness row (a drift constant over the stations, two proportional
// drifts): F = [1 | drifts] is then rank deficient, the Schur complement
// F'A^-1 F of the Cholesky path singular, and the reference's saddle
// matrix singular, which its pinv resolves. Such systems are sent down the
// exact-inverse path (status = n + 1): F'F's Cholesky with pivots under
// 1e-12 of its diagonal's largest entry marks them (a <= GA rows, one
// thread after the block sums).
__global__ __launch_bounds__(FT) void k_drift_check(spi_domain_t dom, spi_systems_t sys,
                                                   int32_t* __restrict__ status) {
  const int s = blockIdx.x;
  const int a = extra_rows(sys.kind, dom.n_drift);
  if (a < 2 || status[s] != 0) return;
  SysView v = sys_view(sys, s);
  const int n = v.n;
  __shared__ double red[FT / 32];
  __shared__ double M[GA][GA];
  auto fcol = [&](int k, int i) {
    return (k == 0) ? 1.0 : dom.stn_drift[(int64_t)v.idx[i] * dom.n_drift + (k - 1)];
  };
  for (int k = 0; k < a; ++k)
    for (int l = 0; l <= k; ++l) {
      double t = 0.0;
      for (int i = threadIdx.x; i < n; i += FT) t = fma(fcol(k, i), fcol(l, i), t);
      t = block_sum(t, red);
      if (threadIdx.x == 0) M[k][l] = M[l][k] = t;
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    double dmax = 0.0;
    for (int k = 0; k < a; ++k) dmax = fmax(dmax, M[k][k]);
    bool dep = !(dmax > 0.0);
    for (int j = 0; j < a && !dep; ++j) {
      double d = M[j][j];
      for (int c = 0; c < j; ++c) d -= M[j][c] * M[j][c];
      if (!(d > 1e-12 * dmax)) {
        dep = true;
        break;
      }
      const double lj = sqrt(d);
      M[j][j] = lj;
      for (int r = j + 1; r < a; ++r) {
        double t = M[r][j];
        for (int c = 0; c < j; ++c) t -= M[r][c] * M[j][c];
        M[r][j] = t / lj;
      }
    }
    if (dep) status[s] = n + 1;
  }
}

// FP32 copy of every system's matrix (the refinement path's factor).
__global__ void k_to_f32(spi_systems_t sys, const double* __restrict__ l_arena,
                         float* __restrict__ l32) {
  const int s = blockIdx.y;
  SysView v = sys_view(sys, s);
  const int64_t nn = (int64_t)v.n * v.n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    l32[v.moff + e] = (float)l_arena[v.moff + e];
}

// Systems whose refinement did not converge fall back to the FP64 factor
// (ir = 2): spi_krige_duals then factors and solves them again.
__global__ void k_ir_fail_gate(spi_systems_t sys, spi_krige_ws_t ws) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= sys.n_sys) return;
  if (ws.ir[s] == 1 && (ws.ir_iters[s] & kIrFailed)) ws.ir[s] = 2;
}

// Which systems keep the FP32 factor: it succeeded with cond <= cond_ir;
// the others' status is reset for the FP64 factorisation.
__global__ void k_ir_gate(spi_systems_t sys, spi_krige_ws_t ws, double cond_ir) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= sys.n_sys) return;
  const int keep = ws.status[s] == 0 && ws.cond[s] <= cond_ir;
  ws.ir[s] = keep;
  ws.ir_iters[s] = 0;
  if (!keep) ws.status[s] = 0;
}

// A deterministic Rademacher sign for entry i of probe k of system s.
__device__ __forceinline__ double probe_sign(int s, int k, int i) {
  uint32_t h = (uint32_t)i * 0x9E3779B1u ^ ((uint32_t)k * 0x85EBCA77u + (uint32_t)s * 0xC2B2AE3Du);
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return (h & 1u) ? 1.0 : -1.0;
}

// cond = n A_00 ||Linv||_F^2 without Linv: ||Linv||_F^2 = trace(A^-1) =
// E |L^-1 g|^2 over Rademacher g (Hutchinson), the mean of KP fixed
// probes (relative spread ~ sqrt(2 / KP) at worst, far inside the orders
// of magnitude the routing thresholds work in). Dynamic shared memory:
// nk x n doubles.
constexpr int KP = 8;
template <typename TL>
__global__ __launch_bounds__(FT) void k_cond_est(spi_systems_t sys,
                                                const TL* __restrict__ l_arena,
                                                const int32_t* __restrict__ status,
                                                double* __restrict__ cond, int nk,
                                                const int32_t* __restrict__ gate, int want) {
  const int s = blockIdx.x;
  if (gate && gate[s] != want) return;
  SysView v = sys_view(sys, s);
  const int n = v.n;
  if (status[s] != 0) {
    if (threadIdx.x == 0) cond[s] = __longlong_as_double(0x7ff0000000000000LL);
    return;
  }
  const TL* L = l_arena + v.moff;
  extern __shared__ double ysm[];
  __shared__ double red[FT / 32];
  double tot = 0.0;
  for (int k0 = 0; k0 < KP; k0 += nk) {
    const int kk = min(nk, KP - k0);
    __syncthreads();
    for (int e = threadIdx.x; e < kk * n; e += FT) {
      const int k = e / n, i = e - k * n;
      ysm[k * n + i] = probe_sign(s, k0 + k, i);
    }
    __syncthreads();
    trsv_lower_multi(L, n, ysm, n, kk);
    for (int e = threadIdx.x; e < kk * n; e += FT) tot = fma(ysm[e], ysm[e], tot);
  }
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < FT / 32; ++w) t += red[w];
    const double l0 = (double)L[0];
    cond[s] = (double)n * (l0 * l0) * (t / KP);
  }
}

// Route-0 duals without Linv (spi_krige_duals when ws.linv_arena is NULL):
// the same quantities as k_duals, A^-1 applied by two triangular solves.
// This kernel: G, S^-1, 1'G per system; k_duals_solve_steps: the steps.
// Dynamic shared memory: nk x n doubles.
__global__ __launch_bounds__(FT) void k_duals_solve(spi_domain_t dom, spi_systems_t sys,
                                                   spi_krige_ws_t ws,
                                                   const double* __restrict__ vals, int nk,
                                                   int only_fallback) {
  const int s = blockIdx.x;
  if (ws.route[s] != 0) return;
  if (only_fallback && ws.ir[s] != 2) return;
  SysView v = sys_view(sys, s);
  const int n = v.n;
  extern __shared__ double ysm[];
  __shared__ double red[FT / 32];
  __shared__ double S[GA][GA];
  __shared__ double Si[GA][GA];
  const int sk = sys.kind == SPI_KIND_SK;
  const int a = sk ? 1 : extra_rows(sys.kind, dom.n_drift);
  double* G = ws.g_cols + v.off * GA;  // column k at G + k * n
  auto fcol = [&](int k, int i) {
    return (k == 0) ? 1.0 : dom.stn_drift[(int64_t)v.idx[i] * dom.n_drift + (k - 1)];
  };
  // G_k = A^-1 F_k
  for (int k0 = 0; k0 < a; k0 += nk) {
    const int kk = min(nk, a - k0);
    __syncthreads();
    for (int e = threadIdx.x; e < kk * n; e += FT) {
      const int k = e / n, i = e - k * n;
      ysm[k * n + i] = fcol(k0 + k, i);
    }
    __syncthreads();
    ainv_apply(ws, s, n, v.moff, ysm, ysm + nk * n, kk,
               [&](int k, int i) { return fcol(k0 + k, i); });
    for (int e = threadIdx.x; e < kk * n; e += FT) G[(int64_t)k0 * n + e] = ysm[e];
  }
  __syncthreads();
  // SK: |u| (u = A^-1 1) as a second column (as k_duals)
  if (sk)
    for (int i = threadIdx.x; i < n; i += FT) G[n + i] = fabs(G[i]);
  // S = F'G, its inverse, 1'G
  for (int k = 0; k < a; ++k)
    for (int l = 0; l < a; ++l) {
      double t = 0.0;
      for (int i = threadIdx.x; i < n; i += FT) t = fma(fcol(k, i), G[(int64_t)l * n + i], t);
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      __syncthreads();
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
      __syncthreads();
      if (threadIdx.x == 0) {
        double u = 0.0;
        for (int w = 0; w < FT / 32; ++w) u += red[w];
        S[k][l] = u;
      }
    }
  __syncthreads();
  if (threadIdx.x == 0) schur_inverse(S, a, Si, ws.s_inv + (int64_t)s * GA * GA);
  for (int k = 0; k < GA; ++k) {
    double t = 0.0;
    if (k < a)
      for (int i = threadIdx.x; i < n; i += FT) t += G[(int64_t)k * n + i];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      double u = 0.0;
      for (int w = 0; w < FT / 32; ++w) u += red[w];
      ws.g_colsum[(int64_t)s * GA + k] = (k < a) ? u : 0.0;
    }
  }
}

// The per-step part of the route-0 duals without Linv: CTA (g, s) takes
// steps g * nk .. of system s (w_hat = A^-1 z - G beta with beta =
// S^-1 G'z; SK: w_hat = A^-1 z), reading G and S^-1 from k_duals_solve.
// Dynamic shared memory: nk x n doubles.
__global__ __launch_bounds__(FT) void k_duals_solve_steps(spi_domain_t dom, spi_systems_t sys,
                                                         spi_krige_ws_t ws,
                                                         const double* __restrict__ vals,
                                                         int nk, int only_fallback) {
  const int s = blockIdx.y;
  if (ws.route[s] != 0) return;
  if (only_fallback && ws.ir[s] != 2) return;
  const int64_t sb = sys.step_off[s], se = sys.step_off[s + 1];
  if (sb + (int64_t)blockIdx.x * nk >= se) return;
  SysView v = sys_view(sys, s);
  const int n = v.n;
  extern __shared__ double ysm[];
  __shared__ double red[FT / 32];
  __shared__ double Si[GA][GA];
  __shared__ double hb[KS][GA];
  const int sk = sys.kind == SPI_KIND_SK;
  const int a = sk ? 1 : extra_rows(sys.kind, dom.n_drift);
  const double* G = ws.g_cols + v.off * GA;
  for (int e = threadIdx.x; e < GA * GA; e += FT)
    Si[e / GA][e % GA] = ws.s_inv[(int64_t)s * GA * GA + e];
  for (int64_t q0 = sb + (int64_t)blockIdx.x * nk; q0 < se; q0 += (int64_t)gridDim.x * nk) {
    const int kk = (int)min((int64_t)nk, se - q0);
    __syncthreads();
    for (int e = threadIdx.x; e < kk * n; e += FT) {
      const int k = e / n, i = e - k * n;
      ysm[k * n + i] = vals[sys.val_off[sys.steps[q0 + k]] + i];
    }
    __syncthreads();
    if (!sk) {
      // h = G'z per vector, before the solves overwrite z
      for (int k = 0; k < kk; ++k)
        for (int l = 0; l < a; ++l) {
          double t = 0.0;
          for (int i = threadIdx.x; i < n; i += FT) t = fma(G[(int64_t)l * n + i], ysm[k * n + i], t);
          for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
          __syncthreads();
          if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
          __syncthreads();
          if (threadIdx.x == 0) {
            double u = 0.0;
            for (int w = 0; w < FT / 32; ++w) u += red[w];
            hb[k][l] = u;
          }
        }
      __syncthreads();
    }
    ainv_apply(ws, s, n, v.moff, ysm, ysm + nk * n, kk, [&](int k, int i) {
      return vals[sys.val_off[sys.steps[q0 + k]] + i];
    });
    for (int k = 0; k < kk; ++k) {
      const int j = sys.steps[q0 + k];
      const int64_t vo = sys.val_off[j];
      double bt[GA];
      for (int m = 0; m < GA; ++m) {
        double t = 0.0;
        if (!sk)
          for (int l = 0; l < a; ++l) t += Si[m][l] * hb[k][l];
        bt[m] = (m < a && !sk) ? t : 0.0;
      }
      for (int i = threadIdx.x; i < n; i += FT) {
        double w = ysm[k * n + i];
        if (!sk)
          for (int m = 0; m < a; ++m) w -= G[(int64_t)m * n + i] * bt[m];
        ws.w_hat[vo + i] = w;
      }
      if (threadIdx.x < GA) ws.beta[(int64_t)j * GA + threadIdx.x] = bt[threadIdx.x];
    }
  }
}

// Per-system G, S^-1, 1'G and per-step dual weights (route 0), or the
// split dual vectors of the inverse saddle matrix (route 1). Dynamic shared
// memory: 3 vectors of n + GA doubles.
__global__ __launch_bounds__(FT) void k_duals(spi_domain_t dom, spi_systems_t sys,
                                             spi_krige_ws_t ws,
                                             const double* __restrict__ vals) {
  const int s = blockIdx.x;
  const int route = ws.route[s];
  if (route == 2) return;
  if (route == 0 && ws.linv_arena == nullptr) return;  // k_duals_solve
  SysView v = sys_view(sys, s);
  const int n = v.n;
  const double* X = ws.linv_arena + v.moff;
  extern __shared__ double sm[];
  double* va = sm;
  double* vb = sm + (n + GA);
  double* vz = sm + 2 * (n + GA);
  __shared__ double red[FT / 32];
  __shared__ double S[GA][GA];
  __shared__ double Si[GA][GA];
  __shared__ double hb[GA];
  const int sk = sys.kind == SPI_KIND_SK;
  const int a = sk ? 1 : extra_rows(sys.kind, dom.n_drift);
  double* G = ws.g_cols + v.off * GA;  // column k at G + k * n
  if (route == 1) {
    const int ar = sk ? 0 : a;
    const int m = n + ar;
    const double* P = ws.l_arena + v.moff;
    for (int i = threadIdx.x; i < n; i += blockDim.x) va[i] = 1.0;
    __syncthreads();
    matvec_rows(P, m, n, va, vb);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) G[i] = vb[i];
    // SK: |u| as a second column, as on the Cholesky path (the FP32 tier's
    // bound of its sum check's rounding)
    if (sk)
      for (int i = threadIdx.x; i < n; i += blockDim.x) G[n + i] = fabs(vb[i]);
    if (threadIdx.x < GA)
      ws.g_colsum[(int64_t)s * GA + threadIdx.x] = (threadIdx.x < ar) ? vb[n + threadIdx.x] : 0.0;
    for (int64_t si = sys.step_off[s]; si < sys.step_off[s + 1]; ++si) {
      const int j = sys.steps[si];
      const int64_t vo = sys.val_off[j];
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x) vz[i] = vals[vo + i];
      __syncthreads();
      matvec_rows(P, m, n, vz, vb);
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x) ws.w_hat[vo + i] = vb[i];
      if (threadIdx.x < GA)
        ws.beta[(int64_t)j * GA + threadIdx.x] = (threadIdx.x < ar) ? vb[n + threadIdx.x] : 0.0;
    }
    return;
  }
  // G_k = Linv' (Linv F_k)
  for (int k = 0; k < a; ++k) {
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      va[i] = (k == 0) ? 1.0 : dom.stn_drift[(int64_t)v.idx[i] * dom.n_drift + (k - 1)];
    __syncthreads();
    matvec_lower(X, n, va, vb);
    __syncthreads();
    matvec_lower_t(X, n, vb, G + (int64_t)k * n);
    __syncthreads();
  }
  // SK: |u| (u = A^-1 1) as a second column. The FP32 cell kernels
  // contract it to bound the rounding of sum(lambda) = u'c per cell
  // (covariances are >= 0, so sum |u_i| c_i bounds sum |u_i c_i|).
  if (sk) {
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) G[n + i] = fabs(G[i]);
  }
  // S = F'G
  for (int k = 0; k < a; ++k) {
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      va[i] = (k == 0) ? 1.0 : dom.stn_drift[(int64_t)v.idx[i] * dom.n_drift + (k - 1)];
    __syncthreads();
    for (int l = 0; l < a; ++l) {
      double d = block_dot(va, G + (int64_t)l * n, n, red);
      if (threadIdx.x == 0) S[k][l] = d;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) schur_inverse(S, a, Si, ws.s_inv + (int64_t)s * GA * GA);
  __syncthreads();
  for (int k = 0; k < GA; ++k) {
    double cs = 0.0;
    if (k < a) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) va[i] = 1.0;
      __syncthreads();
      cs = block_dot(va, G + (int64_t)k * n, n, red);
    }
    if (threadIdx.x == 0) ws.g_colsum[(int64_t)s * GA + k] = cs;
  }
  // per step
  for (int64_t si = sys.step_off[s]; si < sys.step_off[s + 1]; ++si) {
    const int j = sys.steps[si];
    const int64_t vo = sys.val_off[j];
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) vz[i] = vals[vo + i];
    __syncthreads();
    if (!sk) {
      for (int k = 0; k < a; ++k) {
        double d = block_dot(G + (int64_t)k * n, vz, n, red);
        if (threadIdx.x == 0) hb[k] = d;
      }
      __syncthreads();
    }
    matvec_lower(X, n, vz, va);
    __syncthreads();
    matvec_lower_t(X, n, va, vb);
    __syncthreads();
    if (!sk) {
      double bt[GA];
      for (int k = 0; k < GA; ++k) {
        double t = 0.0;
        for (int l = 0; l < a; ++l) t += Si[k][l] * hb[l];
        bt[k] = (k < a) ? t : 0.0;
      }
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double w = vb[i];
        for (int k = 0; k < a; ++k) w -= G[(int64_t)k * n + i] * bt[k];
        ws.w_hat[vo + i] = w;
      }
      if (threadIdx.x < GA) ws.beta[(int64_t)j * GA + threadIdx.x] = bt[threadIdx.x];
    } else {
      for (int i = threadIdx.x; i < n; i += blockDim.x) ws.w_hat[vo + i] = vb[i];
      if (threadIdx.x < GA) ws.beta[(int64_t)j * GA + threadIdx.x] = 0.0;
    }
  }
}

// Leave-one-out cross-validation residuals of every station of every step
// (closed form): with P11 = A^-1 - G S^-1 G' the top-left block of the
// inverse saddle matrix, z_i - (kriged value at station i from the others)
// = (P11 z)_i / (P11)_ii = w_hat_i / (|Linv[:, i]|^2 - g_i' S^-1 g_i).
// Equal to solving the n leave-one-out systems of the reference's
// formulation one by one (interp/steps.py:170-435 with station i left out)
// whenever its pinv is the inverse. Route-0 systems only; others get NaN.
__global__ __launch_bounds__(FT) void k_loo(spi_domain_t dom, spi_systems_t sys,
                                           spi_krige_ws_t ws, double* __restrict__ resid) {
  const int s = blockIdx.x;
  SysView v = sys_view(sys, s);
  const int n = v.n;
  const bool ok = ws.route[s] == 0;
  const int sk = sys.kind == SPI_KIND_SK;
  const int a = sk ? 0 : extra_rows(sys.kind, dom.n_drift);
  extern __shared__ double dg[];  // [n] diagonal of P11
  const double* X = ws.linv_arena + v.moff;
  const double* G = ws.g_cols + v.off * GA;
  const double* Si = ws.s_inv + (int64_t)s * GA * GA;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double d = 0.0;
    if (ok) {
      for (int k = i; k < n; ++k) {
        double x = X[(int64_t)k * n + i];
        d += x * x;
      }
      for (int p = 0; p < a; ++p)
        for (int q = 0; q < a; ++q) d -= G[(int64_t)p * n + i] * Si[p * GA + q] * G[(int64_t)q * n + i];
    }
    dg[i] = d;
  }
  __syncthreads();
  for (int64_t si = sys.step_off[s]; si < sys.step_off[s + 1]; ++si) {
    const int64_t vo = sys.val_off[sys.steps[si]];
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      resid[vo + i] = ok ? ws.w_hat[vo + i] / dg[i] : __longlong_as_double(0x7ff8000000000000LL);
  }
}

}  // namespace spi

using namespace spi;



static int check_sys(const spi_domain_t* dom, const spi_systems_t* sys) {
  if (!dom || !sys) return SPI_ERR_ARG;
  if (sys->n_sys < 0 || sys->max_n < 0) return SPI_ERR_ARG;
  if (sys->kind < SPI_KIND_OK || sys->kind > SPI_KIND_EDK) return SPI_ERR_ARG;
  if (dom->n_drift < 0 || dom->n_drift > SPI_MAX_DRIFT) return SPI_ERR_TOO_LARGE;
  if (sys->kind == SPI_KIND_EDK && dom->n_drift > 0 && (!dom->stn_drift || !dom->cell_drift))
    return SPI_ERR_ARG;
  if (sys->n_sys > 65535) return SPI_ERR_TOO_LARGE;
  return SPI_OK;
}

static int check_ws(const spi_krige_ws_t* ws) {
  if (!ws || !ws->l_arena || !ws->status || !ws->route || !ws->cond || !ws->shift ||
      !ws->w_hat || !ws->beta || !ws->g_cols || !ws->s_inv || !ws->g_colsum)
    return SPI_ERR_ARG;
  return SPI_OK;
}

// Right-hand sides per triangular-solve pass and the shared memory they
// take (KS at most, within 200 KB).
// Right-hand sides per pass of the triangular-solve kernels and their
// dynamic shared memory: nk x n doubles, twice that with the refinement's
// correction vectors (ir).
static int solve_smem(int max_n, int* nk, size_t* bytes, int ir = 0) {
  const size_t per = (size_t)max_n * sizeof(double) * (ir ? 2 : 1);
  int k = (int)((200 * 1024) / per);
  if (k > KS) k = KS;
  if (k < 1) return SPI_ERR_TOO_LARGE;
  *nk = k;
  *bytes = (size_t)k * per;
  return SPI_OK;
}

static bool ir_mode(const spi_krige_ws_t* ws) {
  return ws->l32 && !ws->linv_arena && ws->ir && ws->ir_iters;
}

extern "C" int spi_krige_factor(const spi_domain_t* dom, const spi_systems_t* sys,
                                const spi_krige_ws_t* ws, double cond_max,
                                spi_stream_t stream) {
  int rc = check_sys(dom, sys);
  if (rc) return rc;
  if (sys->n_sys == 0) return SPI_OK;
  if ((rc = check_ws(ws))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  spi_domain_t d = *dom;
  spi_systems_t sy = *sys;
  int64_t nn = (int64_t)sys->max_n * sys->max_n;
  int gx = (int)((nn + 255) / 256);
  if (gx > 64) gx = 64;
  if (gx < 1) gx = 1;
  const bool ir = ir_mode(ws);
  k_build_sys<<<dim3(gx, sys->n_sys), 256, 0, st>>>(d, sy, ws->l_arena, ws->shift, ir ? 1 : 0);
  SPI_LAUNCH_CHECK();
  int nk = 0;
  size_t ysm = 0;
  if (!ws->linv_arena) {
    if ((rc = solve_smem(sys->max_n, &nk, &ysm))) return rc;
    if (!smem_opt_in(k_cond_est<double>, ysm) || !smem_opt_in(k_cond_est<float>, ysm))
      return SPI_ERR_CUDA;
  }
  if (ir) {
    // FP32 factor first; systems that keep it skip the FP64 one
    k_to_f32<<<dim3(gx, sys->n_sys), 256, 0, st>>>(sy, ws->l_arena, ws->l32);
    k_chol<float><<<sys->n_sys, FT, 0, st>>>(sy, ws->l32, ws->status, nullptr, 0);
    k_cond_est<float><<<sys->n_sys, FT, ysm, st>>>(sy, ws->l32, ws->status, ws->cond, nk,
                                                    nullptr, 0);
    k_ir_gate<<<(sys->n_sys + 255) / 256, 256, 0, st>>>(sy, *ws,
                                                       ws->cond_ir > 0 ? ws->cond_ir : 1e10);
    SPI_LAUNCH_CHECK();
  }
  k_chol<double><<<sys->n_sys, FT, 0, st>>>(sy, ws->l_arena, ws->status, ir ? ws->ir : nullptr,
                                            0);
  SPI_LAUNCH_CHECK();
  if (ws->linv_arena) {
    k_trinv<<<sys->n_sys, FT, 0, st>>>(sy, ws->l_arena, ws->linv_arena, ws->status, ws->cond);
  } else {
    k_cond_est<double><<<sys->n_sys, FT, ysm, st>>>(sy, ws->l_arena, ws->status, ws->cond, nk,
                                                     ir ? ws->ir : nullptr, 0);
  }
  SPI_LAUNCH_CHECK();
  size_t gsm = (size_t)(sys->max_n + GA) * (2 * sizeof(double) + sizeof(int));
  if (gsm > 200 * 1024) return SPI_ERR_TOO_LARGE;
  if (!smem_opt_in(k_gj, gsm)) return SPI_ERR_CUDA;
  if (sys->kind == SPI_KIND_EDK) {
    k_drift_check<<<sys->n_sys, FT, 0, st>>>(d, sy, ws->status);
    SPI_LAUNCH_CHECK();
  }
  const int pinv_on = ws->pinv_scratch != nullptr;
  if (ws->gj_scratch) {
    if ((rc = launch_gj_multi(d, sy, *ws, cond_max, pinv_on, st))) return rc;
  } else {
    k_gj<<<sys->n_sys, FT, gsm, st>>>(d, sy, ws->l_arena, ws->status, ws->cond, ws->route,
                                      cond_max, pinv_on);
    SPI_LAUNCH_CHECK();
  }
  if (ws->pinv_used) {
    if (cudaMemsetAsync(ws->pinv_used, 0, sizeof(int32_t) * (size_t)sys->n_sys, st) !=
        cudaSuccess)
      return SPI_ERR_CUDA;
  }
  if (pinv_on) return launch_pinv(d, sy, *ws, st);
  return SPI_OK;
}

extern "C" int spi_krige_duals(const spi_domain_t* dom, const spi_systems_t* sys,
                               const double* vals, const spi_krige_ws_t* ws,
                               spi_stream_t stream) {
  int rc = check_sys(dom, sys);
  if (rc) return rc;
  if (sys->n_sys == 0) return SPI_OK;
  if ((rc = check_ws(ws))) return rc;
  if (!vals) return SPI_ERR_ARG;
  size_t smem = (size_t)3 * (sys->max_n + GA) * sizeof(double);
  if (smem > 200 * 1024) return SPI_ERR_TOO_LARGE;
  if (!smem_opt_in(k_duals, smem)) return SPI_ERR_CUDA;
  k_duals<<<sys->n_sys, FT, smem, (cudaStream_t)stream>>>(*dom, *sys, *ws, vals);
  SPI_LAUNCH_CHECK();
  if (!ws->linv_arena) {
    // route-0 systems without Linv: triangular solves with L (or FP64
    // refinement over the FP32 factor)
    int nk;
    size_t ysm;
    if ((rc = solve_smem(sys->max_n, &nk, &ysm, ir_mode(ws) ? 1 : 0))) return rc;
    if (!smem_opt_in(k_duals_solve, ysm) || !smem_opt_in(k_duals_solve_steps, ysm))
      return SPI_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    // the steps: groups of nk spread over gx CTAs per system
    int gx = (304 + sys->n_sys - 1) / sys->n_sys;
    gx = gx < 1 ? 1 : (gx > 64 ? 64 : gx);
    const int passes = ir_mode(ws) ? 2 : 1;
    for (int pass = 0; pass < passes; ++pass) {
      if (pass == 1) {
        // systems whose refinement did not converge: FP64 factor, then
        // their duals again
        k_ir_fail_gate<<<(sys->n_sys + 255) / 256, 256, 0, st>>>(*sys, *ws);
        k_chol<double><<<sys->n_sys, FT, 0, st>>>(*sys, ws->l_arena, ws->status, ws->ir, 2);
        int nk1;
        size_t ysm1;
        if ((rc = solve_smem(sys->max_n, &nk1, &ysm1))) return rc;
        if (!smem_opt_in(k_cond_est<double>, ysm1)) return SPI_ERR_CUDA;
        k_cond_est<double><<<sys->n_sys, FT, ysm1, st>>>(*sys, ws->l_arena, ws->status,
                                                         ws->cond, nk1, ws->ir, 2);
        SPI_LAUNCH_CHECK();
      }
      k_duals_solve<<<sys->n_sys, FT, ysm, st>>>(*dom, *sys, *ws, vals, nk, pass);
      SPI_LAUNCH_CHECK();
      k_duals_solve_steps<<<dim3(gx, sys->n_sys), FT, ysm, st>>>(*dom, *sys, *ws, vals, nk,
                                                                 pass);
      SPI_LAUNCH_CHECK();
    }
  }
  return SPI_OK;
}

extern "C" int spi_krige_loo(const spi_domain_t* dom, const spi_systems_t* sys,
                             const spi_krige_ws_t* ws, double* resid, spi_stream_t stream) {
  int rc = check_sys(dom, sys);
  if (rc) return rc;
  if (sys->n_sys == 0) return SPI_OK;
  if ((rc = check_ws(ws))) return rc;
  if (!resid || !ws->linv_arena) return SPI_ERR_ARG;
  size_t smem = (size_t)sys->max_n * sizeof(double);
  if (smem > 200 * 1024) return SPI_ERR_TOO_LARGE;
  if (!smem_opt_in(k_loo, smem)) return SPI_ERR_CUDA;
  k_loo<<<sys->n_sys, FT, smem, (cudaStream_t)stream>>>(*dom, *sys, *ws, resid);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
