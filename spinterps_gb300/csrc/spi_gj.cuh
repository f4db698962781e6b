// In-place inverse of a dense m x m row-major FP64 matrix by Gauss-Jordan
// elimination with partial pivoting (the first row of maximum |pivot|),
// columns unscrambled in reverse pivot order. For a nonsingular matrix this
// is what numpy.linalg.pinv returns whenever its singular-value cut-off
// removes nothing (interp/steps.py:351, cyth/interpmthds.pyx:335).
//
// Called by all NT threads of one block. Shared scratch from the caller:
// f and prow of m doubles, piv of m ints. Returns 0, or k + 1 when the
// pivot of step k is zero, infinite or NaN (the matrix is then left
// partially eliminated).
#pragma once
#include "spi_common.cuh"

namespace spi {

template <int NT>
__device__ int gj_invert(double* __restrict__ A, int m, double* __restrict__ f,
                         double* __restrict__ prow, int* __restrict__ piv) {
  __shared__ double rv[NT];
  __shared__ int ri[NT];
  __shared__ int fail;
  __shared__ double dk;
  const int tid = threadIdx.x;
  if (tid == 0) fail = 0;
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    // pivot: first row of maximum |A[i][k]|, i >= k
    double best = -1.0;
    int bi = 0x7fffffff;
    for (int i = k + tid; i < m; i += NT) {
      double x = fabs(A[(int64_t)i * m + k]);
      if (x > best || (x == best && i < bi) || isnan(x)) {
        best = isnan(x) ? __longlong_as_double(0x7ff0000000000000LL) : x;
        bi = i;
      }
    }
    rv[tid] = best;
    ri[tid] = bi;
    __syncthreads();
    for (int o = NT / 2; o > 0; o >>= 1) {
      if (tid < o) {
        double ob = rv[tid + o];
        int oi = ri[tid + o];
        if (ob > rv[tid] || (ob == rv[tid] && oi < ri[tid])) {
          rv[tid] = ob;
          ri[tid] = oi;
        }
      }
      __syncthreads();
    }
    const int p = ri[0];
    if (tid == 0) {
      piv[k] = p;
      if (!(rv[0] > 0.0) || isinf(rv[0])) fail = k + 1;
    }
    __syncthreads();
    if (fail) break;
    if (p != k)
      for (int j = tid; j < m; j += NT) {
        double t = A[(int64_t)k * m + j];
        A[(int64_t)k * m + j] = A[(int64_t)p * m + j];
        A[(int64_t)p * m + j] = t;
      }
    __syncthreads();
    if (tid == 0) dk = A[(int64_t)k * m + k];
    __syncthreads();
    const double dd = dk;
    for (int j = tid; j < m; j += NT) {
      double x = (j == k) ? 1.0 : A[(int64_t)k * m + j];
      x = x / dd;
      A[(int64_t)k * m + j] = x;
      prow[j] = x;
    }
    for (int i = tid; i < m; i += NT) f[i] = (i == k) ? 0.0 : A[(int64_t)i * m + k];
    __syncthreads();
    // eliminate column k from every other row: a warp per row, lanes over
    // its columns (coalesced, no index division)
    for (int i = tid >> 5; i < m; i += NT / 32) {
      if (i == k) continue;
      const double fi = f[i];
      double* row = A + (int64_t)i * m;
      for (int j = tid & 31; j < m; j += 32) {
        const double base = (j == k) ? 0.0 : row[j];
        row[j] = base - fi * prow[j];
      }
    }
    __syncthreads();
  }
  const int failed = fail;
  if (!failed) {
    for (int k = m - 1; k >= 0; --k) {
      const int p = piv[k];
      if (p != k)
        for (int i = tid; i < m; i += NT) {
          double t = A[(int64_t)i * m + k];
          A[(int64_t)i * m + k] = A[(int64_t)i * m + p];
          A[(int64_t)i * m + p] = t;
        }
      __syncthreads();
    }
  }
  return failed;
}

}  // namespace spi
