// One entry of the reference's kriging matrix (interp/steps.py:170-243):
// the saddle matrix [[Gamma, F], [F', 0]] of OK / EDK (F = [1 | drifts]) or
// the covariance matrix of SK, Gamma filled exactly as fill_vg_var_arr
// (cyth/interpmthds.pyx:186-226: the upper triangle from dists[lo, hi],
// mirrored).
#pragma once
#include "spi_common.cuh"

namespace spi {

__device__ __forceinline__ double saddle_entry(const spi_domain_t& dom, const spi_vg_t& vg,
                                               const int32_t* idx, int n, int sk, int i,
                                               int j) {
  if (i < n && j < n) {
    const int lo = min(i, j), hi = max(i, j);
    const int sl = idx[lo], sh = idx[hi];
    const double d = dist_f64(dom.stn_x[sl], dom.stn_y[sl], dom.stn_x[sh], dom.stn_y[sh]);
    return vg_fill_f64(vg, d, sk, dom.min_vg_val);
  }
  if (i >= n && j >= n) return 0.0;
  const int st = (i < n) ? idx[i] : idx[j];
  const int k = (i < n) ? (j - n) : (i - n);
  return (k == 0) ? 1.0 : dom.stn_drift[(int64_t)st * dom.n_drift + (k - 1)];
}

}  // namespace spi
