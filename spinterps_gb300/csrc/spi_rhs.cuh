// One right-hand-side entry of a kriging system at a cell: the cell-station
// variogram term of interp/steps.py:639-650 / cyth/interpmthds.pyx:146-226,
// generated from coordinates instead of read from a cell x station matrix.
#pragma once
#include "spi_common.cuh"

namespace spi {

// FP64, the reference's own order: distance, per-component fill, zeroing of
// entries <= min_vg_val; the covariance form sh - gamma on the Cholesky path
// (sh = total sill), the reference's gamma itself for SK and on the
// exact-inverse path.
__device__ __forceinline__ double rhs_f64(const spi_domain_t& dom, const spi_vg_t& vg, int sk,
                                          bool prim, double sh, double cx, double cy, int st) {
  const double d = dist_f64(cx, cy, dom.stn_x[st], dom.stn_y[st]);
  const double g = vg_fill_f64(vg, d, sk, dom.min_vg_val);
  return (sk || prim) ? g : __dsub_rn(sh, g);
}

// FP32 constants of one system's variogram for rhs_f32.
struct RhsF32 {
  float rr[SPI_MAX_VG_COMP], ss[SPI_MAX_VG_COMP];
  float mvv, shf, band;
  __device__ __forceinline__ void init(const spi_vg_t& vg, int sk, double sh, double mv) {
#pragma unroll
    for (int c = 0; c < SPI_MAX_VG_COMP; ++c) {
      rr[c] = (float)vg.range[c];
      ss[c] = (float)vg.sill[c];
    }
    mvv = (float)mv;
    shf = (float)sh;
    // entries this close to the min_vg_val cut are re-evaluated as the
    // FP64 path does, so that both zero the same entries (a flip costs
    // min_vg_val * |w_i| in the estimate); FP32 error near the cut is
    // ~1e-6 relative for SK and ~1e-7 * s absolute for gamma = s - c
    band = sk ? 1e-4f * mvv : 4e-7f * shf + 1e-4f * mvv;
  }
};

// FP32 covariance entry (Cholesky path only): distance from double-float
// coordinates (cp, sp: x_hi, x_lo, y_hi, y_lo relative to a common origin),
// so the difference is accurate relative to the distance itself; the
// covariance evaluated directly (no s - gamma cancellation); the zeroing
// of gamma <= min_vg_val (OK/EDK) or of the covariance <= min_vg_val (SK)
// applied to it, with entries near the cut taken from rhs_f64.
__device__ __forceinline__ float rhs_f32(const spi_domain_t& dom, const spi_vg_t& vg,
                                         const RhsF32& k, int sk, double sh, float4 cp,
                                         float4 sp, int64_t gc, int st) {
  const float dx = (cp.x - sp.x) + (cp.y - sp.y);
  const float dy = (cp.z - sp.z) + (cp.w - sp.w);
  const float d = sqrtf(dx * dx + dy * dy);
  float cdir = 0.f;
#pragma unroll
  for (int c = 0; c < SPI_MAX_VG_COMP; ++c)
    if (c < vg.n_comp) cdir += cov_eval_f32(vg.code[c], d, k.rr[c], k.ss[c]);
  const float cut = sk ? cdir : k.shf - cdir;
  if (k.band > 0.f && fabsf(cut - k.mvv) <= k.band)
    return (float)rhs_f64(dom, vg, sk, false, sh, dom.cell_x[gc], dom.cell_y[gc], st);
  if (sk) return cdir <= k.mvv ? 0.f : cdir;
  return (k.shf - cdir <= k.mvv) ? k.shf : cdir;
}

// Rounding bound of an FP32-tier sum(lambda), relative to sum |u_i| c_i:
// entries ~1e-6 (FP32 exp, double-float distance), hi/lo products, and
// FP32 partial sums of 128 terms (up to ~8e-6 in the worst case).
constexpr double kSumLambdaRelErr = 1e-5;

// SK's sum(lambda) = u'c of one cell in FP64 (u = the system's first dual
// column), lanes over stations, for cells whose FP32 value is too close to
// the sum-check boundary to decide.
__device__ __forceinline__ double sk_sum_lambda_f64(const spi_domain_t& dom, const spi_vg_t& vg,
                                                    const int32_t* idx, int n, const double* u,
                                                    double cx, double cy) {
  const int lane = threadIdx.x & 31;
  double t = 0.0;
  for (int j = lane; j < n; j += 32) t = fma(u[j], rhs_f64(dom, vg, 1, false, 0.0, cx, cy, idx[j]), t);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  return t;
}

}  // namespace spi
