// Shared device helpers of the spinterps_gb300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "spinterps_gb300.h"

#define SPI_PI 3.14159265358979323846

namespace spi {

constexpr int kSmSlack = 1;

// Distance of cyth/interpmthds.pyx:30-35 / 140: ((x1-x2)^2 + (y1-y2)^2)^0.5,
// every operation separately rounded (no FMA) and the square root
// correctly rounded. The reference's glibc pow(x, 0.5) is within 0.52 ulp of
// the true root, so it agrees with this except for ~0.1% of inputs, where
// the two differ by one ulp.
__device__ __forceinline__ double dist_f64(double x1, double y1, double x2, double y2) {
  double dx = __dsub_rn(x1, x2);
  double dy = __dsub_rn(y1, y2);
  return __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

// The squared distance under dist_f64's root (the same rounded operations).
__device__ __forceinline__ double dist2_f64(double x1, double y1, double x2, double y2) {
  double dx = __dsub_rn(x1, x2);
  double dy = __dsub_rn(y1, y2);
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

// Variogram models of cyth/interpmthds.pyx:38-84 in FP64, same operation
// order, separately rounded.
__device__ __forceinline__ double vg_eval_f64(int code, double h, double r, double s) {
  switch (code) {
    case SPI_VG_RNG:
      return h;
    case SPI_VG_NUG:
      return s;
    case SPI_VG_SPH: {
      if (h >= r) return s;
      double a = __ddiv_rn(__dmul_rn(1.5, h), r);
      double b = __ddiv_rn(__dmul_rn(__dmul_rn(h, h), h), __dmul_rn(2.0, __dmul_rn(__dmul_rn(r, r), r)));
      return __dmul_rn(s, __dsub_rn(a, b));
    }
    case SPI_VG_EXP:
      return __dmul_rn(s, __dsub_rn(1.0, exp(__ddiv_rn(__dmul_rn(-3.0, h), r))));
    case SPI_VG_LIN:
      if (h > r) return s;
      return __dmul_rn(s, __ddiv_rn(h, r));
    case SPI_VG_GAU:
      return __dmul_rn(s, __dsub_rn(1.0, exp(__dmul_rn(-3.0, __ddiv_rn(__dmul_rn(h, h), __dmul_rn(r, r))))));
    case SPI_VG_POW:
      return __dmul_rn(s, pow(h, r));
    case SPI_VG_HOL: {
      if (h == 0.0) return 0.0;
      double a = __ddiv_rn(__dmul_rn(SPI_PI, h), r);
      return __dmul_rn(s, __dsub_rn(1.0, __ddiv_rn(sin(a), a)));
    }
    default:
      return __longlong_as_double(0x7ff8000000000000LL);
  }
}

// The same models in FP32 for the split-precision path.
__device__ __forceinline__ float vg_eval_f32(int code, float h, float r, float s) {
  switch (code) {
    case SPI_VG_RNG:
      return h;
    case SPI_VG_NUG:
      return s;
    case SPI_VG_SPH: {
      if (h >= r) return s;
      float t = h / r;
      return s * (1.5f * t - 0.5f * t * t * t);
    }
    case SPI_VG_EXP:
      return s * (1.0f - expf(-3.0f * h / r));
    case SPI_VG_LIN:
      return h > r ? s : s * (h / r);
    case SPI_VG_GAU: {
      float t = h / r;
      return s * (1.0f - expf(-3.0f * t * t));
    }
    case SPI_VG_POW:
      return s * powf(h, r);
    case SPI_VG_HOL: {
      if (h == 0.0f) return 0.0f;
      float a = (float)SPI_PI * h / r;
      return s * (1.0f - sinf(a) / a);
    }
    default:
      return __int_as_float(0x7fc00000);
  }
}

// Covariance contribution s - gamma(h) of one component, written so that
// it is computed without cancellation (s * rho(h)), for the FP32 path:
// Exp s e^{-3h/r}, Gau s e^{-3h^2/r^2}, Sph s (1-t)^2 (1 + t/2) for
// t = h/r < 1, Lin s (1 - t), Hol s sin(a)/a, Nug 0 (its gamma is s at every
// h, h = 0 included), Pow s (1 - h^r), Rng s - h.
__device__ __forceinline__ float cov_eval_f32(int code, float h, float r, float s) {
  switch (code) {
    case SPI_VG_RNG:
      return s - h;
    case SPI_VG_NUG:
      return 0.0f;
    case SPI_VG_SPH: {
      if (h >= r) return 0.0f;
      float t = h / r, u = 1.0f - t;
      return s * (u * u) * (1.0f + 0.5f * t);
    }
    case SPI_VG_EXP:
      return s * expf(-3.0f * h / r);
    case SPI_VG_LIN:
      return h > r ? 0.0f : s * (1.0f - h / r);
    case SPI_VG_GAU: {
      float t = h / r;
      return s * expf(-3.0f * t * t);
    }
    case SPI_VG_POW:
      return s * (1.0f - powf(h, r));
    case SPI_VG_HOL: {
      if (h == 0.0f) return s;
      float a = (float)SPI_PI * h / r;
      return s * (sinf(a) / a);
    }
    default:
      return __int_as_float(0x7fc00000);
  }
}

// One entry of fill_vg_var_arr (cyth/interpmthds.pyx:186-217) at distance h:
// accumulate every component in order from 0.0, then zero entries
// <= min_vg_val.
__device__ __forceinline__ double vg_fill_f64(const spi_vg_t &vg, double h, int covar,
                                              double min_vg_val) {
  double acc = 0.0;
  for (int c = 0; c < vg.n_comp; ++c) {
    double g = vg_eval_f64(vg.code[c], h, vg.range[c], vg.sill[c]);
    double t = covar ? __dsub_rn(vg.sill[c], g) : g;
    acc = __dadd_rn(acc, t);
  }
  return acc <= min_vg_val ? 0.0 : acc;
}

// x / d from d's correctly rounded reciprocal dinv: q = x dinv, the exact
// remainder x - q d by FMA, q + rem dinv. With dinv = RN(1/d) this is the
// correctly rounded quotient RN(x / d) (Markstein's correction; checked on
// 2e8 random operand pairs, significands of all ones included, with no
// difference from IEEE division): three FP64 operations where a division
// costs about ten on GB300's narrow FP64 pipe.
__device__ __forceinline__ double div_rcp(double x, double d, double dinv) {
  const double q = __dmul_rn(x, dinv);
  const double rem = __fma_rn(-q, d, x);
  return __fma_rn(rem, dinv, q);
}

// A system's variogram with the divisors of vg_eval_f64 and their
// correctly rounded reciprocals precomputed (one per CTA, in shared
// memory), for the FP64 cell kernels' right-hand sides: the same
// operations in the same order as vg_fill_f64, each division by a range
// made by div_rcp.
//
// fill_d2 takes the squared distance instead: where every structure is
// Gaussian (plus nuggets) the root is never taken and h^2 is the squared
// distance itself, within an ulp of the reference's (h^0.5)^2 (the cell
// kernels' bar is 1e-9; the drop-in builders keep the reference's form).
struct VgPre {
  spi_vg_t vg;
  double r2[SPI_MAX_VG_COMP], r3x2[SPI_MAX_VG_COMP];
  double rinv[SPI_MAX_VG_COMP], r2inv[SPI_MAX_VG_COMP], r3x2inv[SPI_MAX_VG_COMP];
  int need_h;  // a structure other than Gau / Nug needs the distance itself
  __device__ void init(const spi_vg_t& v) {
    vg = v;
    need_h = 0;
    for (int c = 0; c < v.n_comp; ++c)
      if (v.code[c] != SPI_VG_GAU && v.code[c] != SPI_VG_NUG) need_h = 1;
    for (int c = 0; c < SPI_MAX_VG_COMP; ++c) {
      const double r = v.range[c];
      r2[c] = __dmul_rn(r, r);
      r3x2[c] = __dmul_rn(2.0, __dmul_rn(__dmul_rn(r, r), r));
      rinv[c] = __drcp_rn(r);
      r2inv[c] = __drcp_rn(r2[c]);
      r3x2inv[c] = __drcp_rn(r3x2[c]);
    }
  }
  // h2: h^2 (RN(h h), or the squared distance when no structure needs h)
  __device__ __forceinline__ double eval(int c, double h, double h2) const {
    const double r = vg.range[c], s = vg.sill[c];
    switch (vg.code[c]) {
      case SPI_VG_RNG:
        return h;
      case SPI_VG_NUG:
        return s;
      case SPI_VG_SPH: {
        if (h >= r) return s;
        const double a = div_rcp(__dmul_rn(1.5, h), r, rinv[c]);
        const double b = div_rcp(__dmul_rn(__dmul_rn(h, h), h), r3x2[c], r3x2inv[c]);
        return __dmul_rn(s, __dsub_rn(a, b));
      }
      case SPI_VG_EXP:
        return __dmul_rn(s, __dsub_rn(1.0, exp(div_rcp(__dmul_rn(-3.0, h), r, rinv[c]))));
      case SPI_VG_LIN:
        if (h > r) return s;
        return __dmul_rn(s, div_rcp(h, r, rinv[c]));
      case SPI_VG_GAU:
        return __dmul_rn(s, __dsub_rn(1.0, exp(__dmul_rn(-3.0, div_rcp(h2, r2[c], r2inv[c])))));
      default:
        return vg_eval_f64(vg.code[c], h, r, s);
    }
  }
  // vg_fill_f64 of the same entry
  __device__ __forceinline__ double fill(double h, int covar, double min_vg_val) const {
    return fill_hh(h, __dmul_rn(h, h), covar, min_vg_val);
  }
  // the same from the squared distance d2 (dist2_f64)
  __device__ __forceinline__ double fill_d2(double d2, int covar, double min_vg_val) const {
    if (need_h) return fill(__dsqrt_rn(d2), covar, min_vg_val);
    return fill_hh(0.0, d2, covar, min_vg_val);
  }
  __device__ __forceinline__ double fill_hh(double h, double h2, int covar,
                                            double min_vg_val) const {
    double acc = 0.0;
    for (int c = 0; c < vg.n_comp; ++c) {
      const double g = eval(c, h, h2);
      const double t = covar ? __dsub_rn(vg.sill[c], g) : g;
      acc = __dadd_rn(acc, t);
    }
    return acc <= min_vg_val ? 0.0 : acc;
  }
};

__device__ __forceinline__ double total_sill(const spi_vg_t &vg) {
  double s = 0.0;
  for (int c = 0; c < vg.n_comp; ++c) s += vg.sill[c];
  return s;
}

// Lagrange / drift rows appended to a system of the given kind: OK 1 (the
// unbiasedness row), EDK 1 + k (plus one row per drift), SK none
// (interp/steps.py:180-219).
__host__ __device__ __forceinline__ int extra_rows(int kind, int n_drift) {
  return kind == SPI_KIND_OK ? 1 : (kind == SPI_KIND_EDK ? 1 + n_drift : 0);
}

// numpy.isclose(a, 1.0) with its defaults (rtol 1e-5, atol 1e-8).
__device__ __forceinline__ bool isclose_one(double a) {
  return fabs(a - 1.0) <= (1e-8 + 1e-5 * 1.0);
}

// Whether an FP32-tier sum(lambda) with rounding bound err could fall on
// the other side of the isclose_one boundary than its FP64 value.
__device__ __forceinline__ bool near_isclose_boundary(double a, double err) {
  return fabs(fabs(a - 1.0) - (1e-8 + 1e-5 * 1.0)) <= err;
}

template <typename T>
__device__ __forceinline__ T cast_out(double v);
template <>
__device__ __forceinline__ double cast_out<double>(double v) { return v; }
template <>
__device__ __forceinline__ float cast_out<float>(double v) { return (float)v; }

__device__ __forceinline__ double clip_est(double v, const spi_out_t &o) {
  if (o.clip_min_on && v < o.clip_min) v = o.clip_min;
  if (o.clip_max_on && v > o.clip_max) v = o.clip_max;
  return v;
}

}  // namespace spi

namespace spi {
// Keeps the CUDA error behind an SPI_ERR_CUDA status for spi_cuda_error.
void record_cuda_error(cudaError_t e);

// Opts a kernel into `bytes` of dynamic shared memory. A launch needs the
// opt-in once its static plus dynamic shared memory passes 48 KB, so a
// dynamic request just under 48 KB already needs it when the kernel has
// static arrays; it is set for every request.
template <typename K>
inline bool smem_opt_in(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)bytes) == cudaSuccess;
}
}  // namespace spi

// Launch check used by every entry point.
#define SPI_LAUNCH_CHECK()                                      \
  do {                                                          \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) {                                    \
      spi::record_cuda_error(_e);                               \
      return SPI_ERR_CUDA;                                      \
    }                                                           \
  } while (0)
