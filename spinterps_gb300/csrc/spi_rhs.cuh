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

// ---- double-float (FP32 pair) arithmetic: value = hi + lo, |lo| <= ulp(hi)/2.
// Knuth's TwoSum, Dekker's Fast2Sum and the FMA product error; explicit
// round-to-nearest intrinsics keep the compiler from contracting them.
struct df {
  float h, l;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df a, df b) {
  const df s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_from(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

// 2^m as an exact float product, m >= -149 (two normal powers of two).
__device__ __forceinline__ float pow2i(int m) {
  const int m1 = max(m, -120), m2 = m - m1;
  return __int_as_float((m1 + 127) << 23) * __int_as_float((m2 + 127) << 23);
}

// 2^(j/16), j = 0..15, as double-floats (head = the float nearest to
// 2^(j/16), tail = the float nearest to the rest; one 128-byte line: the
// lanes of a warp read it with one L1 wavefront).
__device__ const float2 kExp2Sixteenths[16] = {
    {1.0f, 0.0f},
    {1.0442737340927124f, 4.8334701574503924e-08f},
    {1.0905077457427979f, -1.3077539939843064e-08f},
    {1.1387885808944702f, 5.386222312608879e-08f},
    {1.1892070770263672f, 3.797635272917432e-08f},
    {1.2418577671051025f, 4.496838101886169e-08f},
    {1.2968395948410034f, -4.018999533172973e-08f},
    {1.3542555570602417f, -1.0123349269974824e-08f},
    {1.4142135381698608f, 2.4203234971764687e-08f},
    {1.4768261909484863f, -4.500898853621038e-08f},
    {1.5422108173370361f, 8.070904833346049e-09f},
    {1.610490322113037f, 9.836217174097328e-09f},
    {1.6817928552627563f, -2.4755326677450284e-08f},
    {1.7562521696090698f, -9.235770370707996e-09f},
    {1.8340080976486206f, -1.1239277952768134e-08f},
    {1.9152065515518188f, 9.845328108326612e-09f},
};

// exp of a double-float argument (t <= 0 here), relative error ~1e-12, by
// the table-driven method of P. T. P. Tang (ACM TOMS 15(2), 1989) with a
// 16-entry table:
// t = m ln2/16 + r (ln2/16 as a 12-bit head, so m * head is exact for
// |m| < 2^12, plus a two-float tail), |r| <= ln2/32; exp(r) = 1 + r + r^2/2
// (double-float) + r^3 (1/6 + r/24 + r^2/120) (FP32, <= 1.7e-6, truncation
// 1.4e-13); times 2^(j/16) from the table (j = m mod 16) and 2^(m div 16).
__device__ __forceinline__ df df_exp(df t) {
  if (t.h < -103.0f) return {0.f, 0.f};
  // round to an integer by adding 1.5 * 2^23 (no conversion instruction:
  // those run on GB300's 1/64-rate FP64 / conversion pipe); |t| * 16/ln2
  // < 2^22 here, so the integer sits in the low mantissa bits
  const float big = __fadd_rn(__fmul_rn(t.h, 23.083120346069336f), 12582912.0f);
  const int m = __float_as_int(big) - 0x4B400000;
  const float mf = __fsub_rn(big, 12582912.0f);
  const float rh0 = __fmaf_rn(-mf, 0.0433197021484375f, t.h);
  const float rl0 =
      __fmaf_rn(-mf, 1.029107354888481e-13f, __fmaf_rn(-mf, 1.9966364561696537e-06f, t.l));
  const df r = fast_two_sum(rh0, rl0);
  const float sq = __fmul_rn(r.h, r.h);
  const float sq_l = __fmaf_rn(r.h, r.h, -sq) + 2.0f * r.h * r.l;
  const float tail = sq * r.h * (1.0f / 6 + r.h * (1.0f / 24 + r.h * (1.0f / 120)));
  const df a = two_sum(1.0f, r.h);
  const df b = two_sum(a.h, 0.5f * sq);
  const df e = fast_two_sum(b.h, a.l + b.l + r.l + 0.5f * sq_l + tail);
  const float2 tj = __ldg(&kExp2Sixteenths[m & 15]);
  const df v = df_mul(e, df{tj.x, tj.y});
  const float sc = pow2i(m >> 4);
  return {v.h * sc, v.l * sc};
}

// Squared distance from split coordinates (x_hi, x_lo, y_hi, y_lo relative
// to a common origin, heads on a power-of-two grid so that their
// difference is exact: spi_split_coords) as a double-float, squares by the
// FMA product error.
__device__ __forceinline__ df df_dist2(float4 cp, float4 sp) {
  const df dx = fast_two_sum(__fsub_rn(cp.x, sp.x), __fsub_rn(cp.y, sp.y));
  const df dy = fast_two_sum(__fsub_rn(cp.z, sp.z), __fsub_rn(cp.w, sp.w));
  const float xx = __fmul_rn(dx.h, dx.h), yy = __fmul_rn(dy.h, dy.h);
  const float ex = __fmaf_rn(dx.h, dx.h, -xx) + 2.0f * dx.h * dx.l;
  const float ey = __fmaf_rn(dy.h, dy.h, -yy) + 2.0f * dy.h * dy.l;
  const df s = two_sum(xx, yy);
  return fast_two_sum(s.h, s.l + (ex + ey));
}

// Its root: rsqrt, then one correction step (d = h + (d2 - h^2) / (2 h)).
__device__ __forceinline__ df df_sqrt(df d2) {
  if (!(d2.h > 0.f)) return {0.f, 0.f};
  const float r = rsqrtf(d2.h);
  const float h = d2.h * r;
  const float e = __fmaf_rn(-h, h, d2.h) + d2.l;
  return fast_two_sum(h, e * (0.5f * r));
}

// Per-component constants of rhs_df as double-floats: sill, 1 / range,
// -3 / range and -3 / range^2.
// Kernels keep one RhsDf per CTA in shared memory (computed by one thread):
// held in registers, the compiler may recompute its FP64-derived constants
// inside the hot loop, on GB300's 1/64-rate FP64 / conversion pipe.
struct RhsDf {
  df sill[SPI_MAX_VG_COMP], inv_r[SPI_MAX_VG_COMP], k1[SPI_MAX_VG_COMP], k2[SPI_MAX_VG_COMP];
  df shift;
  float mvv, band_sk, band_ok;  // the min_vg_val cut and its bands in FP32
  int ncomp, code[SPI_MAX_VG_COMP];
  int exact;  // every component has a double-float form below
  int single;  // index of the only non-nugget component, or -1
  int nug_clear;  // nuggets alone exceed the cut: OK / EDK entries never zero
  __device__ __forceinline__ void init(const spi_vg_t& vg, double sh, double min_vg_val) {
    mvv = (float)min_vg_val;
    band_sk = 1e-6f * mvv;
    band_ok = 1e-6f * mvv + 4e-9f * (float)sh;
    ncomp = vg.n_comp;
    exact = 1;
    int nst = 0;
    single = -1;
    for (int c = 0; c < vg.n_comp; ++c)
      if (vg.code[c] != SPI_VG_NUG) {
        ++nst;
        single = c;
      }
    if (nst != 1) single = -1;
    double nug = 0.0;
    for (int c = 0; c < vg.n_comp; ++c)
      if (vg.code[c] == SPI_VG_NUG) nug += vg.sill[c];
    nug_clear = nug > min_vg_val * (1.0 + 1e-3) + 1e-8 * sh;
    for (int c = 0; c < SPI_MAX_VG_COMP; ++c) {
      const double r = vg.range[c];
      sill[c] = df_from(vg.sill[c]);
      inv_r[c] = df_from(1.0 / r);
      k1[c] = df_from(-3.0 / r);
      k2[c] = df_from(-3.0 / (r * r));
      code[c] = vg.code[c];
      if (c < vg.n_comp) {
        const int k = vg.code[c];
        if (!(k == SPI_VG_NUG || k == SPI_VG_EXP || k == SPI_VG_GAU || k == SPI_VG_SPH ||
              k == SPI_VG_LIN))
          exact = 0;
      }
    }
    shift = df_from(sh);
  }
};

// Correlation rho(h) of one structure in double-float (Exp, Gau, Sph, Lin).
__device__ __forceinline__ df rho_df(int code, df d, df d2, df k1, df k2, df inv_r) {
  if (code == SPI_VG_EXP) return df_exp(df_mul(d, k1));
  if (code == SPI_VG_GAU) return df_exp(df_mul(d2, k2));
  const df t = df_mul(d, inv_r);  // h / r
  if (!(t.h < 1.0f)) return {0.f, 0.f};
  const df u = df_add(df{1.0f, 0.f}, df{-t.h, -t.l});
  if (code == SPI_VG_LIN) return u;
  const df w = df_add(df{1.0f, 0.f}, df{0.5f * t.h, 0.5f * t.l});
  return df_mul(df_mul(u, u), w);
}

// The min_vg_val zeroing of a double-float covariance entry c (rhs_df).
// gamma = s - c carries ~1e-9 s of c's error; with min_vg_val = 0 both
// paths zero only exact zeros, which they agree on; OK / EDK entries whose
// nuggets exceed the cut are never zeroed (gamma >= nugget). Entries
// within the band of the cut take rhs_f64 itself.
__device__ __forceinline__ df rhs_df_cut(const spi_domain_t& dom, const spi_vg_t* vgp,
                                         const RhsDf& k, int sk, double sh, int64_t gc,
                                         const int32_t* stp, df c) {
  if (k.mvv > 0.f && (sk || !k.nug_clear)) {
    const df cut = sk ? c : df_add(k.shift, df{-c.h, -c.l});
    const float gap = (cut.h - k.mvv) + cut.l;
    if (fabsf(gap) <= (sk ? k.band_sk : k.band_ok))
      return df_from(rhs_f64(dom, *vgp, sk, false, sh, dom.cell_x[gc], dom.cell_y[gc], *stp));
    if (gap <= 0.f) return sk ? df{0.f, 0.f} : k.shift;
  }
  return c;
}

// One covariance entry (Cholesky path) as a double-float, relative error
// ~1e-9, for the FP32 tier's estimates and dual columns, where the
// right-hand side's rounding is amplified by the dual weights, and for the
// tensor-core variance. Same entries as rhs_f64 (covariance form, the
// min_vg_val zeroing); entries within 1e-6 of the cut, and variograms with
// components that have no double-float form here (Pow, Hol, Rng), take
// rhs_f64 itself.
// d2: the squared distance df_dist2(cp, sp) (rhs_df_d2: computed by the
// caller).
__device__ __forceinline__ df rhs_df_d2(const spi_domain_t& dom, const spi_vg_t* vgp,
                                        const RhsDf& k, int sk, double sh, df d2, int64_t gc,
                                        const int32_t* stp) {
  if (!k.exact)
    return df_from(rhs_f64(dom, *vgp, sk, false, sh, dom.cell_x[gc], dom.cell_y[gc], *stp));
  const df d = df_sqrt(d2);
  df c = {0.f, 0.f};
  if (k.single >= 0) {
    // the common case: one structure (plus nuggets, which add nothing to
    // the covariance off the diagonal)
    const int q = k.single;
    c = df_mul(k.sill[q], rho_df(k.code[q], d, d2, k.k1[q], k.k2[q], k.inv_r[q]));
  } else {
#pragma unroll
    for (int q = 0; q < SPI_MAX_VG_COMP; ++q)
      if (q < k.ncomp && k.code[q] != SPI_VG_NUG)
        c = df_add(c, df_mul(k.sill[q],
                             rho_df(k.code[q], d, d2, k.k1[q], k.k2[q], k.inv_r[q])));
  }
  return rhs_df_cut(dom, vgp, k, sk, sh, gc, stp, c);
}

__device__ __forceinline__ df rhs_df(const spi_domain_t& dom, const spi_vg_t* vgp, const RhsDf& k,
                                     int sk, double sh, float4 cp, float4 sp, int64_t gc,
                                     const int32_t* stp) {
  return rhs_df_d2(dom, vgp, k, sk, sh, k.exact ? df_dist2(cp, sp) : df{0.f, 0.f}, gc, stp);
}

// rhs_df for a variogram with one structure (plus nuggets) of the
// compile-time model CODE (Exp, Gau, Sph or Lin; k.single indexes it): no
// model switch per entry, and no square root for Gau. d2 as rhs_df_d2.
template <int CODE>
__device__ __forceinline__ df rhs_df_single_d2(const spi_domain_t& dom, const spi_vg_t* vgp,
                                               const RhsDf& k, int sk, double sh, df d2,
                                               int64_t gc, const int32_t* stp) {
  const int q = k.single;
  df rho;
  if constexpr (CODE == SPI_VG_GAU) {
    rho = df_exp(df_mul(d2, k.k2[q]));
  } else {
    const df d = df_sqrt(d2);
    if constexpr (CODE == SPI_VG_EXP) {
      rho = df_exp(df_mul(d, k.k1[q]));
    } else {
      const df t = df_mul(d, k.inv_r[q]);  // h / r
      if (!(t.h < 1.0f)) {
        rho = df{0.f, 0.f};
      } else {
        const df u = df_add(df{1.0f, 0.f}, df{-t.h, -t.l});
        if constexpr (CODE == SPI_VG_LIN) {
          rho = u;
        } else {
          const df w = df_add(df{1.0f, 0.f}, df{0.5f * t.h, 0.5f * t.l});
          rho = df_mul(df_mul(u, u), w);
        }
      }
    }
  }
  return rhs_df_cut(dom, vgp, k, sk, sh, gc, stp, df_mul(k.sill[q], rho));
}

template <int CODE>
__device__ __forceinline__ df rhs_df_single(const spi_domain_t& dom, const spi_vg_t* vgp,
                                            const RhsDf& k, int sk, double sh, float4 cp,
                                            float4 sp, int64_t gc, const int32_t* stp) {
  return rhs_df_single_d2<CODE>(dom, vgp, k, sk, sh, df_dist2(cp, sp), gc, stp);
}

// The nearest station of a cell from the double-float squared distances of
// its right-hand sides (the FP32 tier), for the cells whose sum check fails:
// the smallest d2 and its index, and whether another station lies within
// the tolerance of it, where the double-float order may differ from the
// FP64 order of dist_f64 (those cells take the exact FP64 search). The
// split coordinates are exact to e = split_res 2^-24 per difference, so a
// squared distance d2 = h^2 is within 2.83 h e + 2 e^2 of the FP64 one;
// the tolerance is four times that, plus 1e-6 d2.
struct NearDf {
  float bh, bl;  // the smallest d2 so far
  float tol;     // its tolerance
  int bj;        // its station index (-1: none yet)
  int amb;       // a station within tol of it
  __device__ __forceinline__ void init() {
    bh = bl = tol = 0.f;
    bj = -1;
    amb = 0;
  }
  __device__ __forceinline__ static float tol_of(float d2, float e) {
    return 4.f * (2.83f * sqrtf(d2) * e + 2.f * e * e) + 1e-6f * d2;
  }
  // stations visited in increasing index order; (bh, bl) stays the running
  // minimum, so a new minimum more than tol below it is more than tol
  // below every station seen
  __device__ __forceinline__ void add(df d2, int j, float e) {
    if (bj < 0) {
      bh = d2.h;
      bl = d2.l;
      bj = j;
      tol = tol_of(d2.h, e);
      return;
    }
    const float dd = (d2.h - bh) + (d2.l - bl);
    if (dd <= tol) {
      if (dd >= -tol) amb = 1;
      else amb = 0;
      if (dd < 0.f) {
        bh = d2.h;
        bl = d2.l;
        bj = j;
        tol = tol_of(d2.h, e);
      }
    }
  }
  // merge another station group's result
  __device__ __forceinline__ void merge(const NearDf& o) {
    if (o.bj < 0) return;
    if (bj < 0) {
      *this = o;
      return;
    }
    const float dd = (o.bh - bh) + (o.bl - bl);
    const float t = fmaxf(tol, o.tol);
    if (dd < -t) {
      *this = o;
    } else if (dd <= t) {
      if (dd < 0.f) *this = o;
      amb = 1;
    }
  }
};

// Rounding bound of an FP32-tier sum(lambda), relative to sum |u_i| c_i:
// entries ~1e-6 (FP32 exp, double-float distance), hi/lo products, and
// FP32 partial sums of 128 terms (up to ~8e-6 in the worst case). The
// shared-memory kernel's FP32 right-hand sides (k_krige_cells<float>).
constexpr double kSumLambdaRelErr = 1e-5;
// The same for the streamed kernel, whose sum check (SK: every dual
// column) takes double-float entries (rhs_df: ~1e-9 relative at most, its
// exp 6e-11), hi/lo weights (2^-48) and double-float sums flushed to FP64
// every 256 terms (~1e-12 of the sum of magnitudes): 1e-9, bounded here
// with a factor 100 to spare.
constexpr double kSumLambdaRelErrDf = 1e-7;

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
